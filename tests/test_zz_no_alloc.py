"""The allocation-free energy + gradient entry point.

deft_fmt_energy_grad_noalloc serves callers that cannot call cudaMalloc
(a framework that has already reserved the GPU's memory, or a loop that may
not allocate once it runs).  It must give what the regular entry point
deft_fmt_energy_grad gives, within the parity tolerances used elsewhere
(energy 1e-10 relative, gradient 1e-9 relative to its max), on consecutive
calls that share its one fixed scratch array.  This file is named to run
last, so a failure here comes after every other test has run; it also runs
on its own in a fresh process.
"""
import ctypes
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

E_TOL = 1e-10
G_TOL = 1e-9


def _case(kind):
    rng = np.random.default_rng({"slit": 17, "fcc": 23, "local": 29}[kind])
    if kind == "local":
        # local terms only (no hard spheres): ideal gas, mu and V_ext
        N = (12, 10, 14)
        lat = np.diag([2.4, 2.0, 2.8])
        n = 0.05 * (1 + 0.2 * rng.standard_normal(int(np.prod(N))))
        V = 0.3 * rng.standard_normal(n.size)
        return N, lat, 1.0, n, V, None
    if kind == "slit":
        N = (24, 20, 32)
        lat = np.diag([4.8, 4.0, 6.4])
        z = np.arange(N[2]) * 0.2
        mask = np.broadcast_to(((z > 0) & (z < 3.2)).astype(float), N).reshape(-1).copy()
        nb = 0.3 / (4 * math.pi / 3)
        n = nb * (1 + 0.05 * rng.standard_normal(mask.size)) * mask
        V = None
        R = 1.0
    else:
        N = (16, 18, 15)
        lat = np.array([[0, 2.6, 2.6], [2.6, 0, 2.6], [2.6, 2.6, 0.0]])
        nb = 0.2 / (4 * math.pi / 3 * 0.8 ** 3)
        n = nb * (1 + 0.1 * rng.standard_normal(int(np.prod(N))))
        mask = None
        V = 0.3 * rng.standard_normal(n.size)
        R = 0.8
    return N, lat, R, n, V, mask


def _regular(L, _lib, ctx_h, N, lat, params, nd, Vd, md):
    import torch
    lat9 = np.ascontiguousarray(lat.reshape(9), dtype=np.float64)
    g = ctypes.c_void_p()
    _lib.check(L.deft_grid_create(ctx_h, lat9.ctypes.data, *N, ctypes.byref(g)))
    f = ctypes.c_void_p()
    _lib.check(L.deft_fmt_create(g, ctypes.byref(params), ctypes.byref(f)))
    if Vd is not None:
        _lib.check(L.deft_fmt_set_vext(f, Vd.data_ptr(), 1))
    if md is not None:
        _lib.check(L.deft_fmt_set_mask(f, md.data_ptr(), 1))
    grad = torch.empty_like(nd)
    E = ctypes.c_double()
    t = np.zeros(_lib.NTERMS)
    torch.cuda.synchronize()
    _lib.check(L.deft_fmt_energy_grad(f, nd.data_ptr(), 1, ctypes.addressof(E), grad.data_ptr(),
                                      t.ctypes.data))
    out = (E.value, grad.cpu().numpy(), t)
    L.deft_fmt_destroy(f)
    L.deft_grid_destroy(g)
    return out


def test_noalloc_matches_regular_entry_point_twice():
    import torch
    from deft_gb300 import _lib
    L = _lib.load()
    assert L.deft_noalloc_scratch_bytes() == 20 << 20
    ctx = ctypes.c_void_p()
    _lib.check(L.deft_ctx_create(0, ctypes.byref(ctx)))
    stream = torch.cuda.current_stream()
    try:
        # three calls in a row sharing the scratch array; the last has no
        # hard-sphere term (the local-terms branch)
        for kind in ("slit", "fcc", "local"):
            N, lat, R, n, V, mask = _case(kind)
            terms = _lib.TERM_IDEAL | _lib.TERM_MU
            if kind != "local":
                terms |= _lib.TERM_HS
            if V is not None:
                terms |= _lib.TERM_VEXT
            if mask is not None:
                terms |= _lib.TERM_MASK
            nb = float(n[n > 0].mean())
            mu = ctypes.c_double()
            _lib.check(L.deft_find_chemical_potential(R, 1.0, nb, ctypes.addressof(mu)))
            params = _lib.FmtParams(R, 1.0, mu.value, terms)
            nd = torch.tensor(n, dtype=torch.float64, device="cuda")
            Vd = None if V is None else torch.tensor(V, dtype=torch.float64, device="cuda")
            md = None if mask is None else torch.tensor(mask, dtype=torch.float64, device="cuda")
            E_ref, g_ref, t_ref = _regular(L, _lib, ctx, N, lat, params, nd, Vd, md)

            grad = torch.full_like(nd, float("nan"))
            E = ctypes.c_double()
            t = np.zeros(_lib.NTERMS)
            lat9 = np.ascontiguousarray(lat.reshape(9), dtype=np.float64)
            torch.cuda.synchronize()
            _lib.check(L.deft_fmt_energy_grad_noalloc(
                lat9.ctypes.data, *N, ctypes.byref(params), nd.data_ptr(),
                None if Vd is None else Vd.data_ptr(), None if md is None else md.data_ptr(),
                ctypes.addressof(E), grad.data_ptr(), t.ctypes.data, stream.cuda_stream))
            g = grad.cpu().numpy()
            assert abs(E.value / E_ref - 1) < E_TOL, kind
            assert np.abs(t - t_ref).max() <= E_TOL * np.abs(t_ref).max(), kind
            assert np.abs(g - g_ref).max() <= G_TOL * np.abs(g_ref).max(), kind
    finally:
        L.deft_ctx_destroy(ctx)


def test_noalloc_rejects_oversized_grid():
    from deft_gb300 import _lib
    L = _lib.load()
    lat9 = np.ascontiguousarray(np.diag([25.6, 25.6, 25.6]).reshape(9))
    params = _lib.FmtParams(1.0, 1.0, 0.0, _lib.TERM_HS)
    E = ctypes.c_double()
    # host buffers of the full size: the host-side size check rejects the
    # call before any pointer is used or any work is queued
    n = np.zeros(128 ** 3)
    g = np.zeros(128 ** 3)
    s = L.deft_fmt_energy_grad_noalloc(lat9.ctypes.data, 128, 128, 128, ctypes.byref(params),
                                       n.ctypes.data, None, None, ctypes.addressof(E),
                                       g.ctypes.data, None, None)
    assert s == _lib.ERR_ARG
    assert b"scratch" in L.deft_last_error()


FIRST_CALL_CHILD = r"""
import ctypes, json, sys
import numpy as np
import torch
sys.path.insert(0, sys.argv[1])
from deft_gb300 import _lib
from tests.test_zz_no_alloc import _case
free, total = torch.cuda.mem_get_info()
hold = torch.empty(int(free * 0.9), dtype=torch.uint8, device="cuda")  # the framework's pool
L = _lib.load()
N, lat, R, n, V, mask = _case("fcc")
terms = _lib.TERM_HS | _lib.TERM_IDEAL | _lib.TERM_MU | _lib.TERM_VEXT
params = _lib.FmtParams(R, 1.0, -2.0, terms)
lat9 = np.ascontiguousarray(lat.reshape(9), dtype=np.float64)
nd = torch.tensor(n, dtype=torch.float64, device="cuda")
Vd = torch.tensor(V, dtype=torch.float64, device="cuda")
grad = torch.empty_like(nd)
E = ctypes.c_double()
torch.cuda.synchronize()
s = L.deft_fmt_energy_grad_noalloc(lat9.ctypes.data, *N, ctypes.byref(params), nd.data_ptr(),
                                   Vd.data_ptr(), None, ctypes.addressof(E), grad.data_ptr(),
                                   None, None)
out = {"status": s, "msg": L.deft_last_error().decode(), "E": E.value,
       "grad": grad.cpu().numpy().tolist(), "held_gb": hold.numel() / 1e9}
del hold
torch.cuda.empty_cache()
ctx = ctypes.c_void_p()
_lib.check(L.deft_ctx_create(0, ctypes.byref(ctx)))
g = ctypes.c_void_p()
_lib.check(L.deft_grid_create(ctx, lat9.ctypes.data, *N, ctypes.byref(g)))
f = ctypes.c_void_p()
_lib.check(L.deft_fmt_create(g, ctypes.byref(params), ctypes.byref(f)))
_lib.check(L.deft_fmt_set_vext(f, Vd.data_ptr(), 1))
g2 = torch.empty_like(nd)
E2 = ctypes.c_double()
_lib.check(L.deft_fmt_energy_grad(f, nd.data_ptr(), 1, ctypes.addressof(E2), g2.data_ptr(), None))
out["E_ref"] = E2.value
out["grad_ref"] = g2.cpu().numpy().tolist()
L.deft_fmt_destroy(f)
L.deft_grid_destroy(g)
L.deft_ctx_destroy(ctx)
print(json.dumps(out))
"""


def test_noalloc_first_call_after_framework_reserved_memory():
    """A fresh process whose framework (torch here) has taken 90 % of the
    free device memory before its first call into the library: the first
    call is the allocation-free entry point, which must still succeed (its
    array comes with the library's module) and agree with the regular entry
    point, called afterwards once the pool is released."""
    import json
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", FIRST_CALL_CHILD, root], capture_output=True,
                       text=True, timeout=300, cwd=root)
    assert r.returncode == 0, r.stderr[-2000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["status"] == 0, out["msg"]
    assert abs(out["E"] / out["E_ref"] - 1) < E_TOL
    g, g_ref = np.array(out["grad"]), np.array(out["grad_ref"])
    assert np.abs(g - g_ref).max() <= G_TOL * np.abs(g_ref).max()
