"""The bulk structure-factor preconditioner (DEFT_PC_STRUCTURE, an extension):
M^-1 r = s F^-1[F[s r] / H_b(k)], s = sqrt(n / n_b) on the free points.

- The operator (deft_fmt_precondition) against a numpy restatement whose
  bulk Hessian H_b(k) is the FFT of the oracle's FP64 Hessian row of the
  uniform fluid (central differences of the oracle's gradient: independent
  of the analytic form the kernels evaluate), and the bulk density the
  library solves from mu against the problem's.
- Solves with it, FP64 and mixed, converge to the FP64 solution at
  |grad F| < 1e-12 within 1e-8 of the density scale and take fewer
  evaluations than with the density preconditioner from the same start.
- The device-driven solve (one graph launch) with it follows the
  host-driven one.
- Unsupported settings are refused."""
import ctypes

import numpy as np
import pytest

from deft_gb300 import _lib

pytestmark = pytest.mark.gpu

TERMS = _lib.TERM_HS | _lib.TERM_IDEAL | _lib.TERM_MU | _lib.TERM_MASK


def _problem(k):
    from deft_gb300.workloads import WallsSolutes
    return [WallsSolutes(N=32, dx=0.2, eta=0.35, width=4.0, solutes=[(3.2, 3.2, 2.0, 1.5)],
                         amp=0.05, seed=4),
            WallsSolutes(N=64, dx=0.2, eta=0.4, width=8.0,
                         solutes=[(2.0, 7.0, 3.0, 2.0), (9.0, 4.0, 5.0, 1.2)], amp=0.05,
                         seed=6)][k]


def _launches(grid):
    name = ctypes.c_char_p()
    launches = ctypes.c_longlong()
    tot = ctypes.c_double()
    out = {}
    for i in range(grid.L.deft_grid_profile_count(grid.h)):
        _lib.check(grid.L.deft_grid_profile_entry(grid.h, i, ctypes.byref(name),
                                                  ctypes.addressof(launches),
                                                  ctypes.addressof(tot)))
        out[name.value.decode()] = launches.value
    return out


def test_structure_preconditioner_matches_restatement(oracle_mod):
    from tests.capi import Ctx, Fmt, Grid
    O = oracle_mod
    s = _problem(0)
    mask = s.mask.reshape(-1)
    ctx = Ctx(0)
    g = Grid(ctx, s.lat, s.shape)
    f = Fmt(g, R=s.R, kT=s.kT, mu=s.mu, terms=TERMS, mask=mask)
    try:
        rng = np.random.default_rng(3)
        n = s.n0.reshape(-1)
        r = rng.standard_normal(n.size) * mask
        z = np.empty_like(n)
        nb = ctypes.c_double()
        _lib.check(f.L.deft_fmt_precondition(f.h, n.ctypes.data, r.ctypes.data, 0,
                                             z.ctypes.data, ctypes.addressof(nb)))
        assert abs(nb.value - s.nb) <= 1e-10 * s.nb
        # H_b(k): the oracle's Hessian row of the uniform fluid at nb
        Pb = O.Problem(s.lat, s.shape, R=s.R, kT=s.kT, mu=s.mu, terms=O.HS | O.IDEAL | O.MU)
        u = np.full(n.size, s.nb)
        e = 1e-4 * s.nb
        d = np.zeros(n.size)
        d[0] = 1.0
        h = (Pb.energy_grad(u + e * d)[1] - Pb.energy_grad(u - e * d)[1]) / (2 * e)
        Hk = np.fft.rfftn(h.reshape(s.shape))
        assert np.abs(Hk.imag).max() <= 1e-10 * np.abs(Hk.real).max()
        sc = np.where((mask != 0) & (n > 0), np.sqrt(np.maximum(n, 0) / s.nb), 0.0)
        zr = sc * np.fft.irfftn(np.fft.rfftn((sc * r).reshape(s.shape)) / Hk.real, s=s.shape,
                                axes=(0, 1, 2)).reshape(-1)
        # FP32 transforms: errors ~1e-6 of the field's scale
        assert np.abs(z - zr).max() <= 2e-5 * np.abs(zr).max()
        assert np.all(z[mask == 0] == 0)
    finally:
        for o in (f, g, ctx):
            o.close()


@pytest.mark.parametrize("k", [0, 1])
@pytest.mark.parametrize("precision", [_lib.PRECISION_FP64, _lib.PRECISION_MIXED])
def test_structure_preconditioned_solve(k, precision):
    from tests.capi import CG, Ctx, Fmt, Grid
    s = _problem(k)
    mask = s.mask.reshape(-1)
    ctx = Ctx(0)
    g = Grid(ctx, s.lat, s.shape)
    f = Fmt(g, R=s.R, kT=s.kT, mu=s.mu, terms=TERMS, mask=mask, precision=precision)
    f64 = Fmt(g, R=s.R, kT=s.kT, mu=s.mu, terms=TERMS, mask=mask)
    try:
        gtol = 5e-10
        runs = {}
        for pc in (_lib.PC_DENSITY, _lib.PC_STRUCTURE):
            _lib.check(g.L.deft_grid_profile(g.h, 0))
            cg = CG(f, gtol=gtol, maxiter=3000, step=1.0, preconditioned=pc)
            cg.set_x(s.n0.reshape(-1))
            code, st = cg.solve()
            assert code == 0, _lib.load().deft_last_error()
            assert st.converged
            runs[pc] = (st.evals, st.hvps, cg.get_x(), _launches(g))
            cg.close()
        ev_d, hv_d, _, _ = runs[_lib.PC_DENSITY]
        ev_s, hv_s, x, n = runs[_lib.PC_STRUCTURE]
        key = "struct_pc_f32"
        assert n[key] > 0
        # fewer evaluations (and, in the mixed form, products) than the
        # density preconditioner
        assert ev_s < ev_d
        if precision == _lib.PRECISION_MIXED:
            assert ev_s + hv_s < ev_d + hv_d
        _, g64, _ = f64.energy_grad(x)
        assert np.linalg.norm(g64) < (1e-9 if precision == _lib.PRECISION_FP64 else gtol)
        ref = CG(f64, gtol=1e-12, maxiter=5000, step=1.0, preconditioned=_lib.PC_DENSITY)
        ref.set_x(s.n0.reshape(-1))
        code, st_r = ref.solve()
        assert code == 0 and st_r.converged
        x_ref = ref.get_x()
        ref.close()
        assert np.abs(x - x_ref).max() <= 1e-8 * float(np.abs(x_ref).max())
    finally:
        for o in (f64, f, g, ctx):
            o.close()


def test_structure_preconditioner_refuses_unsupported_settings():
    from tests.capi import CG, Ctx, Fmt, Grid
    from deft_gb300.workloads import WallsSolutes
    ctx = Ctx(0)
    try:
        # Nz = 48: not a warp-transform length
        s = WallsSolutes(N=48, dx=0.2, eta=0.3, width=4.0, amp=0.05, seed=1)
        g = Grid(ctx, s.lat, s.shape)
        f = Fmt(g, R=s.R, kT=s.kT, mu=s.mu, terms=TERMS, mask=s.mask.reshape(-1))
        p = _lib.CgParams(_lib.LS_SECANT, 1e-9, 0, 1.0, 0.0, 0.0, _lib.PC_STRUCTURE, 0.0, 0.0, 0,
                          0)
        h = ctypes.c_void_p()
        assert f.L.deft_cg_create(f.h, ctypes.byref(p), ctypes.byref(h)) == _lib.ERR_ARG
        z = np.empty(g.size)
        n = s.n0.reshape(-1)
        assert f.L.deft_fmt_precondition(f.h, n.ctypes.data, n.ctypes.data, 0, z.ctypes.data,
                                         None) == _lib.ERR_ARG
        f.close()
        g.close()
        s = _problem(0)
        g = Grid(ctx, s.lat, s.shape)
        # the tensor White Bear kind; the quadratic line search
        f = Fmt(g, R=s.R, kT=s.kT, mu=s.mu, terms=TERMS, mask=s.mask.reshape(-1), functional=3)
        assert f.L.deft_cg_create(f.h, ctypes.byref(p), ctypes.byref(h)) == _lib.ERR_ARG
        f.close()
        f = Fmt(g, R=s.R, kT=s.kT, mu=s.mu, terms=TERMS, mask=s.mask.reshape(-1))
        q = _lib.CgParams(_lib.LS_QUADRATIC_REF, 1e-9, 0, 0.1, 0.0, 0.0, _lib.PC_STRUCTURE, 0.0,
                          0.0, 0, 0)
        assert f.L.deft_cg_create(f.h, ctypes.byref(q), ctypes.byref(h)) == _lib.ERR_ARG
        f.close()
        g.close()
    finally:
        ctx.close()


@pytest.mark.parametrize("precision", [_lib.PRECISION_MIXED, _lib.PRECISION_FP64])
def test_device_driven_structure_preconditioned_solve(precision):
    from tests.capi import CG, Ctx, Fmt, Grid
    s = _problem(1)
    mask = s.mask.reshape(-1)
    ctx = Ctx(0)
    g = Grid(ctx, s.lat, s.shape)
    f = Fmt(g, R=s.R, kT=s.kT, mu=s.mu, terms=TERMS, mask=mask, precision=precision)
    try:
        gtol = 3e-10 if precision == _lib.PRECISION_MIXED else 1e-9
        kw = dict(gtol=gtol, maxiter=3000, step=1.0, preconditioned=_lib.PC_STRUCTURE)
        host = CG(f, **kw)
        host.set_x(s.n0.reshape(-1))
        code, st_h = host.solve()
        assert code == 0 and st_h.converged
        it_h, ev_h, x_h = st_h.iter, st_h.evals, host.get_x()
        host.close()
        dev = CG(f, **kw)
        for rep in range(2):  # the second call replays the same graph
            dev.set_x(s.n0.reshape(-1))
            code, st_d = dev.solve_device()
            assert code == 0, _lib.load().deft_last_error()
            assert st_d.converged and st_d.gnorm < gtol
            x_d = dev.get_x()
            if rep == 0:
                first = x_d.copy()
            else:
                assert np.array_equal(x_d, first)
        dev.close()
        assert abs(st_d.iter - it_h) <= max(2, it_h // 5)
        assert abs(st_d.evals - ev_h) <= max(4, ev_h // 5)
        assert np.abs(x_d - x_h).max() <= 1e-8 * float(np.abs(x_h).max())
    finally:
        for o in (f, g, ctx):
            o.close()


@pytest.mark.parametrize("kind", [1, 2])
def test_structure_preconditioned_mixed_solve_other_kinds_and_vext(kind):
    """The mixed form on FP32 vectors with the structure preconditioner for
    the Rosenfeld and mark II kinds, with an external potential on the free
    points (a soft attraction to the walls): converges to the FP64 solution
    of the same functional within 1e-8 of the density scale, and its bulk
    density is the one deft_bulk_density gives."""
    from tests.capi import CG, Ctx, Fmt, Grid
    s = _problem(0)
    mask = s.mask.reshape(-1)
    ctx = Ctx(0)
    g = Grid(ctx, s.lat, s.shape)
    z = np.arange(s.shape[2]) * s.dx
    V = np.broadcast_to(-0.3 * np.exp(-((z - 1.0) / 0.6) ** 2), s.shape).reshape(-1).copy()
    terms = TERMS | _lib.TERM_VEXT
    f = Fmt(g, R=s.R, kT=s.kT, mu=s.mu, terms=terms, mask=mask, V=V,
            precision=_lib.PRECISION_MIXED, functional=kind)
    f64 = Fmt(g, R=s.R, kT=s.kT, mu=s.mu, terms=terms, mask=mask, V=V, functional=kind)
    try:
        nb_api = ctypes.c_double()
        _lib.check(f.L.deft_bulk_density(s.R, s.kT, s.mu, kind, ctypes.addressof(nb_api)))
        r = np.ones(g.size) * mask
        zz = np.empty(g.size)
        nb_pc = ctypes.c_double()
        _lib.check(f.L.deft_fmt_precondition(f.h, s.n0.reshape(-1).ctypes.data, r.ctypes.data, 0,
                                             zz.ctypes.data, ctypes.addressof(nb_pc)))
        assert nb_pc.value == nb_api.value
        cg = CG(f, gtol=3e-10, maxiter=3000, step=1.0, preconditioned=_lib.PC_STRUCTURE)
        cg.set_x(s.n0.reshape(-1))
        code, st = cg.solve()
        assert code == 0, _lib.load().deft_last_error()
        assert st.converged and st.stage == 1
        x = cg.get_x()
        cg.close()
        _, g64, _ = f64.energy_grad(x)
        assert np.linalg.norm(g64) < 3e-10
        ref = CG(f64, gtol=1e-12, maxiter=5000, step=1.0, preconditioned=_lib.PC_DENSITY)
        ref.set_x(s.n0.reshape(-1))
        code, st_r = ref.solve()
        assert code == 0 and st_r.converged
        x_ref = ref.get_x()
        ref.close()
        assert np.abs(x - x_ref).max() <= 1e-8 * float(np.abs(x_ref).max())
    finally:
        for o in (f64, f, g, ctx):
            o.close()
