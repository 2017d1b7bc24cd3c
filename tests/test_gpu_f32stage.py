"""The mixed form on FP32 vectors (on grids whose z lines the warp transforms
take: Nz = 32, 64, 128, 256): the FP32 stage (the secant CG with the
density preconditioner) and the Newton refinement's linear CG keep their
vectors in FP32.  Their preconditioner, direction, step and update kernels
run on FP32 vectors (their launches are counted under the FP32 kinds, none
under the FP64 ones), the solve meets the FP64 gradient tolerance at the
profile of a tightly converged FP64 solve, and a run checkpointed inside
the FP32 stage and restored into a fresh minimiser continues
bit-identically."""
import ctypes
import os

import numpy as np
import pytest

from deft_gb300 import _lib

pytestmark = pytest.mark.gpu


def _problem(k):
    from deft_gb300.workloads import WallsSolutes
    return [WallsSolutes(N=32, dx=0.2, eta=0.3, width=4.0, solutes=[(3.2, 3.2, 2.0, 1.5)],
                         amp=0.05, seed=4),
            WallsSolutes(N=64, dx=0.2, eta=0.4, width=8.0,
                         solutes=[(2.0, 7.0, 3.0, 2.0), (9.0, 4.0, 5.0, 1.2)], amp=0.05,
                         seed=6)][k]


def _fmt(g, s, precision):
    from tests.capi import Fmt
    return Fmt(g, R=s.R, kT=s.kT, mu=s.mu, terms=_lib.TERM_HS | _lib.TERM_IDEAL | _lib.TERM_MU |
               _lib.TERM_MASK, mask=s.mask.reshape(-1), precision=precision)


def _launches(L, grid):
    name = ctypes.c_char_p()
    launches = ctypes.c_longlong()
    tot = ctypes.c_double()
    out = {}
    for i in range(L.deft_grid_profile_count(grid.h)):
        _lib.check(L.deft_grid_profile_entry(grid.h, i, ctypes.byref(name),
                                             ctypes.addressof(launches), ctypes.addressof(tot)))
        out[name.value.decode()] = launches.value
    return out


@pytest.mark.parametrize("k", [0, 1])
def test_fp32_stage_on_fp32_vectors_meets_fp64_tolerance(k):
    from tests.capi import CG, Ctx, Grid
    s = _problem(k)
    ctx = Ctx(0)
    g = Grid(ctx, s.lat, s.shape)
    f = _fmt(g, s, _lib.PRECISION_MIXED)
    f64 = _fmt(g, s, _lib.PRECISION_FP64)
    try:
        gtol = 5e-10
        _lib.check(g.L.deft_grid_profile(g.h, 0))
        cg = CG(f, linesearch=_lib.LS_SECANT, gtol=gtol, maxiter=2000, step=1.0,
                preconditioned=_lib.PC_DENSITY)
        cg.set_x(s.n0.reshape(-1))
        code, st = cg.solve()
        assert code == 0, _lib.load().deft_last_error()
        assert st.converged and st.stage == 1
        x = cg.get_x()
        cg.close()
        n = _launches(g.L, g)
        assert n["precond_dots_f32"] > 0 and n["axpy_f32"] > 0
        assert n["precond_dots"] == 0  # no FP64-vector stage ran
        assert n["newton_update_f32"] > 0 and n["newton_update"] == 0
        # the stop test is the FP64 gradient: check it independently
        _, g64, _ = f64.energy_grad(x)
        assert np.linalg.norm(g64) < gtol
        ref = CG(f64, linesearch=_lib.LS_SECANT, gtol=1e-12, maxiter=5000, step=1.0,
                 preconditioned=_lib.PC_DENSITY)
        ref.set_x(s.n0.reshape(-1))
        code, st_r = ref.solve()
        assert code == 0 and st_r.converged
        x_ref = ref.get_x()
        ref.close()
        assert np.abs(x - x_ref).max() <= 1e-8 * float(np.abs(x_ref).max())
        assert np.all(x[s.mask.reshape(-1) == 0] == 0)
    finally:
        for o in (f64, f, g, ctx):
            o.close()


def test_checkpoint_inside_the_fp32_stage_resumes_bit_identically(tmp_path):
    from tests.capi import CG, Ctx, Grid
    s = _problem(0)
    ctx = Ctx(0)
    g = Grid(ctx, s.lat, s.shape)
    f = _fmt(g, s, _lib.PRECISION_MIXED)
    path = os.path.join(tmp_path, "cg.bin").encode()
    kw = dict(linesearch=_lib.LS_SECANT, gtol=5e-10, maxiter=0, step=1.0,
              preconditioned=_lib.PC_DENSITY)
    try:
        a = CG(f, **kw)
        a.set_x(s.n0.reshape(-1))
        for _ in range(3):
            code, st = a.step()
            assert code == 0 and st.stage == 0
        _lib.check(f.L.deft_cg_checkpoint(a.h, path))
        for _ in range(4):
            code, st_a = a.step()
            assert code == 0
        xa = a.get_x()
        a.close()
        b = CG(f, **kw)
        _lib.check(f.L.deft_cg_restore(b.h, path))
        for _ in range(4):
            code, st_b = b.step()
            assert code == 0
        xb = b.get_x()
        b.close()
        assert st_a.iter == st_b.iter and st_a.evals == st_b.evals
        assert st_a.energy == st_b.energy and st_a.stage == st_b.stage
        assert np.array_equal(xa, xb)
    finally:
        for o in (f, g, ctx):
            o.close()
