"""Device-driven solves (deft_cg_solve_device): the whole minimisation as one
CUDA graph launch (conditional WHILE / SWITCH / IF nodes, decisions taken by
kernels) against the host-driven minimiser it restates (deft_cg_solve with
DEFT_LS_SECANT and DEFT_PC_DENSITY), on wall + solute problems: both
converge, their profiles agree to 1e-8 of the density scale, and both agree
with the FP64 solution converged to |grad F| < 1e-12.  The loop budget ends
a solve with DEFT_ERR_TIMEOUT and leaves the context usable."""
import numpy as np
import pytest

from deft_gb300 import _lib

pytestmark = pytest.mark.gpu


def _setup(s, precision):
    from tests.capi import Ctx, Fmt, Grid
    ctx = Ctx(0)
    g = Grid(ctx, s.lat, s.shape)
    f = Fmt(g, R=s.R, kT=s.kT, mu=s.mu, terms=_lib.TERM_HS | _lib.TERM_IDEAL | _lib.TERM_MU |
            _lib.TERM_MASK, mask=s.mask.reshape(-1), precision=precision)
    return ctx, g, f


def _close(*objs):
    for o in objs:
        o.close()


def _problems():
    from deft_gb300.workloads import WallsSolutes
    return [WallsSolutes(N=32, dx=0.2, eta=0.3, width=4.0, solutes=[(3.2, 3.2, 2.0, 1.5)],
                         amp=0.05, seed=4),
            WallsSolutes(N=48, dx=0.2, eta=0.4, width=6.0,
                         solutes=[(2.0, 7.0, 3.0, 2.0), (6.0, 2.0, 1.0, 1.2)], amp=0.05, seed=5)]


@pytest.mark.parametrize("k", [0, 1])
@pytest.mark.parametrize("precision", [_lib.PRECISION_MIXED, _lib.PRECISION_FP64])
def test_device_driven_solve_matches_host_driven(k, precision):
    from tests.capi import CG, Fmt
    s = _problems()[k]
    ctx, g, f = _setup(s, precision)
    f64 = Fmt(g, R=s.R, kT=s.kT, mu=s.mu, terms=_lib.TERM_HS | _lib.TERM_IDEAL | _lib.TERM_MU |
              _lib.TERM_MASK, mask=s.mask.reshape(-1), precision=_lib.PRECISION_FP64)
    try:
        gtol = 5e-10 if precision == _lib.PRECISION_MIXED else 1e-9
        kw = dict(linesearch=_lib.LS_SECANT, gtol=gtol, maxiter=2000, step=1.0,
                  preconditioned=_lib.PC_DENSITY)
        host = CG(f, **kw)
        host.set_x(s.n0.reshape(-1))
        code, st_h = host.solve()
        assert code == 0 and st_h.converged
        it_h, ev_h = st_h.iter, st_h.evals
        x_h = host.get_x()
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
        # the same algorithm: counts close to the host-driven run's
        assert abs(st_d.iter - it_h) <= max(2, it_h // 5)
        assert abs(st_d.evals - ev_h) <= max(4, ev_h // 5)
        scale = float(np.abs(x_h).max())
        assert np.abs(x_d - x_h).max() <= 1e-8 * scale
        # and both near the FP64 solution converged to 1e-12
        ref = CG(f64, linesearch=_lib.LS_SECANT, gtol=1e-12, maxiter=5000, step=1.0,
                 preconditioned=_lib.PC_DENSITY)
        ref.set_x(s.n0.reshape(-1))
        code, st = ref.solve()
        assert code == 0 and st.converged
        x_ref = ref.get_x()
        ref.close()
        assert np.abs(x_d - x_ref).max() <= 1e-8 * scale
    finally:
        _close(f64, f, g, ctx)


def test_device_loop_budget_gives_timeout_and_leaves_the_context_usable():
    from tests.capi import CG
    s = _problems()[0]
    ctx, g, f = _setup(s, _lib.PRECISION_MIXED)
    try:
        cg = CG(f, linesearch=_lib.LS_SECANT, gtol=5e-10, maxiter=0, step=1.0,
                preconditioned=_lib.PC_DENSITY, device_loops=5)
        cg.set_x(s.n0.reshape(-1))
        code, st = cg.solve_device()
        assert code == _lib.ERR_TIMEOUT and st.status == _lib.ERR_TIMEOUT
        assert not st.converged and st.evals + st.hvps == 5
        assert np.isfinite(cg.get_x()).all()
        cg.close()
        # a solve with the default budget on the same grid still converges
        cg = CG(f, linesearch=_lib.LS_SECANT, gtol=5e-10, maxiter=2000, step=1.0,
                preconditioned=_lib.PC_DENSITY)
        cg.set_x(s.n0.reshape(-1))
        code, st = cg.solve_device()
        assert code == 0 and st.converged
        cg.close()
    finally:
        _close(f, g, ctx)


def test_device_driven_solve_refuses_unsupported_settings():
    from tests.capi import CG
    s = _problems()[0]
    ctx, g, f = _setup(s, _lib.PRECISION_MIXED)
    try:
        for kw in (dict(linesearch=_lib.LS_QUADRATIC_REF, preconditioned=_lib.PC_NONE),
                   dict(linesearch=_lib.LS_SECANT, preconditioned=_lib.PC_NONE),
                   dict(linesearch=_lib.LS_SECANT, preconditioned=_lib.PC_DENSITY,
                        precision=1e-6)):
            cg = CG(f, gtol=1e-9, **kw)
            cg.set_x(s.n0.reshape(-1))
            code, _ = cg.solve_device()
            assert code == _lib.ERR_ARG
            cg.close()
    finally:
        _close(f, g, ctx)
