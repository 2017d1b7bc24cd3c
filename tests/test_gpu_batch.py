"""Batched solves (many state points and uneven grids on one GPU): every
problem of a batch must match the same problem solved on its own with the
same precision -- both stop at |grad F| < 1e-9, so the profiles agree to
within 1e-8 (the stated tolerance)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_matches_individual_solves(precision):
    from deft_gb300.workloads import batch_sweep
    from tests.capi import CG, Ctx, Fmt, Grid, batch_solve
    probs = batch_sweep(count=6, seed=5, sizes=(32, 48))
    code, st, outs = batch_solve(probs, precision=precision, workers=3)
    assert code == 0
    ctx = Ctx(0)
    for s, stat, out in zip(probs, st, outs):
        assert stat.converged and stat.gnorm < 1e-9
        g = Grid(ctx, s.lat, s.shape)
        f = Fmt(g, mu=s.mu, terms=1 | 2 | 4 | 16, mask=s.mask.reshape(-1), precision=precision)
        cg = CG(f, gtol=1e-9, maxiter=20000)
        cg.set_x(s.n0.reshape(-1))
        c2, st2 = cg.solve()
        assert c2 == 0 and st2.converged
        ref = cg.get_x()
        assert np.abs(out - ref).max() < 1e-8
        # masked (wall) points stay exactly zero
        assert np.all(out[s.mask.reshape(-1) == 0] == 0)
        cg.close()
        f.close()
        g.close()
    ctx.close()


def test_device_batch_matches_individual_solves():
    """deft_batch_solve_device: the whole batch as one graph launch of
    device-driven solves (mixed form, density preconditioner) over the
    sweep's grid mix, 32^3 to 128^3; every problem converges and matches its
    own host-driven solve to 1e-8."""
    from deft_gb300 import _lib
    from deft_gb300.workloads import batch_sweep
    from tests.capi import CG, Ctx, Fmt, Grid, batch_solve
    probs = batch_sweep(count=6, seed=7, sizes=(32, 48, 64, 96, 128))
    code, st, outs = batch_solve(probs, precision=1, gtol=5e-10, device_driven=True)
    assert code == 0, _lib.load().deft_last_error()
    ctx = Ctx(0)
    for s, stat, out in zip(probs, st, outs):
        assert stat.converged and stat.gnorm < 5e-10 and stat.status == 0
        g = Grid(ctx, s.lat, s.shape)
        f = Fmt(g, mu=s.mu, terms=1 | 2 | 4 | 16, mask=s.mask.reshape(-1), precision=1)
        cg = CG(f, gtol=5e-10, maxiter=20000, preconditioned=_lib.PC_DENSITY)
        cg.set_x(s.n0.reshape(-1))
        c2, st2 = cg.solve()
        assert c2 == 0 and st2.converged
        ref = cg.get_x()
        assert np.abs(out - ref).max() < 1e-8
        assert np.all(out[s.mask.reshape(-1) == 0] == 0)
        cg.close()
        f.close()
        g.close()
    ctx.close()


def test_device_batch_with_the_structure_preconditioner():
    """deft_batch_solve_device with DEFT_PC_STRUCTURE over the 32^3-128^3
    mix: the 48^3 and 96^3 problems (no warp z transform) fall back to the
    density preconditioner; every problem converges and matches its own
    host-driven solve with the same preconditioner to 1e-8."""
    from deft_gb300 import _lib
    from deft_gb300.workloads import batch_sweep
    from tests.capi import CG, Ctx, Fmt, Grid, batch_solve
    probs = batch_sweep(count=6, seed=11, sizes=(32, 48, 64, 96, 128))
    code, st, outs = batch_solve(probs, precision=1, gtol=3e-10, device_driven=True,
                                 preconditioned=_lib.PC_STRUCTURE)
    assert code == 0, _lib.load().deft_last_error()
    ctx = Ctx(0)
    for s, stat, out in zip(probs, st, outs):
        assert stat.converged and stat.gnorm < 3e-10 and stat.status == 0
        g = Grid(ctx, s.lat, s.shape)
        f = Fmt(g, mu=s.mu, terms=1 | 2 | 4 | 16, mask=s.mask.reshape(-1), precision=1)
        pc = _lib.PC_STRUCTURE if s.shape[2] in (32, 64, 128, 256) else _lib.PC_DENSITY
        cg = CG(f, gtol=3e-10, maxiter=20000, preconditioned=pc)
        cg.set_x(s.n0.reshape(-1))
        c2, st2 = cg.solve()
        assert c2 == 0 and st2.converged
        ref = cg.get_x()
        assert np.abs(out - ref).max() < 1e-8
        assert np.all(out[s.mask.reshape(-1) == 0] == 0)
        cg.close()
        f.close()
        g.close()
    ctx.close()
