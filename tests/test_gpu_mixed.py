"""GPU tests of the mixed form (FFTs, weights and phi in FP32; energies,
dot products, line search and the final refinement in FP64) against the FP64
oracle.  Stated tolerances: single mixed evaluation -- energy 2e-6 relative,
gradient 2e-5 relative to its max; converged mixed solve -- FP64 gradient
norm below the FP64 tolerance and profile within 1e-8 of the oracle's."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from tests.capi import Ctx
    c = Ctx(0)
    yield c
    c.close()


def _slit(N=32, Nxy=8):
    from deft_gb300.workloads import Slit
    return Slit(N=N, dx=0.2, eta=0.3, Nxy=Nxy, seed=1)


FCC = np.array([[0, 1.0, 1.0], [1.0, 0, 1.0], [1.0, 1.0, 0.0]])


# Shapes with x and y lengths of 32..256 run the register-resident pencil
# kernels for the x and y transforms; the others the shared-memory passes.
@pytest.mark.parametrize("shape,lat_kind", [
    ((8, 8, 32), "ortho"), ((16, 12, 15), "ortho"), ((48, 20, 10), "ortho"),
    ((32, 32, 16), "ortho"), ((64, 32, 20), "ortho"), ((32, 128, 12), "ortho"),
    ((256, 32, 8), "ortho"), ((32, 64, 24), "fcc"), ((64, 64, 64), "fcc"),
    ((32, 32, 32), "ortho"), ((128, 128, 128), "ortho"), ((64, 32, 256), "ortho")])
def test_mixed_energy_grad_vs_oracle(ctx, oracle_mod, shape, lat_kind):
    from deft_gb300 import _lib
    from tests.capi import Fmt, Grid
    O = oracle_mod
    rng = np.random.default_rng(4)
    lat = np.diag([0.2 * s for s in shape]) if lat_kind == "ortho" else \
        FCC * (0.15 * max(shape))
    nb = 0.3 / (4 * math.pi / 3)
    mu = O.find_mu(1.0, 1.0, nb)
    # noise clipped at 4 sigma: the large grids would otherwise draw a
    # negative density somewhere (the ideal gas's log is then undefined)
    n = nb * (1 + 0.2 * np.clip(rng.standard_normal(int(np.prod(shape))), -4, 4))
    P = O.Problem(lat, shape, mu=mu)
    Er, gr = P.energy_grad(n)
    g = Grid(ctx, lat, shape)
    f = Fmt(g, mu=mu, terms=P.terms, precision=_lib.PRECISION_MIXED)
    E, grad, _ = f.energy_grad(n)
    assert abs(E / Er - 1) < 2e-6
    assert np.abs(grad - gr).max() <= 2e-5 * np.abs(gr).max()
    f.close()
    g.close()


@pytest.mark.parametrize("Nxy", [8, 32])
def test_hessian_vector_matches_fp64_gradient_difference(ctx, oracle_mod, Nxy):
    """H dx against (g(n + e dx) - g(n - e dx)) / 2e of the FP64 gradient
    (Nxy = 32: pencil x and y transforms)."""
    from deft_gb300 import _lib
    from tests.capi import Fmt, Grid
    O = oracle_mod
    s = _slit(Nxy=Nxy)
    size = s.size
    mask = s.mask.reshape(-1)
    rng = np.random.default_rng(8)
    n = np.where(mask > 0, s.nb * (1 + 0.1 * rng.standard_normal(size)), 0.0)
    dx = rng.standard_normal(size) * s.nb * mask
    g = Grid(ctx, s.lat, s.shape)
    f64 = Fmt(g, mu=s.mu, terms=O.HS | O.IDEAL | O.MU | O.MASK, mask=mask)
    fmx = Fmt(g, mu=s.mu, terms=O.HS | O.IDEAL | O.MU | O.MASK, mask=mask,
              precision=_lib.PRECISION_MIXED)
    Hd = fmx.hessian_vector(n, dx)
    eps = 1e-4
    _, gp, _ = f64.energy_grad(n + eps * dx)
    _, gm, _ = f64.energy_grad(n - eps * dx)
    fd = (gp - gm) / (2 * eps)
    assert np.abs(Hd - fd).max() <= 1e-4 * np.abs(fd).max()
    assert np.all(Hd[mask == 0] == 0)
    f64.close()
    fmx.close()
    g.close()


@pytest.mark.parametrize("Nxy", [8, 32])
def test_mixed_solve_reaches_fp64_tolerance_and_profile(ctx, oracle_mod, Nxy):
    from deft_gb300 import _lib
    from tests.capi import CG, Fmt, Grid
    O = oracle_mod
    s = _slit(Nxy=Nxy)
    mask = s.mask.reshape(-1)
    g = Grid(ctx, s.lat, s.shape)
    f = Fmt(g, mu=s.mu, terms=O.HS | O.IDEAL | O.MU | O.MASK, mask=mask,
            precision=_lib.PRECISION_MIXED)
    cg = CG(f, gtol=1e-9, maxiter=2000, step=1.0)
    cg.set_x(s.n0.reshape(-1))
    code, st = cg.solve()
    assert code == 0 and st.converged and st.stage == 1
    n = cg.get_x()
    # the convergence test is the FP64 gradient: check it independently
    f64 = Fmt(g, mu=s.mu, terms=O.HS | O.IDEAL | O.MU | O.MASK, mask=mask)
    _, g64, _ = f64.energy_grad(n)
    assert np.linalg.norm(g64) < 1e-9
    P1 = O.Problem(np.diag([s.dx, s.dx, s.L]), (1, 1, s.shape[2]), mu=s.mu,
                   terms=O.HS | O.IDEAL | O.MU, mask=s.mask[0, 0].copy())
    x1, info = P1.cg_solve(np.where(s.mask[0, 0] > 0, s.nb, 0.0), gtol=1e-13, maxiter=20000)
    assert np.abs(n.reshape(s.shape) - x1[None, None, :]).max() < 1e-8
    assert st.evals_fp64 < st.evals  # most evaluations ran in FP32
    cg.close()
    f.close()
    f64.close()
    g.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_density_preconditioned_solve(ctx, oracle_mod, precision):
    """The density-variable preconditioner (M^-1 = n / (kT dV)): in FP64 the
    GPU iterates follow the oracle's (iteration and evaluation counts equal up
    to rounding, same profile); in the mixed form the FP32 stage uses it and the result
    meets the FP64 tolerance at the oracle's profile."""
    from deft_gb300 import _lib
    from tests.capi import CG, Fmt, Grid
    O = oracle_mod
    s = _slit()
    mask = s.mask.reshape(-1)
    g = Grid(ctx, s.lat, s.shape)
    terms = O.HS | O.IDEAL | O.MU | O.MASK
    f = Fmt(g, mu=s.mu, terms=terms, mask=mask, precision=precision)
    cg = CG(f, gtol=1e-9, maxiter=2000, step=1.0, preconditioned=_lib.PC_DENSITY)
    cg.set_x(s.n0.reshape(-1))
    code, st = cg.solve()
    assert code == 0 and st.converged
    n = cg.get_x()
    P1 = O.Problem(np.diag([s.dx, s.dx, s.L]), (1, 1, s.shape[2]), mu=s.mu,
                   terms=O.HS | O.IDEAL | O.MU, mask=s.mask[0, 0].copy())
    x1, _ = P1.cg_solve(np.where(s.mask[0, 0] > 0, s.nb, 0.0), gtol=1e-13, maxiter=20000)
    assert np.abs(n.reshape(s.shape) - x1[None, None, :]).max() < 1e-8
    if precision == 0:
        P = O.Problem(s.lat, s.shape, mu=s.mu, terms=terms, mask=mask)
        xo, info = P.cg_solve(s.n0.reshape(-1), gtol=1e-9, maxiter=2000, preconditioned=2)
        # same iterates up to rounding: the counts agree to a step or two
        assert abs(st.iter - info["iters"]) <= 2 and abs(st.evals - info["evals"]) <= 6
        assert np.abs(n - xo).max() <= 1e-8 * xo.max()
    else:
        f64 = Fmt(g, mu=s.mu, terms=terms, mask=mask)
        _, g64, _ = f64.energy_grad(n)
        assert np.linalg.norm(g64) < 1e-9 and st.stage == 1
        f64.close()
    cg.close()
    f.close()
    g.close()
