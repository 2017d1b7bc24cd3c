"""The hard-sphere solute workload at its stated size: a 256^3 periodic grid
with dx = 0.1 (edge 25.6), eta = 0.35, n = 0 and frozen degrees of freedom
within radius 3 of the cell centre (the cavity geometry of
papers/contact/figs/sphere.cpp:90-105), White Bear + ideal gas + mu.

FP64 form against the oracle (free energy 1e-10 relative, gradient 1e-9
relative to its max); the mixed form's evaluation errors against the FP64
form; and the mixed solve's converged profile against a tightly converged
FP64 solve (within 1e-8, the profile condition of the converged-solve
target)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

E_TOL = 1e-10
G_TOL = 1e-9
PROFILE_TOL = 1e-8


@pytest.fixture(scope="module")
def solute():
    from deft_gb300.workloads import Solute
    return Solute(N=256, dx=0.1, eta=0.35, r_excl=3.0, seed=2)


@pytest.fixture(scope="module")
def ctx():
    from tests.capi import Ctx
    c = Ctx(0)
    yield c
    c.close()


def _fmt(ctx, s, precision):
    from tests.capi import Fmt, Grid
    from deft_gb300 import _lib
    g = Grid(ctx, s.lat, s.shape)
    terms = _lib.TERM_HS | _lib.TERM_IDEAL | _lib.TERM_MU | _lib.TERM_MASK
    return g, Fmt(g, R=s.R, kT=s.kT, mu=s.mu, terms=terms, mask=s.mask.reshape(-1),
                  precision=precision)


def test_fp64_energy_grad_256_matches_oracle(ctx, oracle_mod, solute):
    O = oracle_mod
    s = solute
    g, f = _fmt(ctx, s, 0)
    n = s.n0.reshape(-1)
    E, grad, _ = f.energy_grad(n)
    f.close()
    g.close()
    P = O.Problem(s.lat, s.shape, mu=s.mu, terms=O.HS | O.IDEAL | O.MU, mask=s.mask.reshape(-1))
    Er, gr = P.energy_grad(n)
    assert abs(E / Er - 1) < E_TOL
    assert np.abs(grad - gr).max() <= G_TOL * np.abs(gr).max()


def test_mixed_energy_grad_256_errors(ctx, solute):
    """The mixed form (FP32 transforms and phi, FP64 reductions) at 256^3:
    errors against the FP64 form on the same input, printed and bounded."""
    s = solute
    g, f = _fmt(ctx, s, 0)
    _, fm = _fmt(ctx, s, 1)
    n = s.n0.reshape(-1)
    E, grad, _ = f.energy_grad(n)
    Em, gm, _ = fm.energy_grad(n)
    fm.close()
    f.close()
    g.close()
    dE = abs(Em / E - 1)
    dg = float(np.abs(gm - grad).max() / np.abs(grad).max())
    print(f"256^3 mixed vs FP64: |dF|/|F| = {dE:.3e}, max|dg|/max|g| = {dg:.3e}")
    assert dE < 1e-6
    assert dg < 1e-4


def test_mixed_solve_256_profile_matches_fp64(ctx, solute):
    """Mixed solve (FP32 CG stage, Newton refinement on the FP64 gradient)
    to |grad F| < 1e-9 against the FP64 solve tightened to 1e-12: the
    converged profiles agree within 1e-8 (max |dn|, and relative to max n)."""
    from tests.capi import CG
    from deft_gb300 import _lib
    s = solute
    g, f = _fmt(ctx, s, 0)
    _, fm = _fmt(ctx, s, 1)
    ref = CG(f, gtol=1e-12, maxiter=20000, preconditioned=_lib.PC_DENSITY)
    ref.set_x(s.n0.reshape(-1))
    code, st = ref.solve()
    assert code == 0 and st.converged and st.gnorm < 1e-12
    x_ref = ref.get_x()
    cg = CG(fm, gtol=1e-9, maxiter=20000, preconditioned=_lib.PC_DENSITY)
    cg.set_x(s.n0.reshape(-1))
    code, st = cg.solve()
    assert code == 0 and st.converged and st.gnorm < 1e-9
    x = cg.get_x()
    for h in (cg, ref, fm, f, g):
        h.close()
    d = float(np.abs(x - x_ref).max())
    print(f"256^3 mixed solve: {st.iter} iterations, {st.evals} evaluations "
          f"({st.evals_fp64} FP64), {st.hvps} Hessian-vector products; max|dn| = {d:.3e}, "
          f"relative to max n {d / np.abs(x_ref).max():.3e}")
    assert d <= PROFILE_TOL
    assert d <= PROFILE_TOL * np.abs(x_ref).max()
