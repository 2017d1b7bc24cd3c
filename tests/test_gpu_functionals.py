"""GPU tests of the Rosenfeld (HardSpheresRF), White Bear mark II, tensor
White Bear (HardSpheresWB) and Tarazona functionals: FP64 energies and
gradients against the reference's outputs (tests/golden/) and the oracle, the mixed form within its FP32 tolerances
(energy 2e-6, gradient 2e-5 relative), the Hessian-vector product of the
Newton refinement against a difference of FP64 gradients, and a converged
mixed solve at the oracle's profile.  Stated FP64 tolerances: energy 1e-10,
gradient 1e-9 relative."""
import numpy as np
import pytest

from deft_gb300 import _lib

pytestmark = pytest.mark.gpu

KINDS = [_lib.HS_RF, _lib.HS_WB_MARK2]


@pytest.fixture(scope="module")
def golden():
    import json
    import os
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "golden", "reference_values.json")) as f:
        vals = json.load(f)
    return vals, np.load(os.path.join(here, "golden", "reference_fields.npz"))


@pytest.fixture(scope="module")
def ctx():
    from tests.capi import Ctx
    c = Ctx(0)
    yield c
    c.close()


def _slit(N=32, Nxy=8):
    from deft_gb300.workloads import Slit
    return Slit(N=N, dx=0.2, eta=0.3, Nxy=Nxy, seed=1)


@pytest.mark.parametrize("name", ["cubic12", "ortho_odd"])
@pytest.mark.parametrize("hs", KINDS)
def test_fp64_matches_reference_golden(ctx, oracle_mod, golden, name, hs):
    from tests.capi import Fmt, Grid
    from tests.golden.cases import make_case
    vals, arrs = golden
    P, n = make_case(name, hs)
    g = Grid(ctx, P.lat.reshape(3, 3), P.N)
    f = Fmt(g, R=P.R, kT=P.kT, mu=P.mu, terms=P.terms, V=P.V, mask=P.mask, functional=hs)
    E, grad, terms = f.energy_grad(n)
    ref = vals[f"{name}_hs{hs}"]
    assert abs(E / ref["E"] - 1) < 1e-10
    tr = np.array(ref["terms"])
    assert np.abs(terms[:len(tr)] - tr).max() <= 1e-10 * np.abs(tr).max()
    gr = arrs[f"{name}_hs{hs}_grad"]
    assert np.abs(grad - gr).max() <= 1e-9 * np.abs(gr).max()
    f.close()
    g.close()


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("hs", KINDS)
def test_slit_with_empty_walls_vs_oracle(ctx, oracle_mod, hs, precision):
    """n = 0 across walls wider than the sphere diameter: n3 reaches 0 there,
    which exercises the series branches of the prefactors."""
    from tests.capi import Fmt, Grid
    O = oracle_mod
    s = _slit()
    mask = s.mask.reshape(-1)
    rng = np.random.default_rng(12)
    n = np.where(mask > 0, s.nb * (1 + 0.1 * rng.standard_normal(s.size)), 0.0)
    terms = O.HS | O.IDEAL | O.MU | O.MASK
    P = O.Problem(s.lat, s.shape, mu=s.mu, terms=terms, mask=mask, hs=hs)
    Er, gr = P.energy_grad(n)
    g = Grid(ctx, s.lat, s.shape)
    f = Fmt(g, mu=s.mu, terms=terms, mask=mask, precision=precision, functional=hs)
    E, grad, _ = f.energy_grad(n)
    etol, gtol = (1e-10, 1e-9) if precision == 0 else (2e-6, 2e-5)
    assert abs(E / Er - 1) < etol
    assert np.abs(grad - gr).max() <= gtol * np.abs(gr).max()
    f.close()
    g.close()


@pytest.mark.parametrize("hs", KINDS)
def test_hessian_vector_matches_fp64_gradient_difference(ctx, oracle_mod, hs):
    from tests.capi import Fmt, Grid
    O = oracle_mod
    s = _slit()
    mask = s.mask.reshape(-1)
    rng = np.random.default_rng(8)
    n = np.where(mask > 0, s.nb * (1 + 0.1 * rng.standard_normal(s.size)), 0.0)
    dx = rng.standard_normal(s.size) * s.nb * mask
    g = Grid(ctx, s.lat, s.shape)
    terms = O.HS | O.IDEAL | O.MU | O.MASK
    f64 = Fmt(g, mu=s.mu, terms=terms, mask=mask, functional=hs)
    fmx = Fmt(g, mu=s.mu, terms=terms, mask=mask, precision=_lib.PRECISION_MIXED,
              functional=hs)
    Hd = fmx.hessian_vector(n, dx)
    eps = 1e-4
    _, gp, _ = f64.energy_grad(n + eps * dx)
    _, gm, _ = f64.energy_grad(n - eps * dx)
    fd = (gp - gm) / (2 * eps)
    assert np.abs(Hd - fd).max() <= 1e-4 * np.abs(fd).max()
    f64.close()
    fmx.close()
    g.close()


@pytest.mark.parametrize("hs", KINDS)
def test_mixed_solve_reaches_fp64_tolerance_at_oracle_profile(ctx, oracle_mod, hs):
    from tests.capi import CG, Fmt, Grid
    O = oracle_mod
    s = _slit()
    mask = s.mask.reshape(-1)
    terms = O.HS | O.IDEAL | O.MU | O.MASK
    g = Grid(ctx, s.lat, s.shape)
    f = Fmt(g, mu=s.mu, terms=terms, mask=mask, precision=_lib.PRECISION_MIXED, functional=hs)
    cg = CG(f, gtol=1e-9, maxiter=2000, step=1.0, preconditioned=_lib.PC_DENSITY)
    cg.set_x(s.n0.reshape(-1))
    code, st = cg.solve()
    assert code == 0 and st.converged and st.stage == 1
    n = cg.get_x()
    f64 = Fmt(g, mu=s.mu, terms=terms, mask=mask, functional=hs)
    _, g64, _ = f64.energy_grad(n)
    assert np.linalg.norm(g64) < 1e-9
    P1 = O.Problem(np.diag([s.dx, s.dx, s.L]), (1, 1, s.shape[2]), mu=s.mu,
                   terms=O.HS | O.IDEAL | O.MU, mask=s.mask[0, 0].copy(), hs=hs)
    x1, info = P1.cg_solve(np.where(s.mask[0, 0] > 0, s.nb, 0.0), gtol=1e-13, maxiter=20000)
    assert info["gnorm"] < 1e-13
    assert np.abs(n.reshape(s.shape) - x1[None, None, :]).max() < 1e-8
    cg.close()
    f64.close()
    f.close()
    g.close()


def test_unknown_functional_is_refused(ctx):
    from tests.capi import Grid
    g = Grid(ctx, np.diag([2.4, 2.4, 2.4]), (12, 12, 12))
    p = _lib.FmtParams(1.0, 1.0, 0.0, 7, 0, 9)
    import ctypes
    h = ctypes.c_void_p()
    assert g.L.deft_fmt_create(g.h, ctypes.byref(p), ctypes.byref(h)) == _lib.ERR_ARG
    g.close()


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name,hs", [("cubic12", 3), ("ortho_odd", 3), ("fcc12", 3),
                                     ("cubic12", 4), ("fcc12", 4)])
def test_tensor_matches_reference_golden(ctx, oracle_mod, golden, name, hs, precision):
    """The compiled HardSpheresWB / HardSpheresTarazona energy, per-term
    energies and gradient: FP64 form to 1e-10 / 1e-9; mixed form (eleven
    convolutions in FP32) to 1e-6 / 1e-4 of the largest entry."""
    from tests.capi import Fmt, Grid
    from tests.golden.cases import make_case
    vals, arrs = golden
    P, n = make_case(name, hs)
    g = Grid(ctx, P.lat.reshape(3, 3), P.N)
    f = Fmt(g, R=P.R, kT=P.kT, mu=P.mu, terms=P.terms, V=P.V, mask=P.mask, functional=hs,
            precision=precision)
    E, grad, terms = f.energy_grad(n)
    ref = vals[f"{name}_hs{hs}"]
    e_tol, g_tol = (1e-10, 1e-9) if precision == 0 else (1e-6, 1e-4)
    assert abs(E / ref["E"] - 1) < e_tol
    tr = np.array(ref["terms"])
    assert np.abs(terms[:len(tr)] - tr).max() <= e_tol * np.abs(tr).max()
    gr = arrs[f"{name}_hs{hs}_grad"]
    assert np.abs(grad - gr).max() <= g_tol * np.abs(gr).max()
    E2, _ = f.energy(n)
    assert abs(E2 / E - 1) < (1e-14 if precision == 0 else 1e-6)
    f.close()
    g.close()


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("hs", [_lib.HS_WB_TENSOR, _lib.HS_TARAZONA])
def test_tensor_secant_solve_matches_oracle_profile(ctx, oracle_mod, hs, precision):
    """CG with the tensor functional on the slit, to |grad| < 1e-10 (the
    mixed form: FP32 stage, then FP64 CG): the profile equals the oracle's
    1-D solve of the same functional."""
    from tests.capi import CG, Fmt, Grid
    O = oracle_mod
    s = _slit()
    mask = s.mask.reshape(-1)
    terms = O.HS | O.IDEAL | O.MU | O.MASK
    g = Grid(ctx, s.lat, s.shape)
    f = Fmt(g, mu=s.mu, terms=terms, mask=mask, functional=hs, precision=precision)
    cg = CG(f, gtol=1e-10, maxiter=5000, step=1.0, preconditioned=_lib.PC_DENSITY)
    cg.set_x(s.n0.reshape(-1))
    code, st = cg.solve()
    assert code == 0 and st.converged
    n = cg.get_x()
    P1 = O.Problem(np.diag([s.dx, s.dx, s.L]), (1, 1, s.shape[2]), mu=s.mu,
                   terms=O.HS | O.IDEAL | O.MU, mask=s.mask[0, 0].copy(), hs=hs)
    x1, info = P1.cg_solve(np.where(s.mask[0, 0] > 0, s.nb, 0.0), gtol=1e-13, maxiter=20000)
    assert info["gnorm"] < 1e-13
    assert np.abs(n.reshape(s.shape) - x1[None, None, :]).max() < 1e-8
    cg.close()
    f.close()
    g.close()


def test_tensor_functionals_have_no_hessian_vector_product(ctx):
    """The Newton step's FP32 Hessian covers the vector kinds only: the
    tensor kinds' mixed form refines by FP64 CG, and the product is refused."""
    import ctypes
    from tests.capi import Fmt, Grid
    g = Grid(ctx, np.diag([2.4, 2.4, 2.4]), (12, 12, 12))
    f = Fmt(g, R=1.0, kT=1.0, mu=0.0, terms=7, precision=_lib.PRECISION_MIXED,
            functional=_lib.HS_WB_TENSOR)
    n = np.full(12 ** 3, 0.05)
    out = np.empty_like(n)
    assert f.L.deft_fmt_hessian_vector(f.h, n.ctypes.data, n.ctypes.data, 0,
                                       out.ctypes.data) == _lib.ERR_ARG
    f.close()
    g.close()
