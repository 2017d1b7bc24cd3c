"""GPU parity of the effective-potential parametrisation
(constrain(mask, OfEffectivePotential(HS + ideal + mu)),
src/EffectivePotentialToDensity.cpp:28-91) and of the preconditioned CG
(src/ConjugateGradient.cpp:115-160): the sm_103a path through the C ABI
against the golden fixtures of the unmodified reference and the oracle.

Tolerances (FP64): energy 1e-10 relative, gradient and preconditioned
gradient 1e-9 relative to their max."""
import json
import os

import numpy as np
import pytest

from deft_gb300 import _lib

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def golden():
    with open(os.path.join(HERE, "golden", "reference_values.json")) as f:
        vals = json.load(f)
    return vals, np.load(os.path.join(HERE, "golden", "reference_fields.npz"))


def _setup(P, precision=0):
    from tests.capi import Ctx, Fmt, Grid
    ctx = Ctx(0)
    g = Grid(ctx, P.lat.reshape(3, 3), P.N)
    f = Fmt(g, R=P.R, kT=P.kT, mu=P.mu, terms=P.terms, V=P.V, mask=P.mask, precision=precision)
    return ctx, g, f


def _close(*objs):
    for o in objs:
        o.close()


def test_energy_grad_pgrad_match_reference(oracle_mod, golden):
    from tests.golden.cases import veff_case
    vals, arrs = golden
    P, x, _, _ = veff_case()
    ctx, g, f = _setup(P)
    try:
        E, gr, pg = f.energy_grad_pgrad(x)
        assert abs(E / vals["veff"]["E"] - 1) < 1e-10
        assert np.abs(gr - arrs["veff_grad"]).max() <= 1e-9 * np.abs(arrs["veff_grad"]).max()
        assert np.abs(pg - arrs["veff_pgrad"]).max() <= 1e-9 * np.abs(arrs["veff_pgrad"]).max()
        # deft_fmt_energy_grad gives the same gradient, deft_fmt_energy the same energy
        E2, g2, _ = f.energy_grad(x)
        assert E2 == E and np.array_equal(g2, gr)
        assert f.energy(x)[0] == E
        # the weighted densities are those of n = exp(-x/kT)
        w = f.weighted(x)
        wo = P.weighted(np.exp(-x / P.kT))
        assert np.abs(w - wo).max() <= 1e-12 * np.abs(wo).max()
        # Hessian-vector products stay in the density variable
        out = np.empty_like(x)
        code = f.L.deft_fmt_hessian_vector(f.h, x.ctypes.data, x.ctypes.data, 0, out.ctypes.data)
        assert code == _lib.ERR_ARG
    finally:
        _close(f, g, ctx)


def test_energy_grad_pgrad_match_oracle_random(oracle_mod):
    """Random lattice, V_ext and mask, effective potential around bulk."""
    O = oracle_mod
    rng = np.random.default_rng(21)
    N = (12, 10, 15)
    lat = np.array([[2.6, 0.1, 0.0], [0.0, 2.2, -0.1], [0.2, 0.0, 3.0]])
    size = int(np.prod(N))
    nb = 0.25 / (4 * np.pi / 3)
    P = O.Problem(lat, N, R=0.9, kT=1.2, mu=O.find_mu(0.9, 1.2, nb),
                  terms=O.HS | O.IDEAL | O.MU | O.VEFF, V=0.2 * rng.standard_normal(size),
                  mask=(rng.random(size) > 0.15).astype(float))
    x = -P.kT * np.log(nb * (1 + 0.2 * rng.random(size)))
    E, gr, pg = P.energy_grad_pgrad(x)
    ctx, g, f = _setup(P)
    try:
        Eg, gg, pgg = f.energy_grad_pgrad(x)
        assert abs(Eg / E - 1) < 1e-10
        assert np.abs(gg - gr).max() <= 1e-9 * np.abs(gr).max()
        assert np.abs(pgg - pg).max() <= 1e-9 * np.abs(pg).max()
    finally:
        _close(f, g, ctx)


def test_pcg_quadratic_matches_reference_trajectory(oracle_mod, golden):
    """PreconditionedConjugateGradient + QuadraticLineMinimizer on the GPU:
    energy after each improve_energy() against the reference's."""
    from tests.capi import CG
    from tests.golden.cases import veff_case
    vals, _ = golden
    P, x, iters, step = veff_case()
    er = np.array(vals["pcg_quadratic"]["energies"])
    ctx, g, f = _setup(P)
    cg = CG(f, linesearch=_lib.LS_QUADRATIC_REF, step=step, preconditioned=1)
    try:
        cg.set_x(x)
        e = []
        for _ in range(len(er)):
            s, st = cg.step()
            assert s == 0
            e.append(st.energy)
        assert np.abs(np.array(e) / er - 1).max() < 1e-10
    finally:
        _close(cg, f, g, ctx)


@pytest.mark.parametrize("preconditioned", [0, 1])
def test_secant_cg_in_effective_potential_converges_to_oracle_profile(oracle_mod, preconditioned):
    from tests.capi import CG
    from tests.golden.cases import veff_case
    P, x0, _, _ = veff_case()
    xo, info = P.cg_solve(x0, gtol=1e-12, maxiter=5000, preconditioned=bool(preconditioned))
    assert info["gnorm"] < 1e-12
    no = np.exp(-xo / P.kT)
    ctx, g, f = _setup(P)
    cg = CG(f, gtol=1e-12, maxiter=5000, step=1.0, preconditioned=preconditioned)
    try:
        cg.set_x(x0)
        s, st = cg.solve()
        assert s == 0 and st.converged and st.gnorm < 1e-12
        n = np.exp(-cg.get_x() / P.kT)
        free = P.mask > 0
        assert np.abs(n - no)[free].max() <= 1e-8 * no[free].max()
    finally:
        _close(cg, f, g, ctx)


def test_mixed_form_in_effective_potential_refines_in_fp64(oracle_mod):
    """Mixed evaluator with the effective potential: FP32 CG stage, then FP64
    CG to the tolerance; the profile matches the FP64 solve."""
    from tests.capi import CG
    from tests.golden.cases import veff_case
    P, x0, _, _ = veff_case()
    xo, info = P.cg_solve(x0, gtol=1e-12, maxiter=5000)
    no = np.exp(-xo / P.kT)
    ctx, g, f = _setup(P, precision=_lib.PRECISION_MIXED)
    cg = CG(f, gtol=1e-12, maxiter=5000, step=1.0, preconditioned=1)
    try:
        cg.set_x(x0)
        s, st = cg.solve()
        assert s == 0 and st.converged and st.gnorm < 1e-12 and st.stage == 1
        assert st.evals_fp64 < st.evals
        n = np.exp(-cg.get_x() / P.kT)
        free = P.mask > 0
        assert np.abs(n - no)[free].max() <= 1e-8 * no[free].max()
    finally:
        _close(cg, f, g, ctx)


@pytest.mark.parametrize("key", ["pcg_precision", "pcg_precision_tight"])
def test_precision_stop_rule_matches_reference(oracle_mod, golden, key):
    """The drivers' stop rule, Precision(eps, PreconditionedConjugateGradient(
    f, gd, kT, &x, QuadraticLineMinimizer)) (papers/contact/figs/walls.cpp:
    104-110, src/Precision.cpp:53-151): the GPU minimiser with
    deft_cg_params.precision = eps stops on the same improve_energy() call
    as the reference build, with the same energies along the way."""
    from tests.capi import CG
    from tests.golden.cases import precision_case
    vals, _ = golden
    rec = vals[key]
    P, x0, _, step, cap = precision_case()
    ctx, g, f = _setup(P)
    cg = CG(f, linesearch=_lib.LS_QUADRATIC_REF, step=step, preconditioned=1,
            precision=rec["precision"])
    try:
        cg.set_x(x0)
        e = []
        for _ in range(cap):
            s, st = cg.step()
            assert s == 0
            e.append(st.energy)
            if st.converged:
                break
        assert len(e) == rec["calls"]
        assert np.abs(np.array(e) / np.array(rec["energies"]) - 1).max() < 1e-10
    finally:
        _close(cg, f, g, ctx)
