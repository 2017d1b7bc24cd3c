"""CPU tests of the oracle: the plain-C restatement against the golden
fixtures generated from the unmodified reference (tests/golden/), the
reference's own known-answer value, the weight identities of
tests/convolve.cpp, and (where the reference build exists) live parity with
the reference."""
import json
import math
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def golden():
    with open(os.path.join(HERE, "golden", "reference_values.json")) as f:
        vals = json.load(f)
    arrs = np.load(os.path.join(HERE, "golden", "reference_fields.npz"))
    return vals, arrs


@pytest.mark.parametrize("shape", [(10, 10, 10), (16, 12, 15), (7, 9, 11), (12, 14, 13), (8, 6, 4)])
def test_oracle_fft_matches_numpy(oracle_mod, shape):
    O = oracle_mod
    rng = np.random.default_rng(1)
    x = rng.standard_normal(shape)
    a = O.r2c_3d(x)
    b = np.fft.rfftn(x)
    assert np.abs(a - b).max() <= 2e-15 * np.abs(b).max() * math.log2(x.size)
    back = O.c2r_3d(b, shape[2])
    ref = np.fft.irfftn(b, s=shape, axes=(0, 1, 2)) * x.size
    assert np.abs(back - ref).max() <= 2e-15 * np.abs(x).max() * x.size * math.log2(x.size)


def test_oracle_fft_round_trip_fcc(oracle_mod):
    """tests/fftinverse.cpp:30-50: fft then ifft recovers the field to 1e-15."""
    O = oracle_mod
    rng = np.random.default_rng(2)
    x = rng.standard_normal((10, 10, 10))
    back = O.c2r_3d(O.r2c_3d(x), 10) / x.size
    assert np.abs(back - x).max() < 1e-15 * 10


@pytest.mark.parametrize("name", ["cubic12", "ortho_odd", "fcc12"])
def test_oracle_matches_reference_golden(oracle_mod, golden, name):
    from tests.golden.cases import make_case
    vals, arrs = golden
    P, n = make_case(name)
    E, g, t = P.energy_grad(n, terms=True)
    ref = vals[name]
    assert abs(E / ref["E"] - 1) < 1e-12
    tr = np.array(ref["terms"])
    assert np.abs(t[:len(tr)] - tr).max() <= 1e-12 * np.abs(tr).max()
    gr = arrs[f"{name}_grad"]
    assert np.abs(g - gr).max() <= 1e-12 * np.abs(gr).max()
    w = P.weighted(n)
    wr = arrs[f"{name}_weighted"]
    for a in range(5):
        assert np.abs(w[a] - wr[a]).max() <= 1e-13 * np.abs(wr[a]).max()


@pytest.mark.parametrize("name,hs", [("cubic12", 1), ("ortho_odd", 1), ("cubic12", 2),
                                     ("ortho_odd", 2), ("cubic12", 3), ("ortho_odd", 3),
                                     ("fcc12", 3), ("cubic12", 4), ("fcc12", 4)])
def test_oracle_rosenfeld_mark2_tensor_match_reference_golden(oracle_mod, golden, name, hs):
    """HardSpheresRF, HardSpheresWB (tensor) and HardSpheresTarazona as
    compiled, and White Bear mark II as WhiteBear.hs defines it, evaluated
    by the reference's Functional machinery."""
    from tests.golden.cases import make_case
    vals, arrs = golden
    P, n = make_case(name, hs)
    E, g, t = P.energy_grad(n, terms=True)
    ref = vals[f"{name}_hs{hs}"]
    assert abs(E / ref["E"] - 1) < 1e-12
    tr = np.array(ref["terms"])
    assert np.abs(t[:len(tr)] - tr).max() <= 1e-12 * np.abs(tr).max()
    gr = arrs[f"{name}_hs{hs}_grad"]
    assert np.abs(g - gr).max() <= 1e-12 * np.abs(gr).max()


@pytest.mark.parametrize("hs", [0, 1, 2, 3, 4])
def test_oracle_bulk_equations_of_state(oracle_mod, hs):
    """Uniform density: White Bear (vector or tensor) and mark II give the
    Carnahan-Starling excess free energy eta (4 - 3 eta) / (1 - eta)^2 per
    particle, Rosenfeld and Tarazona the Percus-Yevick (compressibility) one
    -ln(1-eta) + 3 eta (2 - eta) / (2 (1-eta)^2)."""
    O = oracle_mod
    for eta in (0.05, 0.2, 0.4):
        nu = eta / (4 * math.pi / 3)
        P = O.Problem(np.diag([3.2] * 3), (16, 16, 16), terms=O.HS, hs=hs)
        E = P.energy(np.full(16 ** 3, nu))
        if hs in (O.HS_RF, O.HS_TZ):
            fex = -math.log(1 - eta) + 3 * eta * (2 - eta) / (2 * (1 - eta) ** 2)
        else:
            fex = eta * (4 - 3 * eta) / (1 - eta) ** 2
        assert abs(E / (3.2 ** 3 * nu * fex) - 1) < 1e-12


def test_oracle_mark2_small_packing_series(oracle_mod):
    """Near n3 = 0 the mark II prefactors switch to their Taylor series: the
    energy and gradient stay continuous across the switch (|n3| = 0.1)."""
    O = oracle_mod
    vals = []
    for eta in (0.1 - 1e-9, 0.1 + 1e-9):
        nu = eta / (4 * math.pi / 3)
        P = O.Problem(np.diag([3.2] * 3), (16, 16, 16), terms=O.HS, hs=O.HS_M2)
        E, g = P.energy_grad(np.full(16 ** 3, nu))
        vals.append((E / nu, g.mean() / nu))
    assert abs(vals[0][0] / vals[1][0] - 1) < 1e-7 and abs(vals[0][1] / vals[1][1] - 1) < 1e-7


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(HERE), "oracle", "_ref",
                                                    "libdeft_ref.so")),
                    reason="reference build only exists where the reference checkout does")
def test_mark2_vs_compiled_wbm2slow(oracle_mod):
    """The compiled HardSpheresWBm2slow has the mark II Phi1 and Phi2 but
    1/(36 pi) where WhiteBear.hs has 1/(24 pi) in Phi3: its Phi3 term is 2/3
    of the oracle's."""
    from tests.golden.cases import make_case
    P, n = make_case("cubic12", 2)
    P.terms = oracle_mod.HS
    _, t = P.energy(n, terms=True)
    P.hs = 5  # the reference bindings' HardSpheresWBm2slow
    _, _, tr = P.ref_energy_grad(n, grad=False)
    assert abs(tr[0] / t[0] - 2 / 3) < 1e-12
    assert abs(tr[1] / t[1] - 1) < 1e-12 and abs(tr[2] / t[2] - 1) < 1e-12


def test_oracle_white_bear_known_answer(oracle_mod, golden):
    O = oracle_mod
    vals, _ = golden
    P = O.Problem(np.diag([2.0, 2.0, 2.0]), (20, 20, 20), R=1.0, kT=1.0, mu=0.0, terms=O.HS)
    E = P.energy(np.full(8000, 0.1))
    assert abs(E / 2.72225468848892 - 1) < 2e-11  # tests/new-hard-spheres.cpp:56,66
    assert abs(E / vals["white_bear_kat"]["E"] - 1) < 1e-13
    # homogeneous value F/a^3 (tests/new-hard-spheres.cpp:73-77)
    hom = _hs_only_homogeneous(O, 0.1)
    assert abs(hom / (2.72225468848892 / 8) - 1) < 2e-11


def _hs_only_homogeneous(O, nb):
    # HS free-energy density only: total minus ideal gas (mu = 0)
    x = 18.01528 * 1822.8885 * 1.0 / (2 * math.pi)
    nQ = x * math.sqrt(x)
    return O.homogeneous(1.0, 1.0, 0.0, nb) - nb * (math.log(nb / nQ) - 1)


def test_oracle_find_mu(oracle_mod, golden):
    vals, _ = golden
    for eta, mu in vals["find_mu"].items():
        nb = float(eta) / (4 * math.pi / 3)
        assert abs(oracle_mod.find_mu(1.0, 1.0, nb) / mu - 1) < 1e-13


def test_oracle_cg_quadratic_trajectory(oracle_mod, golden):
    from tests.golden.cases import cg_case
    vals, arrs = golden
    P, n, iters, step = cg_case()
    x, e = P.cg_quadratic(n, iters, step=step)
    er = np.array(vals["cg_quadratic"]["energies"])
    assert len(e) == len(er)
    assert np.abs(e / er - 1).max() < 1e-11
    assert np.abs(x - arrs["cg_quadratic_x"]).max() < 1e-5 * np.abs(x).max()


def test_oracle_weight_identities(oracle_mod):
    """tests/convolve.cpp:79-177 on an FCC cell with a sharp Gaussian:
    integral of Step(R) * f = 4/3 pi R^3 integral f, Shell = 4 pi R^2, vector
    shells integrate to 0, |x-shell| <= shell."""
    O = oracle_mod
    lat = np.array([[0, 5, 5], [5, 0, 5], [5, 5, 0.0]])
    N = (40, 40, 40)
    R = np.array(lat).T
    ii = np.arange(40) / 40.0
    rel = np.stack(np.meshgrid(ii, ii, ii, indexing="ij"), -1).reshape(-1, 3)
    rel = rel - np.round(rel)
    cart = rel @ R.T
    f = np.exp(-10.0 * (cart * cart).sum(1))
    P = O.Problem(lat, N, R=1.0)
    dV = P.dvolume()
    w = P.weighted(f)
    I = f.sum() * dV
    assert abs(w[0].sum() * dV / I - 4 * math.pi / 3) < 1e-6 * 4 * math.pi / 3
    assert abs(w[1].sum() * dV / I - 4 * math.pi) < 1e-6 * 4 * math.pi
    for c in (2, 3, 4):
        assert abs(w[c].sum() * dV / I) < 1e-10
        assert np.abs(w[c]).max() <= w[1].max() * (1 + 1e-12)


def test_oracle_secant_cg_1d_slit(oracle_mod):
    O = oracle_mod
    nb = 0.3 / (4 * math.pi / 3)
    mu = O.find_mu(1.0, 1.0, nb)
    z = np.arange(64) * 0.2
    mask = ((z > 0) & (z < 6.4)).astype(float)
    P = O.Problem(np.diag([0.2, 0.2, 12.8]), (1, 1, 64), mu=mu, mask=mask)
    x, info = P.cg_solve(np.where(mask > 0, nb, 0.0), gtol=1e-12, maxiter=5000)
    assert info["gnorm"] < 1e-12
    # symmetric slit: the profile is mirror-symmetric about the slit centre
    inner = x[1:32]
    assert np.abs(inner - inner[::-1]).max() < 1e-10
    # far from the walls the density approaches bulk; at contact it is enhanced
    assert x[1] > 2 * nb


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(HERE), "oracle", "_ref",
                                                    "libdeft_ref.so")),
                    reason="reference build only exists where the reference checkout does")
def test_oracle_matches_live_reference(oracle_mod):
    O = oracle_mod
    rng = np.random.default_rng(9)
    N = (14, 10, 9)
    lat = np.array([[2.8, 0.1, 0.0], [0.0, 2.0, -0.1], [0.2, 0.0, 1.8]])
    size = int(np.prod(N))
    nb = 0.2 / (4 * math.pi / 3)
    P = O.Problem(lat, N, R=0.9, kT=1.3, mu=O.find_mu(0.9, 1.3, nb),
                  V=0.1 * rng.standard_normal(size), mask=(rng.random(size) > 0.1).astype(float))
    n = nb * (1 + 0.1 * rng.standard_normal(size))
    E, g = P.energy_grad(n)
    Er, gr, _ = P.ref_energy_grad(n)
    assert abs(E / Er - 1) < 1e-13
    assert np.abs(g - gr).max() <= 1e-13 * np.abs(gr).max()


def test_oracle_effective_potential_matches_reference_golden(oracle_mod, golden):
    """constrain(mask, OfEffectivePotential(HS + ideal + mu)): energy,
    gradient and preconditioned gradient (src/EffectivePotentialToDensity.cpp:
    28-91) against the reference's values."""
    from tests.golden.cases import veff_case
    vals, arrs = golden
    P, x, _, _ = veff_case()
    E, g, pg = P.energy_grad_pgrad(x)
    assert abs(E / vals["veff"]["E"] - 1) < 1e-12
    assert np.abs(g - arrs["veff_grad"]).max() <= 1e-12 * np.abs(arrs["veff_grad"]).max()
    assert np.abs(pg - arrs["veff_pgrad"]).max() <= 1e-12 * np.abs(arrs["veff_pgrad"]).max()
    # the energy is that of the density exp(-x/kT)
    P2 = oracle_mod.Problem(P.lat.reshape(3, 3), P.N, R=P.R, kT=P.kT, mu=P.mu, mask=P.mask)
    assert abs(P2.energy(np.exp(-x / P.kT)) / E - 1) < 1e-14


def test_oracle_effective_potential_gradient_finite_difference(oracle_mod):
    """Central differences of the energy along a random direction, the
    check of Functional::run_finite_difference_test (src/Functional.cpp:159-210)."""
    from tests.golden.cases import veff_case
    P, x, _, _ = veff_case()
    _, g, _ = P.energy_grad_pgrad(x)
    rng = np.random.default_rng(4)
    d = rng.standard_normal(x.size) * P.mask
    for h in (1e-4, 1e-5):
        fd = (P.energy(x + h * d) - P.energy(x - h * d)) / (2 * h)
        assert abs(fd - g @ d) <= 1e-7 * abs(g @ d)


def test_oracle_pcg_quadratic_trajectory(oracle_mod, golden):
    """PreconditionedConjugateGradient + QuadraticLineMinimizer in the
    effective-potential variable: the reference's energies step by step."""
    from tests.golden.cases import veff_case
    vals, arrs = golden
    P, x0, iters, step = veff_case()
    x, e = P.pcg_quadratic(x0, iters, step=step)
    er = np.array(vals["pcg_quadratic"]["energies"])
    assert len(e) == len(er)
    assert np.abs(e / er - 1).max() < 1e-11
    assert np.abs(x - arrs["pcg_quadratic_x"]).max() < 1e-5 * np.abs(x).max()


def test_oracle_preconditioned_secant_cg_converges(oracle_mod):
    from tests.golden.cases import veff_case
    P, x0, _, _ = veff_case()
    # |dF/dVeff| = |n dF/dn| / kT: a tighter tolerance than the density
    # variable needs for the same profile accuracy
    x1, i1 = P.cg_solve(x0, gtol=1e-11, maxiter=3000, preconditioned=True)
    x2, i2 = P.cg_solve(x0, gtol=1e-11, maxiter=3000, preconditioned=False)
    assert i1["gnorm"] < 1e-11 and i2["gnorm"] < 1e-11
    n1, n2 = np.exp(-x1 / P.kT), np.exp(-x2 / P.kT)
    free = P.mask > 0
    assert np.abs(n1 - n2)[free].max() <= 1e-8 * n1[free].max()


def test_oracle_density_preconditioner_same_profile_fewer_evaluations(oracle_mod):
    """Polak-Ribiere with the diagonal M^-1 = n / (kT dV) (the inverse
    ideal-gas curvature) reaches the same slit profile as the plain secant CG
    with fewer evaluations."""
    O = oracle_mod
    nb = 0.3 / (4 * math.pi / 3)
    mu = O.find_mu(1.0, 1.0, nb)
    z = np.arange(64) * 0.2
    mask = ((z > 0) & (z < 6.4)).astype(float)
    P = O.Problem(np.diag([0.2, 0.2, 12.8]), (1, 1, 64), mu=mu, mask=mask)
    x0 = np.where(mask > 0, nb, 0.0)
    x1, i1 = P.cg_solve(x0, gtol=1e-12, maxiter=5000, preconditioned=2)
    x2, i2 = P.cg_solve(x0, gtol=1e-12, maxiter=5000, preconditioned=0)
    assert i1["gnorm"] < 1e-12 and i2["gnorm"] < 1e-12
    assert np.abs(x1 - x2).max() <= 1e-9 * x2.max()
    assert i1["evals"] < i2["evals"]


@pytest.mark.parametrize("hs", [0, 2])
@pytest.mark.parametrize("which", [0, 1, 2, 3, 4])
def test_oracle_contact_values_match_reference_golden(oracle_mod, golden, hs, which):
    """gSigmaS (WhiteBear.hs, through the reference's partial derivatives),
    gSigmaA (gSigmaAcpp / gSigmaAm2cpp), GrossCorrelation, YuWuCorrelation
    and YuWuCorrelation_S on a converged slit profile."""
    from tests.golden.cases import cg_case
    _, arrs = golden
    P, _, _, _ = cg_case()
    P.hs = hs
    x = arrs["contact_slit_x"]
    got = P.contact(x, which)
    ref = arrs[f"contact_slit_hs{hs}_{which}"]
    assert np.all(np.isfinite(ref))
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("name", ["saft_cubic12", "saft_ortho_mask"])
def test_oracle_water_saft_matches_reference_golden(oracle_mod, golden, name):
    """Water SAFT (ideal gas + White Bear + association + dispersion + mu N,
    constrained by the mask when given): energy and gradient against the
    compiled WaterSaft (src/WaterSaftFast.cpp)."""
    from tests.golden.cases import saft_case
    vals, arrs = golden
    P, n = saft_case(name)
    E, g = P.energy_grad(n)
    assert abs(E / vals[name]["E"] - 1) < 1e-12
    gr = arrs[f"{name}_grad"]
    assert np.abs(g - gr).max() <= 1e-12 * np.abs(gr).max()


def test_oracle_water_saft_gradient_is_the_energy_derivative(oracle_mod):
    """Directional finite difference of the SAFT association + dispersion
    energy against the chain-rule gradient (central, two step sizes)."""
    from tests.golden.cases import WATER_SAFT, saft_case
    P, n = saft_case("saft_cubic12")
    _, g, _ = P.saft(n, WATER_SAFT)
    rng = np.random.default_rng(3)
    d = rng.standard_normal(n.size) * n * 0.01
    gd = g @ d
    for h in (1e-3, 5e-4):
        Ep, _, _ = P.saft(n + h * d, WATER_SAFT, grad=False)
        Em, _, _ = P.saft(n - h * d, WATER_SAFT, grad=False)
        assert abs((Ep - Em) / (2 * h) / gd - 1) < 1e-6


def test_oracle_new_api_minimize_matches_reference(oracle_mod, golden):
    """The "new" API's Minimize (src/new/Minimize.cpp) restated: on the
    random cubic case the energies after each improve_energy call match the
    reference's to 1e-12; on the slit its energy-difference line search is
    sensitive to the last bits of the energies (its first step starts from
    0.001 |E0| / slope), so the first call may differ at 1e-7 while the
    trajectory re-converges: the end point's energy agrees to 1e-12 and its
    profile to 1e-6."""
    from tests.golden.cases import cg_case, make_case
    vals, arrs = golden
    P, n = make_case("cubic12")
    _, e = P.new_minimize(n, 8)
    er = np.array(vals["new_minimize_cubic12"]["energies"])
    assert len(e) == len(er) and np.abs(e / er - 1).max() < 1e-12
    P, n, _, _ = cg_case()
    x, e = P.new_minimize(n, 60)
    er = np.array(vals["new_minimize_slit"]["energies"])
    assert abs(e[-1] / er[-1] - 1) < 1e-12
    m = min(len(e), len(er))
    assert np.abs(e[:m] / er[:m] - 1).max() < 1e-7
    xr = arrs["new_minimize_slit_x"]
    assert np.abs(x - xr).max() <= 1e-6 * xr.max()


def precision_rule_stop(E0, energies, precision):
    """Restatement of PrecisionMinimizer::improve_energy (src/Precision.cpp:
    39-151) over a sequence of energies: the 1-based index of the
    improve_energy() call that returns false (the inner minimiser assumed
    not done), or None if the rule never stops."""
    w, deltaE, log_avg = 0.1, 0.0, 0.0
    dEdn = 0.0
    old = E0
    for k, new in enumerate(energies, start=1):
        old_deltaE = deltaE
        deltaE = old - new
        dEdn = max(deltaE, old_deltaE)
        nl = math.log(abs(deltaE / old_deltaE)) if (deltaE and old_deltaE) else 0.0
        log_avg = (1 - w) * log_avg + w * nl
        ratio = math.exp(log_avg)
        guess = abs(max(dEdn, deltaE) / log_avg) if log_avg else math.inf
        if ratio >= 1:
            guess = precision + abs(new)
        err = 2 * guess
        if deltaE == 0 and old_deltaE == 0:
            return k
        if not err < precision:
            old = new
            continue
        return k
    return None


@pytest.mark.parametrize("key", ["pcg_precision", "pcg_precision_tight"])
def test_precision_rule_restatement_stops_where_the_reference_stops(oracle_mod, key):
    """The drivers' Precision(eps, PreconditionedConjugateGradient(...)) stop
    (papers/contact/figs/walls.cpp:104-110): the restated rule applied to the
    reference's own energy sequence stops on the same call as the reference
    build (tests/golden/reference_values.json)."""
    from tests.golden.cases import precision_case
    vals = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                                       "reference_values.json")))
    rec = vals[key]
    P, x0, _, _, _ = precision_case()
    E0, _, _ = P.energy_grad_pgrad(x0)
    assert precision_rule_stop(E0, rec["energies"], rec["precision"]) == rec["calls"]
