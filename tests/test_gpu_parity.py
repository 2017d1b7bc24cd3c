"""GPU parity: the sm_103a path through the C ABI against the oracle
restatement (oracle/deft_oracle.c) on the same seeded inputs.

Tolerances (FP64 form): free energy 1e-10 relative, gradient 1e-9 relative
to its max, FFT 1e-14 relative, weighted densities 1e-13 relative."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

E_TOL = 1e-10
G_TOL = 1e-9


@pytest.fixture(scope="module")
def ctx():
    from tests.capi import Ctx
    c = Ctx(0)
    yield c
    c.close()


def _grid(ctx, lat, N):
    from tests.capi import Grid
    return Grid(ctx, lat, N)


CASES = [
    # name, lattice rows, N
    ("cubic16", np.diag([3.2, 3.2, 3.2]), (16, 16, 16)),
    ("ortho_odd", np.diag([2.4, 2.8, 3.0]), (12, 14, 15)),
    ("fcc12", np.array([[0, 2.5, 2.5], [2.5, 0, 2.5], [2.5, 2.5, 0.0]]), (12, 12, 12)),
    ("mixed48", np.diag([9.6, 9.6, 9.6]), (48, 20, 10)),
    ("prime7", np.diag([1.4, 2.2, 2.6]), (7, 11, 13)),
]


@pytest.mark.parametrize("name,lat,N", CASES)
def test_fft_matches_numpy(ctx, name, lat, N):
    g = _grid(ctx, lat, N)
    dV, vol, _ = g.info()
    rng = np.random.default_rng(7)
    x = rng.standard_normal(N)
    c = g.fft(x)
    ref = np.fft.rfftn(x) * dV
    assert np.abs(c - ref).max() <= 1e-14 * np.abs(ref).max() * math.log2(x.size)
    back = g.ifft(c)
    assert np.abs(back * vol / dV / x.size - x).max() <= 1e-14 * math.log2(x.size)
    g.close()


@pytest.mark.parametrize("name,lat,N", CASES)
def test_weighted_densities(ctx, oracle_mod, name, lat, N):
    from tests.capi import Fmt
    O = oracle_mod
    g = _grid(ctx, lat, N)
    rng = np.random.default_rng(3)
    n = 0.05 * (1 + 0.3 * rng.standard_normal(N))
    f = Fmt(g, R=0.9, kT=1.0)
    w = f.weighted(n)
    wr = O.Problem(lat, N, R=0.9).weighted(n)
    for a in range(5):
        scale = np.abs(wr[a]).max()
        assert np.abs(w[a] - wr[a]).max() <= 1e-13 * scale, a
    f.close()
    g.close()


def _problem(O, lat, N, seed, with_V=False, with_mask=False, zero_walls=False):
    rng = np.random.default_rng(seed)
    size = int(np.prod(N))
    nb = 0.3 / (4 * math.pi / 3)
    mu = O.find_mu(1.0, 1.0, nb)
    n = nb * (1 + 0.2 * rng.standard_normal(size))
    V = 0.2 * rng.standard_normal(size) if with_V else None
    mask = (rng.random(size) > 0.25).astype(np.float64) if with_mask else None
    if zero_walls:
        n = np.where(mask > 0, n, 0.0)
    P = O.Problem(lat, N, R=1.0, kT=1.0, mu=mu, terms=O.HS | O.IDEAL | O.MU, V=V, mask=mask)
    return P, n


@pytest.mark.parametrize("name,lat,N", CASES)
@pytest.mark.parametrize("variant", ["plain", "V_mask", "zero_walls"])
def test_energy_grad_matches_oracle(ctx, oracle_mod, name, lat, N, variant):
    from tests.capi import Fmt
    O = oracle_mod
    P, n = _problem(O, lat, N, seed=11, with_V=variant != "plain",
                    with_mask=variant != "plain", zero_walls=variant == "zero_walls")
    g = _grid(ctx, lat, N)
    f = Fmt(g, R=P.R, kT=P.kT, mu=P.mu, terms=P.terms, V=P.V, mask=P.mask)
    E, grad, terms = f.energy_grad(n)
    Er, gr, tr = P.energy_grad(n, terms=True)
    assert abs(E / Er - 1) < E_TOL
    assert np.abs(terms - tr).max() <= E_TOL * np.abs(tr).max()
    assert np.abs(grad - gr).max() <= G_TOL * np.abs(gr).max()
    E2, t2 = f.energy(n)
    assert E2 == E  # energy-only and energy+gradient share the arithmetic
    f.close()
    g.close()


def test_white_bear_known_answer(ctx):
    """tests/new-hard-spheres.cpp:52-63: n = 0.1, R = 1, kT = 1, 20^3, a = 2."""
    from tests.capi import Fmt
    g = _grid(ctx, np.diag([2.0, 2.0, 2.0]), (20, 20, 20))
    f = Fmt(g, R=1.0, kT=1.0, mu=0.0, terms=1)
    E, _ = f.energy(np.full(8000, 0.1))
    assert abs(E / 2.72225468848892 - 1) < 2e-11
    f.close()
    g.close()


def test_find_chemical_potential(oracle_mod):
    import ctypes
    from deft_gb300 import _lib
    for eta in (0.05, 0.3, 0.45):
        nb = eta / (4 * math.pi / 3)
        mu = ctypes.c_double()
        _lib.check(_lib.load().deft_find_chemical_potential(1.0, 1.0, nb, ctypes.addressof(mu)))
        assert abs(mu.value / oracle_mod.find_mu(1.0, 1.0, nb) - 1) < 1e-13


def test_finite_difference_gradient(ctx, oracle_mod):
    """Directional derivative of the GPU energy vs the GPU gradient, with the
    pass rule of Functional::run_finite_difference_test
    (src/Functional.cpp:197-210)."""
    from tests.capi import Fmt
    O = oracle_mod
    lat = np.array([[0, 2.5, 2.5], [2.5, 0, 2.5], [2.5, 2.5, 0.0]])
    N = (16, 16, 16)
    P, n = _problem(O, lat, N, seed=5)
    g = _grid(ctx, lat, N)
    f = Fmt(g, R=P.R, kT=P.kT, mu=P.mu, terms=P.terms)
    E0, grad, _ = f.energy_grad(n)
    # Direction n * grad (normalised): a step stays inside n > 0 up to
    # eps = min(n / |d|), which is large, so the schedule can start where the
    # central difference's O(eps^2) error dominates rounding and the
    # convergence-rate rule has something to measure.
    d = n * grad
    d /= np.linalg.norm(d)
    lderiv = d @ grad
    eps_max = 1e-15 * abs(E0) / abs(lderiv) / 1e-15
    min_p = int(-math.floor(math.log10(eps_max) + 0.5))
    min_p = max(min_p, int(math.ceil(-math.log10(0.5 * np.min(n / np.abs(d))))))
    grads, best, mn = [], 1.0, 1e300
    for p in range(min_p, min_p + 8):
        eps = 10.0 ** (-p)
        Ep, _ = f.energy(n + eps * d)
        Em, _ = f.energy(n - eps * d)
        grads.append((Ep - Em) / (2 * eps))
        best = min(best, abs(grads[-1] / lderiv - 1))
        if len(grads) > 1 and grads[-1] != grads[-2]:
            diff = (grads[-2] - lderiv) * (-1 + 1 / 100.0) / (grads[-1] - grads[-2])
            mn = min(mn, abs(diff - 1))
    # the reference's first pass branch: reasonable scaling and accuracy
    assert mn < 1e-3 and best < 1e-7, (mn, best)
    f.close()
    g.close()


def test_cg_quadratic_matches_reference_cg(ctx, oracle_mod):
    """ConjugateGradient + QuadraticLineMinimizer: the GPU trajectory against
    the restated reference algorithm, energy after each improve_energy()."""
    from tests.capi import CG, Fmt
    from deft_gb300 import _lib
    O = oracle_mod
    N = (12, 12, 16)
    lat = np.diag([2.4, 2.4, 3.2])
    nb = 0.3 / (4 * math.pi / 3)
    mu = O.find_mu(1.0, 1.0, nb)
    z = np.arange(16) * 0.2
    mask = np.broadcast_to(((z > 0) & (z < 1.6)).astype(float), N).copy().reshape(-1)
    rng = np.random.default_rng(1)
    n = nb * (1 + 0.05 * rng.standard_normal(mask.size))
    n = np.where(mask > 0, n, 1e-4 * nb)
    P = O.Problem(lat, N, mu=mu, mask=mask)
    _, e_ref = P.cg_quadratic(n, 6, step=0.1)
    g = _grid(ctx, lat, N)
    f = Fmt(g, R=1.0, kT=1.0, mu=mu, terms=P.terms, mask=mask)
    cg = CG(f, linesearch=_lib.LS_QUADRATIC_REF, step=0.1)
    cg.set_x(n)
    e_gpu = []
    for _ in range(len(e_ref)):
        s, st = cg.step()
        assert s == 0
        e_gpu.append(st.energy)
    assert np.abs(np.array(e_gpu) / e_ref - 1).max() < 1e-10
    cg.close()
    f.close()
    g.close()


def test_cg_secant_converged_slit_matches_1d_oracle(ctx, oracle_mod):
    """3-D slit with noise converges (|grad| < 1e-9) to the z-only profile the
    oracle finds on a 1x1xN grid with the same cell volume."""
    from tests.capi import CG, Fmt
    from deft_gb300.workloads import Slit
    O = oracle_mod
    s = Slit(N=32, dx=0.2, eta=0.3, Nxy=8, seed=1)
    g = _grid(ctx, s.lat, s.shape)
    f = Fmt(g, R=1.0, kT=1.0, mu=s.mu, terms=O.HS | O.IDEAL | O.MU | O.MASK,
            mask=s.mask.reshape(-1))
    cg = CG(f, gtol=1e-11, maxiter=5000, step=1.0)
    cg.set_x(s.n0.reshape(-1))
    st_code, st = cg.solve()
    assert st_code == 0 and st.converged and st.gnorm < 1e-9
    n = cg.get_x().reshape(s.shape)
    P1 = O.Problem(np.diag([s.dx, s.dx, s.L]), (1, 1, s.shape[2]), mu=s.mu,
                   terms=O.HS | O.IDEAL | O.MU, mask=s.mask[0, 0].copy())
    x1, info = P1.cg_solve(np.where(s.mask[0, 0] > 0, s.nb, 0.0), gtol=1e-13, maxiter=20000)
    assert info["gnorm"] < 1e-12
    assert np.abs(n - x1[None, None, :]).max() < 1e-8
    cg.close()
    f.close()
    g.close()


@pytest.mark.parametrize("N", [64, 128])
def test_full_size_energy_grad(ctx, oracle_mod, N):
    """The slit workloads at full size (64^3 and the 128^3 bench grid)."""
    from tests.capi import Fmt
    from deft_gb300.workloads import Slit
    O = oracle_mod
    s = Slit(N=N, dx=0.2, eta=0.3, seed=1)
    P = O.Problem(s.lat, s.shape, mu=s.mu, terms=O.HS | O.IDEAL | O.MU, mask=s.mask.reshape(-1))
    g = _grid(ctx, s.lat, s.shape)
    f = Fmt(g, R=1.0, kT=1.0, mu=s.mu, terms=P.terms, mask=s.mask.reshape(-1))
    n = s.n0.reshape(-1)
    E, grad, _ = f.energy_grad(n)
    Er, gr = P.energy_grad(n)
    assert abs(E / Er - 1) < E_TOL
    assert np.abs(grad - gr).max() <= G_TOL * np.abs(gr).max()
    f.close()
    g.close()


def test_config1_slit_64_solve_matches_oracle(ctx, oracle_mod):
    """The 64^3 hard-wall slit at its stated size (dx = 0.2, walls at z = 0
    and z = 6.4, eta = 0.3, smoothed-noise start, seed 1): plain FP64 CG to
    |grad F| < 1e-9.  The converged profile is within 1e-8 of the oracle's
    1-D solution (1 x 1 x 64 grid, same cell volume, converged to 1e-13) and
    the free energy within 1e-10 of 64 x 64 times the 1-D energy.  (F and the
    gradient at the start are compared in test_full_size_energy_grad.)"""
    from tests.capi import CG, Fmt
    from deft_gb300.workloads import Slit
    O = oracle_mod
    s = Slit(N=64, dx=0.2, eta=0.3, seed=1)
    assert abs(s.width - 6.4) < 1e-12
    g = _grid(ctx, s.lat, s.shape)
    f = Fmt(g, R=1.0, kT=1.0, mu=s.mu, terms=O.HS | O.IDEAL | O.MU | O.MASK,
            mask=s.mask.reshape(-1))
    cg = CG(f, gtol=1e-9, maxiter=5000, step=1.0)
    cg.set_x(s.n0.reshape(-1))
    code, st = cg.solve()
    assert code == 0 and st.converged and st.gnorm < 1e-9
    n = cg.get_x().reshape(s.shape)
    E, _ = f.energy(n.reshape(-1))
    P1 = O.Problem(np.diag([s.dx, s.dx, s.L]), (1, 1, s.shape[2]), mu=s.mu,
                   terms=O.HS | O.IDEAL | O.MU, mask=s.mask[0, 0].copy())
    x1, info = P1.cg_solve(np.where(s.mask[0, 0] > 0, s.nb, 0.0), gtol=1e-13, maxiter=20000)
    assert info["gnorm"] < 1e-12
    assert np.abs(n - x1[None, None, :]).max() < 1e-8
    assert abs(E / (P1.energy(x1) * s.shape[0] * s.shape[1]) - 1) < E_TOL
    cg.close()
    f.close()
    g.close()
