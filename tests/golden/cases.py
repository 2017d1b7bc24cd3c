"""Seeded inputs of the golden cases (shared by make_golden.py and the tests)."""
import math

import numpy as np

from oracle import oracle as O

CASES = ("cubic12", "ortho_odd", "fcc12")
# (case, hard-sphere functional) pairs of the Rosenfeld, mark II, tensor
# White Bear and Tarazona fixtures
HS_CASES = (("cubic12", O.HS_RF), ("ortho_odd", O.HS_RF), ("cubic12", O.HS_M2),
            ("ortho_odd", O.HS_M2), ("cubic12", O.HS_WBT), ("ortho_odd", O.HS_WBT),
            ("fcc12", O.HS_WBT), ("cubic12", O.HS_TZ), ("fcc12", O.HS_TZ))


def make_case(name, hs=O.HS_WB):
    P, n = _make_case(name)
    P.hs = hs
    return P, n


def _make_case(name):
    if name == "cubic12":
        rng = np.random.Generator(np.random.PCG64(101))
        N, lat, R, kT = (12, 12, 12), np.diag([2.4, 2.4, 2.4]), 1.0, 1.0
        nb = 0.3 / (4 * math.pi / 3)
        mu = O.find_mu(R, kT, nb)
        n = nb * (1 + 0.2 * rng.standard_normal(int(np.prod(N))))
        return O.Problem(lat, N, R=R, kT=kT, mu=mu, terms=O.HS | O.IDEAL | O.MU), n
    if name == "ortho_odd":
        rng = np.random.Generator(np.random.PCG64(102))
        N, lat, R, kT = (10, 12, 15), np.diag([2.0, 2.6, 3.0]), 1.0, 1.0
        size = int(np.prod(N))
        nb = 0.25 / (4 * math.pi / 3)
        mu = O.find_mu(R, kT, nb)
        mask = (rng.random(size) > 0.3).astype(np.float64)
        V = 0.3 * rng.standard_normal(size)
        n = nb * (1 + 0.1 * rng.standard_normal(size))
        n = np.where(mask > 0, n, 1e-4 * nb)  # floor density in walls, as the drivers do
        return O.Problem(lat, N, R=R, kT=kT, mu=mu, terms=O.HS | O.IDEAL | O.MU, V=V, mask=mask), n
    if name == "fcc12":
        rng = np.random.Generator(np.random.PCG64(103))
        N = (12, 12, 12)
        lat = np.array([[0, 2.5, 2.5], [2.5, 0, 2.5], [2.5, 2.5, 0.0]])
        R, kT = 0.7, 0.8
        size = int(np.prod(N))
        mask = (rng.random(size) > 0.2).astype(np.float64)
        V = 0.1 * rng.standard_normal(size)
        n = 0.05 * (1 + 0.3 * rng.random(size))
        return O.Problem(lat, N, R=R, kT=kT, mu=-1.2, terms=O.HS | O.IDEAL | O.MU, V=V,
                         mask=mask), n
    raise KeyError(name)


def cg_case():
    N, lat = (12, 12, 16), np.diag([2.4, 2.4, 3.2])
    nb = 0.3 / (4 * math.pi / 3)
    mu = O.find_mu(1.0, 1.0, nb)
    z = np.arange(16) * 0.2
    mask = np.broadcast_to(((z > 0) & (z < 1.6)).astype(float), N).copy().reshape(-1)
    rng = np.random.Generator(np.random.PCG64(104))
    n = nb * (1 + 0.05 * rng.standard_normal(mask.size))
    n = np.where(mask > 0, n, 1e-4 * nb)
    P = O.Problem(lat, N, mu=mu, mask=mask)
    return P, n, 6, 0.1


def precision_case():
    """The stop rule of the paper drivers on the cg_case slit
    (papers/contact/figs/walls.cpp:86-110): effective-potential variable
    started at -kT ln((eta mask + 1e-4 eta) / (4 pi / 3)), precision =
    |F_bulk(nb) x slit volume| x 1e-4, PreconditionedConjugateGradient with
    QuadraticLineMinimizer at the default step 10.  Returns (problem, x0,
    precision, step, iteration cap)."""
    P, _, _, _ = cg_case()
    P.terms |= O.VEFF
    eta = 0.3
    mask = P.mask
    x0 = -P.kT * np.log((eta * mask + 1e-4 * eta) / (4 * math.pi / 3))
    nb = eta / (4 * math.pi / 3)
    dV = P.dvolume()
    approx = O.lib().oracle_homogeneous(P.R, P.kT, P.mu, nb) * float(mask.sum()) * dV
    return P, x0, abs(approx * 1e-4), 10.0, 100


def veff_case():
    """The cg_case slit in the effective-potential variable, as
    papers/contact/figs/walls.cpp:86-101 sets it up: x = -kT ln n with the wall
    density floored at 1e-4 nb, constrain(mask, OfEffectivePotential(...))."""
    P, n, iters, step = cg_case()
    P.terms |= O.VEFF
    return P, -P.kT * np.log(n), iters, step


# Water SAFT (src/water-constants.cpp:22-40, hughes_water_prop) in atomic units
KB_HARTREE = 3.16681539628059e-6
ANGSTROM = 1.8897261
WATER_R = 3.03420 * ANGSTROM / 2
WATER_KT = 298.15 * KB_HARTREE
WATER_N = 4.9388942e-3
# (epsilon_association, kappa_association, epsilon_dispersion, lambda_dispersion, length_scaling)
WATER_SAFT = (1400.0 * KB_HARTREE, 0.0381876 * (3.03420 * ANGSTROM) ** 3, 250.0 * KB_HARTREE,
              1.78890, 0.353)
SAFT_CASES = ("saft_cubic12", "saft_ortho_mask")


def saft_case(name):
    if name == "saft_cubic12":
        rng = np.random.Generator(np.random.PCG64(201))
        N, lat = (12, 12, 12), np.diag([6.0, 6.0, 6.0])
        n = np.abs(WATER_N * (1 + 0.1 * rng.standard_normal(int(np.prod(N)))))
        return O.Problem(lat, N, R=WATER_R, kT=WATER_KT, mu=-0.01, terms=O.HS | O.IDEAL | O.MU,
                         saft=WATER_SAFT), n
    if name == "saft_ortho_mask":
        rng = np.random.Generator(np.random.PCG64(202))
        N, lat = (10, 14, 9), np.diag([5.8, 8.2, 5.3])
        size = int(np.prod(N))
        n = np.abs(WATER_N * (1 + 0.3 * rng.standard_normal(size)))
        mask = (rng.random(size) > 0.2).astype(np.float64)
        return O.Problem(lat, N, R=WATER_R, kT=WATER_KT, mu=0.02, terms=O.HS | O.IDEAL | O.MU,
                         mask=mask, saft=WATER_SAFT), n
    raise KeyError(name)
