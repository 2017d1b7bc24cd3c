"""The Python mirror of the reference API (deft_gb300.api) driven the way the
reference's drivers drive deft, e.g. papers/contact/figs/walls.cpp:83-116:

    f = OfEffectivePotential(HardSpheresWBnotensor(1) + IdealGas())
    mu = find_chemical_potential(f, 1, eta/(4 pi/3))
    f = constrain(mask, OfEffectivePotential(HS + IdealGas() + ChemicalPotential(mu)))
    potential = -log((eta mask + 1e-4 eta) / (4 pi/3))
    min = Precision(eps, PreconditionedConjugateGradient(f, gd, 1, &potential,
                                                         QuadraticLineMinimizer))
    while min.improve_energy(): ...

with every improve_energy() checked against the restated reference
minimiser (oracle), whose trajectory is itself pinned to the reference's."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _walls(Nz=24, Nxy=6, dz=0.2):
    import deft_gb300 as d
    lat = d.Lattice([Nxy * dz, 0, 0], [0, Nxy * dz, 0], [0, 0, Nz * dz])
    gd = d.GridDescription(lat, Nxy, Nxy, Nz)
    z = np.arange(Nz) * dz
    mask = np.broadcast_to(((z > 0) & (z < Nz * dz / 2)).astype(float), (Nxy, Nxy, Nz)).copy()
    return d, lat, gd, mask


@pytest.mark.parametrize("preconditioned", [False, True])
def test_walls_driver_matches_restated_reference(oracle_mod, preconditioned):
    d, lat, gd, mask = _walls()
    O = oracle_mod
    eta = 0.3
    fhs = d.HardSpheresWBnotensor(1.0)
    mu = d.find_chemical_potential(d.OfEffectivePotential(fhs + d.IdealGas()), 1, eta / (4 * math.pi / 3))
    assert abs(mu - O.find_mu(1.0, 1.0, eta / (4 * math.pi / 3))) < 1e-12
    f = d.constrain(mask, d.OfEffectivePotential(fhs + d.IdealGas() + d.ChemicalPotential(mu)))
    potential = -np.log((eta * mask + 1e-4 * eta) / (4 * math.pi / 3))
    x0 = potential.copy()
    mk = d.PreconditionedConjugateGradient if preconditioned else d.ConjugateGradient
    m = d.Precision(1e-12, mk(f, gd, 1.0, potential, d.QuadraticLineMinimizer, 0.1))
    energies = []
    for _ in range(5):
        more = m.improve_energy(False)
        energies.append(m.energy())
        if not more:
            break
    P = O.Problem(lat.R, gd.shape, mu=mu, terms=O.HS | O.IDEAL | O.MU | O.VEFF,
                  mask=mask.reshape(-1))
    run = P.pcg_quadratic if preconditioned else P.cg_quadratic
    _, eo = run(x0.reshape(-1), len(energies), step=0.1)
    # the quadratic search branches on energy comparisons, so rounding-level
    # differences grow along the trajectory (the first step agrees to ~1e-13;
    # the reference-pinned trajectory check is in test_gpu_veff.py)
    assert abs(energies[0] / eo[0] - 1) < 1e-11
    assert np.abs(np.array(energies) / eo - 1).max() < 1e-4
    # the gradient / pgrad of the mirror equal the oracle's at the final point
    g = np.zeros(gd.NxNyNz)
    pg = np.zeros(gd.NxNyNz)
    E = f.integralgrad(1.0, gd, potential, g, pg)
    Eo, go, pgo = P.energy_grad_pgrad(potential.reshape(-1))
    assert abs(E / Eo - 1) < 1e-10
    assert np.abs(g - go).max() <= 1e-9 * np.abs(go).max()
    assert np.abs(pg - pgo).max() <= 1e-9 * np.abs(pgo).max()
    density = d.EffectivePotentialToDensity()(1.0, gd, potential)
    assert np.all(density > 0)
    m.close()
    f.close()
    gd.close()


def test_density_variable_driver_and_secant_solve(oracle_mod):
    """ConjugateGradient on n itself with the derivative line search to
    |grad| < 1e-9: the converged profile equals the oracle's."""
    d, lat, gd, mask = _walls()
    O = oracle_mod
    nb = 0.3 / (4 * math.pi / 3)
    mu = d.find_chemical_potential(d.HardSpheresWBnotensor(1.0) + d.IdealGas(), 1.0, nb)
    f = d.constrain(mask, d.HardSpheresWBnotensor(1.0) + d.IdealGas() + d.ChemicalPotential(mu))
    n = nb * mask
    m = d.ConjugateGradient(f, gd, 1.0, n, d.SecantLineMinimizer, 1.0)
    m.gtol = 1e-11
    m.maxiter = 5000
    st = m.solve()
    assert st.converged and st.gnorm < 1e-11
    P = O.Problem(lat.R, gd.shape, mu=mu, mask=mask.reshape(-1))
    xo, info = P.cg_solve(nb * mask.reshape(-1), gtol=1e-11, maxiter=5000)
    assert np.abs(n.reshape(-1) - xo).max() <= 1e-8 * xo.max()
    E, t = f.energy_terms(gd, 1.0, n)
    Eo, to = P.energy(xo, terms=True)
    assert abs(E / Eo - 1) < 1e-10
    m.close()
    f.close()
    gd.close()
