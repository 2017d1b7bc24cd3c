"""Generates the golden fixtures in this directory from the UNMODIFIED
reference sources (oracle/_ref/libdeft_ref.so, built by `make -C oracle ref`
where the reference checkout exists).  Run from the repository root:

    python tests/golden/make_golden.py

Inputs are regenerated from the seeds below by tests/golden/cases.py, so the
fixtures store only the reference's outputs (plus the small inputs of the CG
trajectory case, for convenience)."""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from tests.golden.cases import (CASES, HS_CASES, SAFT_CASES, WATER_SAFT, cg_case,  # noqa: E402
                                make_case, precision_case, saft_case, veff_case)


def main():
    O.build(ref=True)
    assert O.ref_available(), "reference build missing"
    out = {}
    arrays = {}
    for name in CASES:
        P, n = make_case(name)
        E, g, t = P.ref_energy_grad(n)
        w = P.ref_weighted(n)
        out[name] = {"E": E, "terms": [float(x) for x in t]}
        arrays[f"{name}_grad"] = g
        arrays[f"{name}_weighted"] = w
    # the Rosenfeld functional (HardSpheresRF), White Bear mark II (the
    # WhiteBear.hs definition through the reference's Functional algebra),
    # the tensor White Bear (HardSpheresWB) and Tarazona functionals
    for name, hs in HS_CASES:
        P, n = make_case(name, hs)
        E, g, t = P.ref_energy_grad(n)
        out[f"{name}_hs{hs}"] = {"E": E, "terms": [float(x) for x in t]}
        arrays[f"{name}_hs{hs}_grad"] = g
    # contact values (src/ContactDensity.cpp; gSigmaS as WhiteBear.hs defines
    # it) on the slit of the CG case, converged by the oracle's secant CG
    P, n, _, _ = cg_case()
    x, _ = P.cg_solve(n, gtol=1e-9, maxiter=3000)
    arrays["contact_slit_x"] = x
    for hs in (O.HS_WB, O.HS_M2):
        P.hs = hs
        for which in range(5):
            arrays[f"contact_slit_hs{hs}_{which}"] = P.ref_contact(x, which)
    # the water SAFT functional (WaterSaft, src/WaterSaftFast.cpp): total
    # energy and (masked) gradient
    for name in SAFT_CASES:
        P, n = saft_case(name)
        E, g = P.ref_saft(n, WATER_SAFT)
        out[name] = {"E": E}
        arrays[f"{name}_grad"] = g
    # the "new" API minimiser (src/new/Minimize.cpp) on the random cubic case
    # (8 calls) and on the CG case's slit (to its own stopping rule)
    P, n = make_case("cubic12")
    x, e = P.ref_new_minimize(n, 8)
    out["new_minimize_cubic12"] = {"energies": [float(v) for v in e]}
    P, n, _, _ = cg_case()
    x, e = P.ref_new_minimize(n, 60)
    out["new_minimize_slit"] = {"energies": [float(v) for v in e]}
    arrays["new_minimize_slit_x"] = x
    # known-answer value of tests/new-hard-spheres.cpp:52-63
    P = O.Problem(np.diag([2.0, 2.0, 2.0]), (20, 20, 20), R=1.0, kT=1.0, mu=0.0, terms=O.HS)
    E, _, _ = P.ref_energy_grad(np.full(8000, 0.1), grad=False)
    out["white_bear_kat"] = {"E": E, "published": 2.72225468848892}
    # bulk chemical potentials
    out["find_mu"] = {str(eta): O.ref().ref_find_mu(1.0, 1.0, eta / (4 * np.pi / 3))
                      for eta in (0.05, 0.1, 0.2, 0.3, 0.4, 0.45)}
    # reference CG + QuadraticLineMinimizer trajectory
    P, n, iters, step = cg_case()
    x, e = P.ref_cg(n, iters, step=step)
    out["cg_quadratic"] = {"energies": [float(v) for v in e], "iters": iters, "step": step}
    arrays["cg_quadratic_x"] = x
    # OfEffectivePotential: energy, gradient, preconditioned gradient, and a
    # PreconditionedConjugateGradient + QuadraticLineMinimizer trajectory
    P, xv, iters, step = veff_case()
    E, g, pg = P.ref_eval_veff(xv)
    out["veff"] = {"E": E}
    arrays["veff_grad"] = g
    arrays["veff_pgrad"] = pg
    x, e = P.ref_pcg(xv, iters, step=step)
    out["pcg_quadratic"] = {"energies": [float(v) for v in e], "iters": iters, "step": step}
    arrays["pcg_quadratic_x"] = x
    # the drivers' Precision stop rule around PreconditionedConjugateGradient
    P, x0, prec, step, cap = precision_case()
    x, e = P.ref_pcg_precision(x0, cap, step, prec)
    out["pcg_precision"] = {"energies": [float(v) for v in e], "calls": len(e),
                            "precision": prec, "step": step}
    # and with the precision 1e4 times tighter (more calls of the rule)
    x, e = P.ref_pcg_precision(x0, cap, step, prec * 1e-4)
    out["pcg_precision_tight"] = {"energies": [float(v) for v in e], "calls": len(e),
                                  "precision": prec * 1e-4, "step": step}
    with open(os.path.join(HERE, "reference_values.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    np.savez_compressed(os.path.join(HERE, "reference_fields.npz"), **arrays)
    print("wrote", sorted(out), sorted(arrays))


if __name__ == "__main__":
    main()
