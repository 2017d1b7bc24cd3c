"""The "new" API's minimiser (DEFT_LS_NEW_API, src/new/Minimize.cpp) on the
GPU against the reference's own trajectories (tests/golden/): energies
after each improve_energy call on the random cubic case to 1e-10; on the
slit the end point's energy to 1e-10 and profile to 1e-6 (its
energy-difference line search is sensitive to the last bits of the
energies on that case)."""
import json
import os

import numpy as np
import pytest

from deft_gb300 import _lib

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def ctx():
    from tests.capi import Ctx
    c = Ctx(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def golden():
    with open(os.path.join(HERE, "golden", "reference_values.json")) as f:
        vals = json.load(f)
    return vals, np.load(os.path.join(HERE, "golden", "reference_fields.npz"))


def _run(ctx, P, n, calls):
    from tests.capi import CG, Fmt, Grid
    g = Grid(ctx, P.lat.reshape(3, 3), P.N)
    f = Fmt(g, R=P.R, kT=P.kT, mu=P.mu, terms=P.terms, V=P.V, mask=P.mask)
    cg = CG(f, linesearch=_lib.LS_NEW_API, gtol=0.0, maxiter=0)
    cg.set_x(n)
    energies = []
    for _ in range(calls):
        code, st = cg.step()
        assert code == 0
        energies.append(st.energy)
        if st.converged:
            break
    x = cg.get_x()
    cg.close()
    f.close()
    g.close()
    return x, np.array(energies)


def test_new_api_cubic_trajectory(ctx, oracle_mod, golden):
    from tests.golden.cases import make_case
    vals, _ = golden
    P, n = make_case("cubic12")
    _, e = _run(ctx, P, n, 8)
    er = np.array(vals["new_minimize_cubic12"]["energies"])
    assert len(e) == len(er) and np.abs(e / er - 1).max() < 1e-10


def test_new_api_slit_end_point(ctx, oracle_mod, golden):
    from tests.golden.cases import cg_case
    vals, arrs = golden
    P, n, _, _ = cg_case()
    x, e = _run(ctx, P, n, 60)
    er = np.array(vals["new_minimize_slit"]["energies"])
    assert abs(e[-1] / er[-1] - 1) < 1e-10
    xr = arrs["new_minimize_slit_x"]
    assert np.abs(x - xr).max() <= 1e-6 * xr.max()
