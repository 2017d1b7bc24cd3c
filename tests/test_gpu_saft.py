"""GPU water SAFT (DEFT_TERM_SAFT): the compiled reference WaterSaft's energy
and gradient (tests/golden/) and a converged slit solve against the
oracle's, in the FP64 form and in the mixed form (every transform in FP32,
refinement by FP64 CG).  Stated tolerances: energy 1e-10, gradient 1e-9
relative (FP64); energy 1e-6, gradient 1e-4 of its largest entry (mixed,
one evaluation); converged slit profile 1e-6 relative in both forms (the
tolerance the gradient norm pins it to)."""
import ctypes
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


def _saft_fmt(g, P, terms, precision=0):
    from tests.capi import Fmt
    from tests.golden.cases import WATER_SAFT
    f = Fmt(g, R=P.R, kT=P.kT, mu=P.mu, terms=terms | _lib.TERM_SAFT, mask=P.mask,
            precision=precision)
    sp = np.array(WATER_SAFT)
    _lib.check(f.L.deft_fmt_set_saft(f.h, sp.ctypes.data))
    return f


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name", ["saft_cubic12", "saft_ortho_mask"])
def test_saft_matches_reference_golden(ctx, oracle_mod, name, precision):
    from tests.capi import Grid
    from tests.golden.cases import saft_case
    with open(os.path.join(HERE, "golden", "reference_values.json")) as fh:
        vals = json.load(fh)
    arrs = np.load(os.path.join(HERE, "golden", "reference_fields.npz"))
    P, n = saft_case(name)
    g = Grid(ctx, P.lat.reshape(3, 3), P.N)
    f = _saft_fmt(g, P, P.terms, precision)
    E, grad, _ = f.energy_grad(n)
    e_tol, g_tol = (1e-10, 1e-9) if precision == 0 else (1e-6, 1e-4)
    gr = arrs[f"{name}_grad"]
    dE = abs(E / vals[name]["E"] - 1)
    dg = float(np.abs(grad - gr).max() / np.abs(gr).max())
    print(f"{name} precision {precision}: |dF/F| = {dE:.3e}, max|dg|/max|g| = {dg:.3e}")
    assert dE < e_tol
    assert dg <= g_tol
    E2, _ = f.energy(n)
    assert abs(E2 / E - 1) < (1e-13 if precision == 0 else 1e-6)
    f.close()
    g.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_saft_slit_solve_matches_oracle(ctx, oracle_mod, precision):
    """Liquid water against two hard walls (the wall density floored at
    1e-5 of the liquid's, as the drivers floor it): CG with the density
    preconditioner converges to the oracle's 1-D profile, in the FP64 form
    and in the mixed form (FP32 stage, then FP64 CG to the same gtol)."""
    from tests.capi import CG, Grid
    from tests.golden.cases import WATER_KT, WATER_N, WATER_R, WATER_SAFT
    O = oracle_mod
    Nz, dz, Nxy = 64, 0.5, 4
    z = np.arange(Nz) * dz
    mask1 = ((z > 0) & (z < 0.6 * Nz * dz)).astype(float)
    P1 = O.Problem(np.diag([dz, dz, Nz * dz]), (1, 1, Nz), R=WATER_R, kT=WATER_KT, mu=0.0,
                   terms=O.HS | O.IDEAL | O.MU, saft=WATER_SAFT)
    h = 1e-7 * WATER_N
    vol = dz * dz * Nz * dz
    mu = -(P1.energy(np.full(Nz, WATER_N + h)) - P1.energy(np.full(Nz, WATER_N - h))) / (2 * h * vol)
    P1 = O.Problem(np.diag([dz, dz, Nz * dz]), (1, 1, Nz), R=WATER_R, kT=WATER_KT, mu=mu,
                   terms=O.HS | O.IDEAL | O.MU, mask=mask1, saft=WATER_SAFT)
    x0 = np.where(mask1 > 0, WATER_N, 1e-5 * WATER_N)  # floored walls, as the drivers
    x1, info = P1.cg_solve(x0, gtol=1e-13, maxiter=20000, preconditioned=2)
    assert info["gnorm"] < 1e-13
    shape = (Nxy, Nxy, Nz)
    lat = np.diag([Nxy * dz, Nxy * dz, Nz * dz])
    mask = np.broadcast_to(mask1, shape).reshape(-1).copy()
    P = O.Problem(lat, shape, R=WATER_R, kT=WATER_KT, mu=mu, terms=O.HS | O.IDEAL | O.MU,
                  mask=mask, saft=WATER_SAFT)
    g = Grid(ctx, lat, shape)
    f = _saft_fmt(g, P, P.terms, precision)
    cg = CG(f, gtol=1e-12, maxiter=20000, step=1.0, preconditioned=_lib.PC_DENSITY)
    cg.set_x(np.broadcast_to(x0, shape).reshape(-1))
    code, st = cg.solve()
    assert code == 0 and st.converged, (code, st.gnorm, st.iter)
    n = cg.get_x().reshape(shape)
    # |grad| < 1e-12 (kT = 9.4e-4 Hartree, dV = 1/8 bohr^3) pins this profile
    # to ~1e-7: the oracle's own plain and preconditioned solves at 1e-13
    # differ by 5e-8
    assert np.abs(n - x1[None, None, :]).max() < 1e-6 * x1.max()
    cg.close()
    f.close()
    g.close()


def test_saft_needs_parameters_and_the_white_bear_functional(ctx):
    from tests.capi import Fmt, Grid
    g = Grid(ctx, np.diag([6.0] * 3), (12, 12, 12))
    f = Fmt(g, R=2.87, kT=1e-3, terms=_lib.TERM_HS | _lib.TERM_SAFT)
    n = np.full(12 ** 3, 4.9e-3)
    E = ctypes.c_double()
    assert f.L.deft_fmt_energy(f.h, n.ctypes.data, 0, ctypes.addressof(E), None) == _lib.ERR_ARG
    f.close()
    p = _lib.FmtParams(2.87, 1e-3, 0.0, _lib.TERM_HS | _lib.TERM_SAFT, _lib.PRECISION_MIXED,
                       _lib.HS_RF)
    h = ctypes.c_void_p()
    assert g.L.deft_fmt_create(g.h, ctypes.byref(p), ctypes.byref(h)) == _lib.ERR_ARG
    g.close()
