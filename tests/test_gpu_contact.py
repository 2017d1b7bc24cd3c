"""GPU contact values (deft_fmt_contact) against the reference's outputs on
a converged slit profile (tests/golden/) and against the oracle on an
orthorhombic odd-sized random case.  Stated tolerance: 1e-10 relative to the
field's maximum (FP64 post-processing)."""
import ctypes
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


def _contact(f, n, which, on_device=False):
    out = np.empty(n.size)
    n = np.ascontiguousarray(n, dtype=np.float64)
    _lib.check(f.L.deft_fmt_contact(f.h, n.ctypes.data, 0, which, out.ctypes.data))
    return out


@pytest.mark.parametrize("hs", [0, 2])
@pytest.mark.parametrize("which", [0, 1, 2, 3, 4])
def test_contact_values_match_reference_golden(ctx, oracle_mod, hs, which):
    from tests.capi import Fmt, Grid
    from tests.golden.cases import cg_case
    arrs = np.load(os.path.join(HERE, "golden", "reference_fields.npz"))
    P, _, _, _ = cg_case()
    x = arrs["contact_slit_x"]
    g = Grid(ctx, P.lat.reshape(3, 3), P.N)
    f = Fmt(g, R=P.R, kT=P.kT, mu=P.mu, terms=_lib.TERM_HS | _lib.TERM_IDEAL | _lib.TERM_MU,
            functional=hs)
    got = _contact(f, x, which)
    ref = arrs[f"contact_slit_hs{hs}_{which}"]
    assert np.abs(got - ref).max() <= 1e-10 * np.abs(ref).max()
    f.close()
    g.close()


@pytest.mark.parametrize("which", [0, 1, 2, 3, 4])
def test_contact_values_vs_oracle_odd_grid(ctx, oracle_mod, which):
    from tests.capi import Fmt, Grid
    O = oracle_mod
    rng = np.random.default_rng(21)
    N = (10, 14, 9)
    lat = np.array([[2.2, 0.1, 0.0], [0.0, 2.8, 0.0], [0.1, 0.0, 2.0]])
    nb = 0.25 / (4 * np.pi / 3)
    n = nb * (1 + 0.2 * rng.standard_normal(int(np.prod(N))))
    P = O.Problem(lat, N, R=0.9, hs=O.HS_M2)
    ref = P.contact(n, which)
    g = Grid(ctx, lat, N)
    f = Fmt(g, R=0.9, functional=_lib.HS_WB_MARK2)
    got = _contact(f, n, which)
    assert np.abs(got - ref).max() <= 1e-10 * np.abs(ref).max()
    # device pointers give the same field
    import torch
    nd = torch.tensor(n, device="cuda:0")
    od = torch.empty_like(nd)
    _lib.check(f.L.deft_fmt_contact(f.h, nd.data_ptr(), 1, which, od.data_ptr()))
    torch.cuda.synchronize()
    assert np.array_equal(od.cpu().numpy(), got)
    f.close()
    g.close()


def test_unknown_contact_field_is_refused(ctx):
    from tests.capi import Fmt, Grid
    g = Grid(ctx, np.diag([2.4, 2.4, 2.4]), (12, 12, 12))
    f = Fmt(g)
    n = np.full(12 ** 3, 0.05)
    out = np.empty_like(n)
    assert f.L.deft_fmt_contact(f.h, n.ctypes.data, 0, 9, out.ctypes.data) == _lib.ERR_ARG
    f.close()
    g.close()
