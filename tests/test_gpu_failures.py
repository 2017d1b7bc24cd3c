"""Failure paths and checkpoint / resume, with every failure made on the host:
a NaN planted in the input density, a tolerance below rounding (the line
search then runs out of resolution), an iteration limit; none of them hangs,
each returns its status.  A CG run checkpointed to disk and restored into a
fresh minimiser continues bit-identically."""
import ctypes
import os

import numpy as np
import pytest

from deft_gb300 import _lib

pytestmark = pytest.mark.gpu


def _problem(precision=0, N=24):
    from tests.capi import Ctx, Fmt, Grid
    from deft_gb300.workloads import Slit
    s = Slit(N=N, dx=0.2, eta=0.3, seed=4, Nxy=12)
    ctx = Ctx(0)
    g = Grid(ctx, s.lat, s.shape)
    f = Fmt(g, R=s.R, kT=s.kT, mu=s.mu, terms=_lib.TERM_HS | _lib.TERM_IDEAL | _lib.TERM_MU |
            _lib.TERM_MASK, mask=s.mask.reshape(-1), precision=precision)
    return s, ctx, g, f


def _close(*objs):
    for o in objs:
        o.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_nan_in_the_input_gives_an_error_status(precision):
    from tests.capi import CG
    s, ctx, g, f = _problem(precision)
    try:
        n = s.n0.reshape(-1).copy()
        n[np.flatnonzero(s.mask.reshape(-1))[5]] = np.nan
        E = ctypes.c_double()
        out = np.empty_like(n)
        code = f.L.deft_fmt_energy_grad(f.h, n.ctypes.data, 0, ctypes.addressof(E),
                                        out.ctypes.data, None)
        assert code == _lib.ERR_NAN
        cg = CG(f, gtol=1e-9, maxiter=100)
        try:
            cg.set_x(n)
            code, st = cg.solve()
            assert code == _lib.ERR_NAN and not st.converged
        finally:
            cg.close()
        # the context stays usable: a clean evaluation right after succeeds
        E2, _, _ = f.energy_grad(s.n0.reshape(-1))
        assert np.isfinite(E2)
    finally:
        _close(f, g, ctx)


def test_tolerance_below_rounding_ends_with_a_line_search_status():
    """|grad F| < 1e-30 cannot be reached in FP64: the secant search runs out
    of resolution, the minimiser retries along steepest descent, then stops
    with DEFT_ERR_LINESEARCH at a point that is converged to rounding."""
    from tests.capi import CG
    s, ctx, g, f = _problem(0)
    try:
        cg = CG(f, gtol=1e-30, maxiter=3000, step=1.0)
        try:
            cg.set_x(s.n0.reshape(-1))
            code, st = cg.solve()
            assert code == _lib.ERR_LINESEARCH and not st.converged
            assert st.iter < 3000 and st.gnorm < 1e-9
            assert b"line search" in f.L.deft_last_error()
        finally:
            cg.close()
    finally:
        _close(f, g, ctx)


def test_iteration_limit_status():
    from tests.capi import CG
    s, ctx, g, f = _problem(0)
    try:
        cg = CG(f, gtol=1e-9, maxiter=3, step=1.0)
        try:
            cg.set_x(s.n0.reshape(-1))
            code, st = cg.solve()
            assert code == _lib.ERR_MAXITER and st.iter == 3 and not st.converged
        finally:
            cg.close()
    finally:
        _close(f, g, ctx)


@pytest.mark.parametrize("precision,linesearch,preconditioned", [
    (0, _lib.LS_SECANT, 0), (1, _lib.LS_SECANT, 0), (0, _lib.LS_QUADRATIC_REF, 1)])
def test_checkpoint_resume_is_bit_identical(tmp_path, precision, linesearch, preconditioned):
    from tests.capi import CG
    s, ctx, g, f = _problem(precision)
    path = os.path.join(tmp_path, "cg.bin").encode()
    kw = dict(linesearch=linesearch, gtol=1e-12, maxiter=0, step=1.0 if linesearch == 0 else 0.1,
              preconditioned=preconditioned)
    try:
        a = CG(f, **kw)
        a.set_x(s.n0.reshape(-1))
        for _ in range(6):
            code, _ = a.step()
            assert code == 0
        _lib.check(f.L.deft_cg_checkpoint(a.h, path))
        for _ in range(6):
            code, st_a = a.step()
            assert code == 0
        xa = a.get_x()
        it_a = st_a.iter
        a.close()
        b = CG(f, **kw)
        _lib.check(f.L.deft_cg_restore(b.h, path))
        for _ in range(6):
            code, st_b = b.step()
            assert code == 0
        xb = b.get_x()
        b.close()
        assert it_a == st_b.iter and st_a.energy == st_b.energy
        assert np.array_equal(xa, xb)
        # a minimiser on another grid refuses the checkpoint
        from tests.capi import Fmt, Grid
        g2 = Grid(ctx, np.diag([2.4, 2.4, 4.8]), (12, 12, 20))
        f2 = Fmt(g2, R=1.0, kT=1.0, mu=s.mu, terms=_lib.TERM_HS | _lib.TERM_IDEAL |
                 _lib.TERM_MU)
        c2 = CG(f2, **kw)
        assert f.L.deft_cg_restore(c2.h, path) == _lib.ERR_ARG
        _close(c2, f2, g2)
    finally:
        _close(f, g, ctx)


@pytest.mark.parametrize("precision,linesearch", [(0, _lib.LS_SECANT), (1, _lib.LS_SECANT),
                                                  (0, _lib.LS_QUADRATIC_REF)])
def test_per_iteration_log(tmp_path, precision, linesearch):
    """deft_cg_set_log: one JSON line per deft_cg_step with the step's
    iteration, energy, gradient norm and counters as deft_cg_status reports
    them, and the energies of the terms of the last evaluation; NULL stops
    the log, a path that cannot be opened is an argument error."""
    import json
    from tests.capi import CG
    s, ctx, g, f = _problem(precision)
    path = os.path.join(tmp_path, "cg.jsonl")
    try:
        cg = CG(f, linesearch=linesearch, gtol=1e-9, maxiter=400,
                step=1.0 if linesearch == _lib.LS_SECANT else 0.1)
        cg.set_x(s.n0.reshape(-1))
        _lib.check(f.L.deft_cg_set_log(cg.h, path.encode()))
        seen = []
        for _ in range(400):
            code, st = cg.step()
            assert code == 0
            seen.append((st.iter, st.energy, st.gnorm, st.evals, st.converged))
            if st.converged:
                break
        _lib.check(f.L.deft_cg_set_log(cg.h, None))
        cg.step()  # not logged
        recs = [json.loads(line) for line in open(path)]
        assert len(recs) == len(seen)
        for r, (it, E, gn, ev, conv) in zip(recs, seen):
            assert (r["iter"], r["evals"], r["converged"]) == (it, ev, conv)
            assert r["energy"] == E and r["gnorm"] == gn
            assert set(r["terms"]) == {"hs_phi3", "hs_phi1", "hs_phi2", "ideal_gas",
                                       "chemical_potential", "external_potential"}
            assert all(np.isfinite(v) for v in r["terms"].values())
        assert recs[-1]["converged"] == 1
        # the terms of the last evaluation add up to an energy near the final one
        assert abs(sum(recs[-1]["terms"].values()) / recs[-1]["energy"] - 1) < 1e-6
        assert f.L.deft_cg_set_log(cg.h, str(tmp_path).encode()) == _lib.ERR_ARG
        cg.close()
    finally:
        _close(f, g, ctx)
