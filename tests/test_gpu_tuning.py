"""Launch shapes and radix orders: every valid choice gives the same energy
and gradient up to rounding, invalid ones are refused, registered choices
reach new grids, and the autotuner returns a usable entry."""
import ctypes

import numpy as np
import pytest

from deft_gb300 import _lib

pytestmark = pytest.mark.gpu


def _setup(shape, precision):
    from tests.capi import Ctx, Fmt, Grid
    from deft_gb300.workloads import Slit
    s = Slit(N=shape[2], dx=0.2, eta=0.3, seed=3, Nxy=shape[0])
    ctx = Ctx(0)
    g = Grid(ctx, s.lat, s.shape)
    f = Fmt(g, R=s.R, kT=s.kT, mu=s.mu, terms=_lib.TERM_HS | _lib.TERM_IDEAL | _lib.TERM_MU |
            _lib.TERM_MASK, mask=s.mask.reshape(-1), precision=precision)
    return s, ctx, g, f


def _tiles(g, precision):
    t = np.zeros(6, dtype=np.int32)
    r = np.zeros(24, dtype=np.int32)
    _lib.check(g.L.deft_grid_get_tiles(g.h, precision, t.ctypes.data, r.ctypes.data))
    return t, r


def _set(g, precision, t, r):
    t = np.ascontiguousarray(t, dtype=np.int32)
    r = np.ascontiguousarray(r, dtype=np.int32)
    return g.L.deft_grid_set_tiles(g.h, precision, t.ctypes.data, r.ctypes.data)


@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (1, 2e-5)])
def test_choices_change_results_only_by_rounding(precision, tol):
    s, ctx, g, f = _setup((24, 24, 48), precision)
    try:
        E0, g0, _ = f.energy_grad(s.n0.reshape(-1))
        t, r = _tiles(g, precision)
        assert all(t > 0)
        rng = np.random.default_rng(5)
        orders_z = [[8, 3, 2], [2, 3, 8], [3, 4, 4], [4, 4, 3]]
        orders_x = [[8, 3], [3, 8], [2, 3, 4], [4, 3, 2]]
        for k in range(6):
            tt = rng.integers(1, 12, size=6)
            rr = np.zeros(24, dtype=np.int32)
            ox, oz = orders_x[k % 4], orders_z[k % 4]
            rr[:len(ox)] = ox
            rr[8:8 + len(ox)] = ox
            rr[16:16 + len(oz)] = oz
            assert _set(g, precision, tt, rr) == 0
            t2, r2 = _tiles(g, precision)
            assert list(t2) == list(tt)  # all below the clamps of this shape
            assert list(r2[16:16 + len(oz)]) == oz
            E, gr, _ = f.energy_grad(s.n0.reshape(-1))
            assert abs(E / E0 - 1) < tol
            assert np.abs(gr - g0).max() <= tol * np.abs(g0).max()
        # the FFT interface follows the FP64 choice and still inverts exactly
        x = s.n0.reshape(s.shape)
        back = g.ifft(g.fft(x))
        assert np.abs(back - x).max() <= 1e-14 * np.abs(x).max()
    finally:
        f.close()
        g.close()
        ctx.close()


def test_invalid_choices_are_refused():
    s, ctx, g, f = _setup((16, 16, 32), 0)
    try:
        t, r = _tiles(g, 0)
        bad = r.copy()
        bad[16:24] = 0
        bad[16:19] = [8, 8, 8]  # product 512, not 32
        assert _set(g, 0, t, bad) == _lib.ERR_ARG
        bad[16:19] = [6, 2, 0]  # 6 is not a supported radix
        assert _set(g, 0, t, bad) == _lib.ERR_ARG
        t2, r2 = _tiles(g, 0)
        assert np.array_equal(t2, t) and np.array_equal(r2, r)
    finally:
        f.close()
        g.close()
        ctx.close()


def test_registered_choice_reaches_new_grids():
    L = _lib.load()
    N = np.array([20, 20, 40], dtype=np.int32)
    t = np.array([3, 2, 5, 1, 4, 3], dtype=np.int32)
    r = np.zeros(24, dtype=np.int32)
    r[16:19] = [5, 2, 4]
    _lib.check(L.deft_tuning_set(N.ctypes.data, 1, t.ctypes.data, r.ctypes.data))
    try:
        s, ctx, g, f = _setup((20, 20, 40), 1)
        try:
            t2, r2 = _tiles(g, 1)
            assert list(t2) == list(t)
            assert list(r2[16:19]) == [5, 2, 4]
        finally:
            f.close()
            g.close()
            ctx.close()
    finally:
        _lib.check(L.deft_tuning_clear())


def test_autotuner_entry(tmp_path):
    from deft_gb300 import autotune
    e = autotune.tune((24, 24, 24), _lib.PRECISION_MIXED, repeats=1, trials=1)
    assert len(e["tiles"]) == 6 and all(v > 0 for v in e["tiles"])
    assert e["ms_per_workload_after"] <= 1.5 * e["ms_per_workload_before"]
    path = str(tmp_path / "tuning.json")
    autotune.save([e], path)
    L = _lib.load()
    try:
        assert autotune.load(path) == 1
        s, ctx, g, f = _setup((24, 24, 24), 1)
        try:
            t2, _ = _tiles(g, 1)
            assert list(t2) == e["tiles"]
        finally:
            f.close()
            g.close()
            ctx.close()
    finally:
        _lib.check(L.deft_tuning_clear())


@pytest.mark.parametrize("precision", [0, 1])
def test_graph_replay_is_bitwise_identical_to_direct_launches(precision):
    """Captured evaluation and Hessian-vector sequences replay to the same
    bits as kernel-by-kernel launches, including after parameter changes
    that require a new capture, and the minimiser reaches the same point."""
    import torch
    from tests.capi import CG
    s, ctx, g, f = _setup((24, 24, 32), precision)
    L = g.L
    try:
        n = torch.tensor(s.n0.reshape(-1), device="cuda:0")
        out = torch.empty_like(n)
        E = ctypes.c_double()

        def eg():
            _lib.check(L.deft_fmt_energy_grad(f.h, n.data_ptr(), 1, ctypes.addressof(E),
                                              out.data_ptr(), None))
            return E.value, out.cpu().numpy().copy()

        def run_all():
            res = [eg(), eg()]
            if precision == 1:
                dx = torch.tensor(0.01 * s.nb * s.mask.reshape(-1), device="cuda:0")
                _lib.check(L.deft_fmt_hessian_vector(f.h, n.data_ptr(), dx.data_ptr(), 1,
                                                     out.data_ptr()))
                res.append((0.0, out.cpu().numpy().copy()))
            p = _lib.FmtParams(s.R, s.kT, s.mu + 0.01, _lib.TERM_HS | _lib.TERM_IDEAL |
                               _lib.TERM_MU | _lib.TERM_MASK, precision)
            _lib.check(L.deft_fmt_set_params(f.h, ctypes.byref(p)))
            res.append(eg())
            p.mu = s.mu
            _lib.check(L.deft_fmt_set_params(f.h, ctypes.byref(p)))
            res.append(eg())
            cg = CG(f, gtol=1e-9, maxiter=3000, step=1.0)
            cg.set_x(s.n0.reshape(-1))
            code, st = cg.solve()
            assert code == 0 and st.converged
            res.append((st.energy, cg.get_x()))
            cg.close()
            return res

        _lib.check(L.deft_grid_graphs(g.h, 1))
        with_graphs = run_all()
        _lib.check(L.deft_grid_graphs(g.h, 0))
        direct = run_all()
        for (ea, a), (eb, b) in zip(with_graphs, direct):
            assert ea == eb and np.array_equal(a, b)
    finally:
        f.close()
        g.close()
        ctx.close()


def test_register_resident_transform_matches_shared_memory_passes():
    """The register-resident FFT (radix order [16, N/16], FP32 kernels only)
    gives the mixed evaluator's energy, gradient and Hessian-vector product
    to FP32 rounding; the FP64 kernels refuse it."""
    s, ctx, g, f = _setup((32, 32, 64), 1)
    try:
        n = s.n0.reshape(-1)
        E0, g0, _ = f.energy_grad(n)
        dx = 0.01 * s.nb * s.mask.reshape(-1)
        h0 = f.hessian_vector(n, dx)
        t, r = _tiles(g, 1)
        rr = np.zeros(24, dtype=np.int32)  # axes x, y, z
        rr[0:2] = [16, 2]
        rr[8:10] = [16, 2]
        rr[16:18] = [16, 4]
        for tt in ([4, 16, 8, 4, 8, 4], [32, 16, 32, 8, 32, 8]):
            assert _set(g, 1, tt, rr) == 0
            t2, r2 = _tiles(g, 1)
            assert list(r2[16:18]) == [16, 4] and r2[18] == 0
            E, gr, _ = f.energy_grad(n)
            h = f.hessian_vector(n, dx)
            assert abs(E / E0 - 1) < 2e-6
            assert np.abs(gr - g0).max() <= 2e-5 * np.abs(g0).max()
            assert np.abs(h - h0).max() <= 2e-5 * np.abs(h0).max()
        assert _set(g, 0, t, rr) == _lib.ERR_ARG
    finally:
        f.close()
        g.close()
        ctx.close()
