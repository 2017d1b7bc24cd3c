"""Learned warm start on the GPU: the Fourier-operator forward and backward
kernels against the CPU FP64 restatement (torch CPU autograd), training,
weight files, the checked warm start's fallback, and the gain over the bulk
start on held-out problems."""
import ctypes
import os

import numpy as np
import pytest

from deft_gb300 import _lib

from . import fno_reference as ref

pytestmark = pytest.mark.gpu


def _net(N, C, m, L, seed=7):
    from deft_gb300.warmstart import FourierOperator
    return FourierOperator(N=N, channels=C, modes=m, layers=L, seed=seed)


def _sample(N, seed):
    rng = np.random.default_rng(seed)
    x = np.arange(N)
    mask = np.ones((N, N, N), dtype=np.float32)
    mask[:, :, : N // 5] = 0  # a wall
    c = N // 2
    r2 = ((x[:, None, None] - c) ** 2 + (x[None, :, None] - c) ** 2 + (x[None, None, :] - c) ** 2)
    mask[r2 < (N // 6) ** 2] = 0  # a solute
    target = (1 + 0.3 * np.cos(2 * np.pi * x / N)[None, None, :]
              + 0.1 * rng.standard_normal((N, N, N))).astype(np.float32) * mask
    return mask.reshape(-1), target.reshape(-1)


@pytest.mark.parametrize("N,C,m,L", [(12, 4, 3, 2), (16, 16, 4, 4), (20, 8, 5, 3)])
def test_forward_and_gradient_match_fp64_restatement(N, C, m, L):
    net = _net(N, C, m, L)
    try:
        rng = np.random.default_rng(N + C)
        p = net.get_params()
        # move away from the initial point so every parameter matters
        p = (p + 0.05 * rng.standard_normal(p.size)).astype(np.float32)
        net.set_params(p)
        mask, target = _sample(N, seed=N)
        eta = 0.27
        y, loss, grad = net.eval(mask, eta, target, want_grad=True)
        loss_r, y_r, grad_r = ref.loss_and_grad(p, mask, eta, target, N, C, m, L)
        # FP32 accumulation against FP64: relative to the field / gradient scale
        assert np.max(np.abs(y - y_r)) <= 2e-5 * max(1.0, np.max(np.abs(y_r)))
        assert abs(loss - loss_r) <= 1e-4 * loss_r
        scale = np.max(np.abs(grad_r))
        err = np.abs(grad - grad_r)
        assert np.max(err) <= 2e-4 * scale, (np.max(err), scale)
        # per parameter block, the gradient's direction
        off, _ = ref.layout(C, L, m)
        for name, (o, k) in off.items():
            a, b = grad[o:o + k].astype(np.float64), grad_r[o:o + k]
            nb = np.linalg.norm(b)
            if nb > 1e-6 * scale:
                assert np.linalg.norm(a - b) <= 1e-3 * nb, name
    finally:
        net.close()


@pytest.mark.parametrize("N,C,m,L", [(12, 4, 3, 2), (16, 16, 4, 4), (20, 8, 5, 3),
                                     (32, 16, 12, 4)])
def test_inference_layers_match_training_forward(N, C, m, L):
    """Inference (no gradient asked) fuses the z synthesis into the pointwise
    layer; its output equals the training forward's (separate synthesis,
    stored z) and the FP64 restatement's to FP32 accumulation error."""
    net = _net(N, C, m, L)
    try:
        rng = np.random.default_rng(N + 7 * C)
        p = (net.get_params() + 0.05 * rng.standard_normal(net.nparam)).astype(np.float32)
        net.set_params(p)
        mask, target = _sample(N, seed=N + 1)
        eta = 0.31
        y_inf, loss_inf, _ = net.eval(mask, eta, target, want_grad=False)
        y_tr, loss_tr, _ = net.eval(mask, eta, target, want_grad=True)
        _, y_r, _ = ref.loss_and_grad(p, mask, eta, target, N, C, m, L)
        scale = max(1.0, float(np.max(np.abs(y_r))))
        assert np.max(np.abs(y_inf - y_tr)) <= 1e-5 * scale
        assert np.max(np.abs(y_inf - y_r)) <= 2e-5 * scale
        assert abs(loss_inf - loss_tr) <= 1e-5 * loss_tr
    finally:
        net.close()


def test_eval_is_deterministic_and_device_inputs_agree():
    import torch
    N, C, m, L = 16, 8, 4, 2
    net = _net(N, C, m, L)
    try:
        mask, target = _sample(N, seed=3)
        y1, l1, g1 = net.eval(mask, 0.3, target, want_grad=True)
        y2, l2, g2 = net.eval(mask, 0.3, target, want_grad=True)
        assert np.array_equal(y1, y2) and l1 == l2 and np.array_equal(g1, g2)
        md = torch.tensor(mask, device="cuda:0")
        td = torch.tensor(target, device="cuda:0")
        assert net.loss_device(md.data_ptr(), 0.3, td.data_ptr()) == l1
    finally:
        net.close()


def test_training_reduces_loss_and_weights_round_trip(tmp_path):
    import torch
    from deft_gb300.warmstart import FourierOperator
    N, C, m, L = 16, 8, 4, 2
    net = _net(N, C, m, L, seed=1)
    try:
        samples = [_sample(N, seed=s) for s in range(4)]
        dev = [(torch.tensor(a, device="cuda:0"), torch.tensor(b, device="cuda:0"))
               for a, b in samples]
        first = [net.loss_device(a.data_ptr(), 0.3, b.data_ptr()) for a, b in dev]
        for it in range(200):
            a, b = dev[it % 4]
            net.train_step(a.data_ptr(), 0.3, b.data_ptr(), 3e-3)
        last = [net.loss_device(a.data_ptr(), 0.3, b.data_ptr()) for a, b in dev]
        assert np.mean(last) < 0.5 * np.mean(first), (first, last)
        path16 = os.path.join(tmp_path, "w16.bin")
        net.save(path16, dtype="bfloat16")
        net16 = FourierOperator.load(path16)
        try:
            # the BF16 file holds exactly the values every pass uses
            y_a, _, _ = net.eval(samples[1][0], 0.3)
            y_b, _, _ = net16.eval(samples[1][0], 0.3)
            assert np.array_equal(y_a, y_b)
        finally:
            net16.close()
        path = os.path.join(tmp_path, "w.bin")
        net.save(path)
        net2 = FourierOperator.load(path)
        try:
            assert np.array_equal(net2.get_params(), net.get_params())
            y1, _, _ = net.eval(samples[0][0], 0.3)
            y2, _, _ = net2.eval(samples[0][0], 0.3)
            assert np.array_equal(y1, y2)
        finally:
            net2.close()
    finally:
        net.close()


def _fmt_for(s, precision=0):
    from .capi import Ctx, Fmt, Grid
    ctx = Ctx(0)
    g = Grid(ctx, s.lat, s.shape)
    terms = _lib.TERM_HS | _lib.TERM_IDEAL | _lib.TERM_MU | _lib.TERM_MASK
    f = Fmt(g, R=s.R, kT=s.kT, mu=s.mu, terms=terms, mask=s.mask.reshape(-1), precision=precision)
    return ctx, g, f


def test_warm_start_falls_back_to_bulk():
    import torch
    from deft_gb300.workloads import WallsSolutes
    N = 16
    s = WallsSolutes(N=N, dx=0.2, eta=0.3, width=3.0, solutes=[(1.6, 1.6, 1.5, 0.6)])
    ctx, g, f = _fmt_for(s)
    net = _net(N, 4, 3, 2)
    try:
        mask = torch.tensor(s.mask.reshape(-1), device="cuda:0")
        out = torch.empty_like(mask)
        bulk = (s.nb * s.mask).reshape(-1)
        # y = 1 exactly (all weights zero, q2 = 1): the bulk density, accepted
        p = np.zeros(net.nparam, dtype=np.float32)
        p[-1] = 1.0
        net.set_params(p)
        used, E = net.initial_density(f.h, mask.data_ptr(), s.eta, s.nb, out.data_ptr())
        assert used and np.allclose(out.cpu().numpy(), bulk, rtol=0, atol=1e-18)
        # a non-finite network output falls back to the bulk start
        p[-1] = np.nan
        net.set_params(p)
        used, E2 = net.initial_density(f.h, mask.data_ptr(), s.eta, s.nb, out.data_ptr())
        assert not used and np.array_equal(out.cpu().numpy(), bulk) and np.isfinite(E2)
        # an output that raises the energy (three times the bulk density,
        # packing fraction 0.9) falls back too
        p[-1] = 3.0
        net.set_params(p)
        used, E3 = net.initial_density(f.h, mask.data_ptr(), s.eta, s.nb, out.data_ptr())
        assert not used and np.array_equal(out.cpu().numpy(), bulk)
        # a grid that does not match the network's is refused
        net2 = _net(12, 4, 3, 2)
        try:
            code = net2.L.deft_fno_initial_density(net2.h, f.h, mask.data_ptr(), 0.3, s.nb, 1e-3,
                                                   out.data_ptr(), None, None, None)
            assert code == _lib.ERR_ARG
        finally:
            net2.close()
    finally:
        net.close()
        f.close()
        g.close()
        ctx.close()


def _solve_from(f, n0_dev, precision, refine_abs=0.0):
    from .capi import CG
    cg = CG(f, linesearch=_lib.LS_SECANT, gtol=1e-9, maxiter=20000, step=1.0,
            refine_abs=refine_abs)
    try:
        _lib.check(cg.L.deft_cg_set_x(cg.h, n0_dev.data_ptr(), 1))
        st = _lib.CgStatus()
        _lib.check(cg.L.deft_cg_solve(cg.h, ctypes.byref(st)))
        return st.iter, st.evals, st.gnorm, st.converged, cg.get_x()
    finally:
        cg.close()


def test_trained_warm_start_beats_bulk_start_on_held_out_problems():
    """Train a small network on converged solutions of seeded wall + solute
    problems at 40^3, then solve held-out seeds to |grad F| < 1e-9 from the
    network's start and from the bulk start: both converge to the same
    profile, and the warm start takes fewer CG iterations on average."""
    import torch
    from deft_gb300.warmstart import FourierOperator, make_dataset, train
    from deft_gb300.workloads import walls_solutes_set
    N = 40
    kw = dict(N=N, dx=0.2, width=(3.0, 5.0), radius=(0.6, 1.4), eta=(0.1, 0.4))
    train_set = walls_solutes_set(48, seed=11, **kw)
    held = walls_solutes_set(6, seed=12, **kw)
    ds = make_dataset(train_set, chunk=16)
    assert len(ds) >= 40
    net = FourierOperator(N=N, channels=8, modes=6, layers=4, seed=0)
    try:
        losses = train(net, ds, epochs=8, lr=3e-3, lr_final=3e-4)
        assert np.mean(losses[-48:]) < 0.5 * np.mean(losses[:48])
        it_bulk, it_ws, used_all = [], [], []
        for s in held:
            ctx, g, f = _fmt_for(s, precision=_lib.PRECISION_MIXED)
            try:
                mask = torch.tensor(s.mask.reshape(-1), device="cuda:0")
                n_ws = torch.empty_like(mask)
                used, _, g_bulk = net.initial_density(f.h, mask.data_ptr(), s.eta, s.nb,
                                                      n_ws.data_ptr(), bulk_gnorm=True)
                used_all.append(used)
                n_b = torch.tensor(s.n0.reshape(-1), device="cuda:0")
                ib, eb, gb, cb, xb = _solve_from(f, n_b, _lib.PRECISION_MIXED)
                # leave the FP32 stage where the bulk start would (1e-4 of its gradient)
                iw, ew, gw, cw, xw = _solve_from(f, n_ws, _lib.PRECISION_MIXED,
                                                 refine_abs=1e-4 * g_bulk)
                assert cb and cw and gb < 1e-9 and gw < 1e-9
                assert np.max(np.abs(xb - xw)) <= 1e-8 * np.max(np.abs(xb)) + 1e-12
                it_bulk.append(ib)
                it_ws.append(iw)
            finally:
                f.close()
                g.close()
                ctx.close()
        # the energy check may reject some estimates; most must pass it
        assert sum(used_all) >= len(held) // 2
        assert np.mean(it_ws) < np.mean(it_bulk), (it_ws, it_bulk)
    finally:
        net.close()
