"""Learned warm start: host side of the Fourier neural operator in
csrc/fno.cu (no reference counterpart; CG from the bulk density, the
reference's only start, stays the fallback and what decides convergence).

* ``FourierOperator``: the network (create, parameters, save / load, one
  forward / backward pass, Adam training steps on device-resident samples,
  the checked warm start ``initial_density``).
* ``solve_batch``: converged solves of many problems through
  ``deft_batch_solve`` (the training data: profiles the minimiser itself
  produces, to |grad F| < gtol with the FP64 gradient).
* ``make_dataset`` / ``train``: data generation on the GPU and the training
  loop, with samples kept in HBM as FP32 (mask, relative density n / nb).

Everything runs through the C ABI (include/deft_gb300.h); torch is used only
to hold device buffers.
"""
import ctypes
import json
import time

import numpy as np

from . import _lib
from ._lib import check


class FourierOperator:
    """deft_fno: N^3 grid, `channels` in {4, 8, 16}, `modes` retained per
    axis (|kx|, |ky| < modes, kz < modes), `layers` Fourier layers."""

    def __init__(self, N=128, channels=16, modes=12, layers=4, seed=0, device=0):
        self.L = _lib.load()
        self.N, self.channels, self.modes, self.layers = N, channels, modes, layers
        self.device = device
        h = ctypes.c_void_p()
        check(self.L.deft_fno_create(device, N, channels, modes, layers, seed, ctypes.byref(h)))
        self.h = h
        self.nparam = int(self.L.deft_fno_param_count(h))

    # -- parameters ---------------------------------------------------------
    def get_params(self):
        p = np.empty(self.nparam, dtype=np.float32)
        check(self.L.deft_fno_get_params(self.h, p.ctypes.data))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != self.nparam:
            raise ValueError(f"expected {self.nparam} parameters, got {p.size}")
        check(self.L.deft_fno_set_params(self.h, p.ctypes.data))

    def header(self, dtype="float32"):
        return {"format": "deft_fno", "N": self.N, "channels": self.channels,
                "modes": self.modes, "layers": self.layers, "nparam": self.nparam,
                "dtype": dtype + " little-endian"}

    def save(self, path, dtype="float32"):
        """Raw little-endian parameters in `path` and a JSON header in
        `path + '.json'`.  dtype "bfloat16" stores the values every pass
        uses (round to nearest even), half the size; training from such a
        file restarts from those values."""
        p = self.get_params()
        if dtype == "bfloat16":
            u = p.astype("<f4").view("<u4").astype(np.uint64)
            u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype("<u2")
            u.tofile(path)
        elif dtype == "float32":
            p.astype("<f4").tofile(path)
        else:
            raise ValueError(dtype)
        with open(path + ".json", "w") as f:
            json.dump(self.header(dtype), f)

    @classmethod
    def load(cls, path, device=0):
        with open(path + ".json") as f:
            h = json.load(f)
        if h.get("format") != "deft_fno":
            raise ValueError(f"{path}: not a deft_fno weight file")
        net = cls(h["N"], h["channels"], h["modes"], h["layers"], device=device)
        if h["dtype"].startswith("bfloat16"):
            u = np.fromfile(path, dtype="<u2").astype(np.uint32) << 16
            p = u.view(np.float32)
        else:
            p = np.fromfile(path, dtype="<f4")
        net.set_params(p)
        return net

    # -- passes -------------------------------------------------------------
    def eval(self, mask, eta, target=None, want_grad=False):
        """Host arrays: returns (y, loss, grad) (loss / grad None when not asked)."""
        mask = np.ascontiguousarray(mask, dtype=np.float32).reshape(-1)
        y = np.empty_like(mask)
        loss = ctypes.c_float(0)
        grad = np.empty(self.nparam, dtype=np.float32) if want_grad else None
        t = None
        if target is not None:
            t = np.ascontiguousarray(target, dtype=np.float32).reshape(-1)
        check(self.L.deft_fno_eval(self.h, mask.ctypes.data, float(eta),
                                   t.ctypes.data if t is not None else None, 0, y.ctypes.data,
                                   ctypes.addressof(loss),
                                   grad.ctypes.data if grad is not None else None))
        return y, (loss.value if t is not None else None), grad

    def train_step(self, mask_ptr, eta, target_ptr, lr):
        """One Adam step on a device-resident sample (raw device addresses of
        N^3 floats); returns the loss before the step."""
        loss = ctypes.c_float(0)
        check(self.L.deft_fno_train_step(self.h, mask_ptr, float(eta), target_ptr, 1, float(lr),
                                         ctypes.addressof(loss)))
        return loss.value

    def loss_device(self, mask_ptr, eta, target_ptr):
        loss = ctypes.c_float(0)
        check(self.L.deft_fno_eval(self.h, mask_ptr, float(eta), target_ptr, 1, None,
                                   ctypes.addressof(loss), None))
        return loss.value

    def initial_density(self, fmt_handle, mask_ptr, eta, nb, n_out_ptr, floor_rel=1e-3,
                        bulk_gnorm=False):
        """Checked warm start into the device array n_out_ptr (N^3 doubles)
        for the functional fmt_handle; returns (used_network, energy) and,
        with bulk_gnorm, the bulk start's gradient norm as a third value."""
        used = ctypes.c_int(0)
        E = ctypes.c_double(0)
        gb = ctypes.c_double(0)
        check(self.L.deft_fno_initial_density(self.h, fmt_handle, mask_ptr, float(eta), float(nb),
                                              float(floor_rel), n_out_ptr,
                                              ctypes.addressof(used), ctypes.addressof(E),
                                              ctypes.addressof(gb) if bulk_gnorm else None))
        if bulk_gnorm:
            return bool(used.value), E.value, gb.value
        return bool(used.value), E.value

    def close(self):
        if self.h:
            self.L.deft_fno_destroy(self.h)
            self.h = None


def solve_batch(problems, precision=_lib.PRECISION_MIXED, workers=8, gtol=1e-9, maxiter=20000,
                device=0, preconditioned=_lib.PC_NONE, device_driven=False):
    """Converged solves of problems with .lat/.shape/.R/.kT/.mu/.mask/.n0
    through deft_batch_solve (`workers` host threads and streams) or, with
    device_driven, deft_batch_solve_device (one graph launch for all; needs
    preconditioned = PC_DENSITY or PC_STRUCTURE, the latter falling back to
    the former on grids it does not take); returns (status, [CgStatus],
    [profiles])."""
    keep, outs = [], []
    arr = (_lib.BatchProblem * len(problems))()
    for k, s in enumerate(problems):
        mask = np.ascontiguousarray(s.mask.reshape(-1), dtype=np.float64)
        n0 = np.ascontiguousarray(s.n0.reshape(-1), dtype=np.float64)
        out = np.empty_like(n0)
        keep += [mask, n0]
        outs.append(out)
        p = arr[k]
        for i, v in enumerate(np.asarray(s.lat, dtype=np.float64).reshape(9)):
            p.lat[i] = v
        for i, v in enumerate(s.shape):
            p.N[i] = v
        p.R, p.kT, p.mu = s.R, s.kT, s.mu
        p.terms = _lib.TERM_HS | _lib.TERM_IDEAL | _lib.TERM_MU | _lib.TERM_MASK
        p.precision = precision
        p.mask = mask.ctypes.data
        p.V = None
        p.n_init = n0.ctypes.data
        p.n_out = out.ctypes.data
    cp = _lib.CgParams(_lib.LS_SECANT, gtol, maxiter, 1.0, 0.0, 0.0, int(preconditioned))
    st = (_lib.CgStatus * len(problems))()
    if device_driven:
        code = _lib.load().deft_batch_solve_device(device, len(problems), arr, ctypes.byref(cp),
                                                   st)
    else:
        bp = _lib.BatchParams(workers, cp)
        code = _lib.load().deft_batch_solve(device, len(problems), arr, ctypes.byref(bp), st)
    return code, list(st), outs


class Dataset:
    """Training samples in HBM: per problem an FP32 mask and the FP32
    relative density n / nb of its converged solution (torch device tensors),
    and eta."""

    def __init__(self):
        self.mask, self.target, self.eta, self.stats = [], [], [], []

    def __len__(self):
        return len(self.eta)


def make_dataset(problems, chunk=16, workers=8, gtol=1e-9, device=0, log=None):
    """Solves `problems` (mixed form: FP32 CG stage, then the FP64-gradient
    refinement to |grad F| < gtol) and keeps the converged relative
    densities on the device.  Problems whose minimiser stops without
    converging are skipped; an error of the batch call itself (bad
    arguments, CUDA) raises, and so does a chunk that keeps no problem."""
    import torch
    dev = f"cuda:{device}"
    ds = Dataset()
    t0 = time.perf_counter()
    for c0 in range(0, len(problems), chunk):
        part = problems[c0:c0 + chunk]
        code, st, outs = solve_batch(part, workers=workers, gtol=gtol, device=device)
        if code not in (_lib.OK, _lib.ERR_LINESEARCH, _lib.ERR_MAXITER, _lib.ERR_NAN):
            _lib.check(code)
        kept = len(ds)
        for s, r, n in zip(part, st, outs):
            if r.status or not r.converged:
                continue
            ds.mask.append(torch.tensor(s.mask.reshape(-1), dtype=torch.float32, device=dev))
            ds.target.append(torch.tensor(n / s.nb, dtype=torch.float32, device=dev))
            ds.eta.append(float(s.eta))
            ds.stats.append((r.iter, r.evals, r.gnorm))
        if len(ds) == kept:
            raise RuntimeError(f"no problem of {len(part)} converged (batch status {code})")
        if log:
            log(f"solved {min(c0 + chunk, len(problems))}/{len(problems)} "
                f"({time.perf_counter() - t0:.1f} s, kept {len(ds)})")
    return ds


def train(net, ds, epochs=2, lr=1e-3, lr_final=1e-4, seed=0, log=None, log_every=100):
    """Adam over the samples in a seeded random order, learning rate decayed
    geometrically from lr to lr_final; returns the per-step losses."""
    rng = np.random.Generator(np.random.PCG64(seed))
    steps = epochs * len(ds)
    losses = []
    t0 = time.perf_counter()
    k = 0
    for _ in range(epochs):
        for i in rng.permutation(len(ds)):
            a = lr * (lr_final / lr) ** (k / max(1, steps - 1))
            losses.append(net.train_step(ds.mask[i].data_ptr(), ds.eta[i], ds.target[i].data_ptr(),
                                         a))
            k += 1
            if log and k % log_every == 0:
                log(f"step {k}/{steps} loss {np.mean(losses[-log_every:]):.3e} "
                    f"({time.perf_counter() - t0:.1f} s)")
    return losses


class Solver:
    """One grid with a functional and a CG minimiser per precision, reused
    for every problem on that grid (the functional's mu, R, kT and mask are
    reset per problem; CG restarts on each deft_cg_set_x)."""

    def __init__(self, shape, lat, device=0, gtol=1e-9):
        L = self.L = _lib.load()
        self.gtol = gtol
        self.shape = tuple(int(v) for v in shape)
        self.size = int(np.prod(self.shape))
        h = ctypes.c_void_p()
        check(L.deft_ctx_create(device, ctypes.byref(h)))
        self.ctx = h
        lat9 = np.ascontiguousarray(np.asarray(lat, dtype=np.float64).reshape(9))
        h = ctypes.c_void_p()
        check(L.deft_grid_create(self.ctx, lat9.ctypes.data, *self.shape, ctypes.byref(h)))
        self.grid = h
        self.terms = _lib.TERM_HS | _lib.TERM_IDEAL | _lib.TERM_MU | _lib.TERM_MASK
        self.fmt, self.cg = {}, {}
        for prec in (_lib.PRECISION_FP64, _lib.PRECISION_MIXED):
            p = _lib.FmtParams(1.0, 1.0, 0.0, self.terms, prec)
            h = ctypes.c_void_p()
            check(L.deft_fmt_create(self.grid, ctypes.byref(p), ctypes.byref(h)))
            self.fmt[prec] = h
            cp = _lib.CgParams(_lib.LS_SECANT, gtol, 20000, 1.0, 0.0, 0.0)
            h = ctypes.c_void_p()
            check(L.deft_cg_create(self.fmt[prec], ctypes.byref(cp), ctypes.byref(h)))
            self.cg[prec] = h

    def set_problem(self, s, mask_ptr):
        """s: a problem (R, kT, mu); mask_ptr: device address of its mask."""
        for prec, f in self.fmt.items():
            p = _lib.FmtParams(s.R, s.kT, s.mu, self.terms, prec)
            check(self.L.deft_fmt_set_params(f, ctypes.byref(p)))
            check(self.L.deft_fmt_set_mask(f, mask_ptr, 1))

    def solve(self, precision, n0_ptr, refine_abs=0.0, preconditioned=_lib.PC_NONE, gtol=None,
              maxiter=20000, device=False):
        """Solve from the device array n0_ptr; returns (CgStatus, seconds).
        refine_abs > 0 sets the mixed form's FP32-stage exit |grad| < refine_abs;
        preconditioned = PC_DENSITY runs the CG with the density-variable
        diagonal preconditioner; gtol overrides the solver's tolerance for
        this solve; device = True runs it device-driven (deft_cg_solve_device,
        one graph launch; needs preconditioned = PC_DENSITY).
        A minimiser that stops without converging (line search, iteration
        limit, non-finite values) is reported in CgStatus.status, not raised."""
        t0 = time.perf_counter()
        cp = _lib.CgParams(_lib.LS_SECANT, self.gtol if gtol is None else float(gtol),
                           int(maxiter), 1.0, 0.0, 0.0, int(preconditioned), float(refine_abs))
        check(self.L.deft_cg_set_params(self.cg[precision], ctypes.byref(cp)))
        check(self.L.deft_cg_set_x(self.cg[precision], n0_ptr, 1))
        st = _lib.CgStatus()
        solve = self.L.deft_cg_solve_device if device else self.L.deft_cg_solve
        code = solve(self.cg[precision], ctypes.byref(st))
        if code not in (_lib.OK, _lib.ERR_LINESEARCH, _lib.ERR_MAXITER, _lib.ERR_NAN,
                        _lib.ERR_TIMEOUT):
            check(code)
        st.status = code
        return st, time.perf_counter() - t0

    def x_ptr(self, precision):
        return self.L.deft_cg_x_device(self.cg[precision])

    def close(self):
        for h in self.cg.values():
            self.L.deft_cg_destroy(h)
        for h in self.fmt.values():
            self.L.deft_fmt_destroy(h)
        self.L.deft_grid_destroy(self.grid)
        self.L.deft_ctx_destroy(self.ctx)


def compare_starts(net, problems, device=0, fp64=True, floor_rel=1e-3, switch=(None,),
                   preconditioned=_lib.PC_DENSITY):
    """Solves each problem to |grad F| < 1e-9 from the bulk start and from
    the checked warm start, in the mixed form (and in FP64 if asked); the
    warm-start time includes the network's forward pass and the energy
    checks.  `switch` lists the mixed warm-start variants: None leaves the
    FP32 stage at 1e-4 of the start's gradient norm (the default rule), a
    number c at c times the bulk start's gradient norm.  Mixed solves use
    the `preconditioned` setting (the density preconditioner by default);
    FP64 solves are the plain reference CG.  Returns one record per
    problem."""
    import torch
    dev = f"cuda:{device}"
    sv = Solver(problems[0].shape, problems[0].lat, device=device)
    recs = []

    def rec(st, t, extra=None):
        r = {"s": t, "iter": st.iter, "evals": st.evals, "evals_fp64": st.evals_fp64,
             "hvps": st.hvps, "gnorm": st.gnorm, "status": st.status,
             "converged": bool(st.converged) and st.status == 0}
        if extra:
            r.update(extra)
        return r

    try:
        for s in problems:
            mask = torch.tensor(s.mask.reshape(-1), dtype=torch.float64, device=dev)
            bulk = torch.tensor(s.n0.reshape(-1), dtype=torch.float64, device=dev)
            n_ws = torch.empty_like(mask)
            x = torch.empty_like(mask)
            sv.set_problem(s, mask.data_ptr())
            r = {"eta": s.eta, "solutes": len(getattr(s, "solutes", ())),
                 "width": getattr(s, "width", None)}
            runs = [(_lib.PRECISION_FP64, "fp64")] if fp64 else []
            runs.append((_lib.PRECISION_MIXED, "mixed"))
            ref_x = None
            for prec, name in runs:
                pc = preconditioned if prec == _lib.PRECISION_MIXED else _lib.PC_NONE
                st, t = sv.solve(prec, bulk.data_ptr(), preconditioned=pc)
                r[f"{name}_bulk"] = rec(st, t)
                if ref_x is None:
                    ref_x = torch.empty_like(mask)
                    check(sv.L.deft_cg_get_x(sv.cg[prec], ref_x.data_ptr(), 1))
                variants = switch if prec == _lib.PRECISION_MIXED else (None,)
                for c in variants:
                    t0 = time.perf_counter()
                    used, _, gb = net.initial_density(sv.fmt[prec], mask.data_ptr(), s.eta, s.nb,
                                                      n_ws.data_ptr(), floor_rel=floor_rel,
                                                      bulk_gnorm=True)
                    t_ws = time.perf_counter() - t0
                    st, t = sv.solve(prec, n_ws.data_ptr(), refine_abs=c * gb if c else 0.0,
                                     preconditioned=pc)
                    check(sv.L.deft_cg_get_x(sv.cg[prec], x.data_ptr(), 1))
                    dmax = float((x - ref_x).abs().max() / ref_x.abs().max())
                    key = f"{name}_warm" if c is None else f"{name}_warm_abs{c:g}"
                    r[key] = rec(st, t + t_ws, {"s_network": t_ws, "used_network": used,
                                                "profile_rel_diff": dmax})
            recs.append(r)
    finally:
        sv.close()
    return recs


def summarize(recs):
    """Means over the problems every run converged on (failures counted
    separately, with their status codes)."""
    keys = [k for k in recs[0] if k.endswith("_bulk") or "_warm" in k]
    ok = [r for r in recs if all(r[k]["converged"] for k in keys)]
    out = {"problems": len(recs), "all_converged": len(ok)}
    for key in keys:
        col = lambda f: [r[key][f] for r in ok]  # noqa: E731
        out[key] = {"mean_s": float(np.mean(col("s"))), "median_s": float(np.median(col("s"))),
                    "mean_iter": float(np.mean(col("iter"))),
                    "mean_evals": float(np.mean(col("evals"))),
                    "mean_evals_fp64": float(np.mean(col("evals_fp64"))),
                    "mean_hvps": float(np.mean(col("hvps"))),
                    "converged": int(sum(r[key]["converged"] for r in recs)),
                    "failures": [(i, r[key]["status"]) for i, r in enumerate(recs)
                                 if not r[key]["converged"]]}
        if "_warm" in key:
            out[key]["used_network"] = int(sum(col("used_network")))
            out[key]["max_profile_rel_diff"] = float(np.max(col("profile_rel_diff")))
            out[key]["mean_network_s"] = float(np.mean(col("s_network")))
    if "fp64_bulk" in out:
        out["speedup_mixed_bulk_vs_fp64_bulk"] = (out["fp64_bulk"]["mean_s"]
                                                  / out["mixed_bulk"]["mean_s"])
        out["speedup_fp64_warm_vs_fp64_bulk"] = (out["fp64_bulk"]["mean_s"]
                                                 / out["fp64_warm"]["mean_s"])
    for key in keys:
        if key.startswith("mixed_warm"):
            out[f"speedup_{key}_vs_fp64_bulk"] = (out["fp64_bulk"]["mean_s"] / out[key]["mean_s"]
                                                  if "fp64_bulk" in out else None)
            out[f"speedup_{key}_vs_mixed_bulk"] = out["mixed_bulk"]["mean_s"] / out[key]["mean_s"]
    return out


def main(argv=None):
    """Trains the warm-start network at N^3 on converged solutions of seeded
    wall + solute problems and reports the held-out gain as one JSON object."""
    import argparse
    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("--N", type=int, default=128)
    ap.add_argument("--count", type=int, default=2000)
    ap.add_argument("--held", type=int, default=200)
    ap.add_argument("--channels", type=int, default=16)
    ap.add_argument("--modes", type=int, default=12)
    ap.add_argument("--layers", type=int, default=4)
    ap.add_argument("--epochs", type=int, default=3)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--lr-final", type=float, default=1e-4)
    ap.add_argument("--seed", type=int, default=5)
    ap.add_argument("--held-seed", type=int, default=6)
    ap.add_argument("--fp64-held", type=int, default=None,
                    help="held-out problems also solved in FP64 (default: all)")
    ap.add_argument("--save", default=None, help="weight file to write")
    ap.add_argument("--save-dtype", default="bfloat16", choices=["bfloat16", "float32"])
    ap.add_argument("--load", default=None, help="weight file to start from (skips training "
                                                  "unless --count > 0 is given as well)")
    ap.add_argument("--switch", default="",
                    help="comma-separated c values: mixed warm-start variants leaving the "
                         "FP32 stage at c x the bulk start's gradient norm")
    ap.add_argument("--json", default=None, help="summary file to write")
    ap.add_argument("--no-precond", action="store_true",
                    help="mixed solves without the density preconditioner")
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args(argv)
    import sys
    from .workloads import walls_solutes_set

    def log(m):
        print(m, file=sys.stderr, flush=True)

    res = {}
    if a.load:
        net = FourierOperator.load(a.load, device=a.device)
        res["network"] = dict(net.header(), loaded_from=a.load)
    else:
        net = FourierOperator(a.N, a.channels, a.modes, a.layers, seed=a.seed, device=a.device)
        res["network"] = net.header()
    if not a.load or a.count > 0:
        t0 = time.perf_counter()
        ds = make_dataset(walls_solutes_set(a.count, a.seed, N=net.N), device=a.device, log=log)
        t_data = time.perf_counter() - t0
        t0 = time.perf_counter()
        losses = train(net, ds, epochs=a.epochs, lr=a.lr, lr_final=a.lr_final, seed=a.seed,
                       log=log, log_every=max(1, len(ds) // 4))
        t_train = time.perf_counter() - t0
        res["data"] = {"problems": a.count, "kept": len(ds), "seed": a.seed, "seconds": t_data,
                       "mean_iter": float(np.mean([x[0] for x in ds.stats])),
                       "form": "mixed solves refined on the FP64 gradient to |grad F| < 1e-9"}
        res["training"] = {"steps": len(losses), "epochs": a.epochs, "seconds": t_train,
                           "ms_per_step": t_train / max(1, len(losses)) * 1e3,
                           "loss_first_epoch": float(np.mean(losses[:len(ds)])),
                           "loss_last_epoch": float(np.mean(losses[-len(ds):]))}
        del ds
    if a.save:
        net.save(a.save, dtype=a.save_dtype)
    switch = (None,) + tuple(float(c) for c in a.switch.split(",") if c)
    held = walls_solutes_set(a.held, a.held_seed, N=net.N)
    nf = a.held if a.fp64_held is None else a.fp64_held
    pc = _lib.PC_NONE if a.no_precond else _lib.PC_DENSITY
    recs = compare_starts(net, held[:nf], device=a.device, fp64=True, switch=switch,
                          preconditioned=pc) if nf else []
    if nf < len(held):
        recs += compare_starts(net, held[nf:], device=a.device, fp64=False, switch=switch,
                               preconditioned=pc)
    res["held_out"] = {"seed": a.held_seed, **summarize(recs[:nf])} if nf else None
    res["held_out_mixed_only"] = summarize(recs) if nf < len(recs) else None
    net.close()
    txt = json.dumps(res, indent=1)
    if a.json:
        with open(a.json, "w") as f:
            f.write(txt)
    print(txt)
    return res


if __name__ == "__main__":
    main()
