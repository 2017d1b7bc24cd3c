"""Benchmark: converged FMT solve at 128^3 on one GB300, learned warm start
plus mixed precision against the plain FP64 GPU solve.

Workload (named in the JSON line's config): White Bear hard spheres R = 1,
kT = 1, ideal gas + mu, periodic 128^3 grid with dx = 0.2 (edge 25.6), hard
walls (n = 0, frozen by the constraint mask) outside a slit of width 3-10,
1-4 hard-sphere solutes of radius 1-4 inside it, bulk packing fraction
0.1-0.4: seeded problems held out from the network's training set.  One step
= one converged solve to |grad F|_2 < 1e-9 of the next held-out problem.

Our arm (default): value = seconds per converged solve from the checked
warm start (the Fourier-operator estimate, or the bulk density if the
estimate is non-finite or has a higher energy) with the mixed evaluator
(FP32 CG stage, then refinement on the FP64 gradient); the network's
forward pass and the start's energy checks are inside the timed step.  A
converged solve meets |grad F| < 1e-9 and has its profile within 1e-8 of
the FP64 solution of the same problem (converged to |grad F| < 1e-12 before
the timing): every timed step is checked and the run fails otherwise.  The
plain FP64 solve from the bulk density of the same problems is timed beside
it, and so are the parts of the speed-up (FP64 with the density
preconditioner, mixed from the bulk start).  Also reported: per-kernel event timings of one profiled solve (roofline
of the dominant kernel, the whole-evaluation "conv HBM GB/s"), the same step
end to end through the public API with host buffers, a cuFFT comparison of
one 3-D transform, the batched sweep, and a CPU baseline (the oracle port,
one core, on a bounded sample).

The network is the bundled one (deft_gb300/weights/fno_wb128_2000.bf16:
trained by `python -m deft_gb300.warmstart --count 2000 --epochs 3` on 2000
converged solves of the same problem family, training seed 5, disjoint from
the held-out seed), or the one --weights names, or, with --weights train (or
no bundled file), trained inside the run on --train-count solves.

--impl reference: the reference's CPU path (the plain-C restatement of it,
since the reference sources are not present where this runs): each step is
one full converged solve of that step's problem on one core, the steps run
concurrently on the host's cores.
"""
import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "converged-solve s at 128\u00b3 (warm-start+mixed vs plain FP64 GPU); conv HBM GB/s"
UNIT = "s"
GTOL = 1e-9
# The converged-solve target: |grad F| < 1e-9 and the density profile within
# 1e-8 of the FP64 solution.  The mixed solve stops at |grad F| < 3e-10 with
# the structure preconditioner (5e-10 with the density one): the structure
# preconditioner's Newton steps leave a residual spread over all
# wavelengths, whose short-wavelength part moves the profile most, so the
# same |grad F| bound leaves a larger profile error (worst of 20 held-out
# 128^3 problems: 1.2e-8 at 5e-10, 4.3e-9 at 3e-10; density
# preconditioner, 3.1e-9 at 5e-10).  Every timed step's profile is checked
# against the FP64 solution of the same problem converged to
# |grad F| < 1e-12, and a step outside 1e-8 fails the run.
MIXED_GTOL = None  # per preconditioner, below
MIXED_GTOL_PC = {"density": 5e-10, "structure": 3e-10, "none": 5e-10}
PROFILE_TOL = 1e-8
REF_GTOL = 1e-12
HELD_SEED = 6
TRAIN_SEED = 5
HBM_FALLBACK_GBS = 6800.0
BUNDLED_WEIGHTS = os.path.join(ROOT, "deft_gb300", "weights", "fno_wb128_2000.bf16")


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return HBM_FALLBACK_GBS, "fallback"


def held_out(N, count):
    from deft_gb300.workloads import walls_solutes_set
    return walls_solutes_set(count, HELD_SEED, N=N)


def config(N, extra=None):
    c = {
        "workload": f"White Bear FMT, {N}^3, dx=0.2, R=1, kT=1: hard-wall slit (width 3-10) "
                    f"with 1-4 hard-sphere solutes (radius 1-4), eta 0.1-0.4, seeded held-out "
                    f"problems (seed {HELD_SEED}); CG to |grad F|<1e-9",
        "grid": [N, N, N],
        "dx": 0.2,
        "gtol": GTOL,
        "l2": "inputs larger than L2 between steps: each step is a different problem and "
              "streams ~0.4 GB of fields through every evaluation",
    }
    if extra:
        c.update(extra)
    return c


# ---------------------------------------------------------------------------
# clocks sampling

class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                for nm, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(nm)
            except Exception:
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "samples": len(sm),
                "reasons": sorted(reasons)}


# ---------------------------------------------------------------------------
# our arm

def alg_bytes(N, fp32, vec_bytes=8):
    """Algorithmic bytes per launch of each kernel: the compulsory field reads
    and writes of the stage (nothing for the analytic weights).  Real fields
    at the boundary (n, mask, gradient) are R = vec_bytes N^3: FP64 (8) in
    general, FP32 (4) on the FP32 vectors of the mixed form's CG stages;
    spectra are C = 16 N^2 (N/2+1) in the FP64 form and 8 N^2 (N/2+1) in the
    mixed form."""
    NR = N ** 3
    NC = N * N * (N // 2 + 1)
    R, C = vec_bytes * NR, (8 if fp32 else 16) * NC
    return {
        "z_r2c": R + C,
        "y_fft_1field": 2 * C,
        "y_fft_5fields": 10 * C,
        "x_conv_fwd": C + 5 * C,
        "z_phi_grad": 5 * C + R + 5 * C,
        "z_phi_energy": 5 * C + R,
        "x_conv_adj": 5 * C + C,
        "z_grad": C + 3 * R,
        "z_hess": 5 * C + 8 * NR + 44 * NR,  # set up at the FP64 iterate
        "z_jac": 5 * C + 40 * NR + 5 * C,
        "z_hvp_out": C + 4 * NR + 3 * R,
        "eval_model": 4 * R + 24 * C,  # one energy+gradient evaluation
    }


CONV_KERNELS = ("z_r2c", "y_fft_1field", "y_fft_5fields", "x_conv_fwd", "z_phi_grad",
                "z_phi_energy", "x_conv_adj", "z_grad")


def f32_vectors(N, pc_none):
    """Whether the mixed solves keep their CG vectors in FP32 (the library's
    rule: a preconditioned secant CG, hard spheres on, Nz = 32, 64, 128 or
    256, and DEFT_F32_VECTORS not set to 0)."""
    ev = os.environ.get("DEFT_F32_VECTORS")
    try:
        on = int(ev) != 0 if ev else True
    except ValueError:
        on = False
    return on and not pc_none and N in (32, 64, 128, 256)


def kernel_profile(L, grid):
    name = ctypes.c_char_p()
    launches = ctypes.c_longlong()
    tot = ctypes.c_double()
    prof = {}
    for i in range(L.deft_grid_profile_count(grid)):
        L.deft_grid_profile_entry(grid, i, ctypes.byref(name), ctypes.addressof(launches),
                                  ctypes.addressof(tot))
        if launches.value:
            prof[name.value.decode()] = (launches.value, tot.value)
    return prof


def kernel_table(prof):
    total = sum(v[1] for v in prof.values()) or 1.0
    return {k: {"launches": round(v[0], 2), "ms_total": round(v[1], 3),
                "share": round(v[1] / total, 4),
                "us_per_launch": round(1e3 * v[1] / v[0], 2)}
            for k, v in sorted(prof.items(), key=lambda kv: -kv[1][1])}


def by_precision(prof, fp32):
    """The profile entries of one arithmetic type, under their kernel names
    (FP32 launches carry a "_f32" suffix in the engine's accounting)."""
    out = {}
    for k, v in prof.items():
        if k.endswith("_f32") == fp32:
            out[k[:-4] if fp32 else k] = v
    return out


def roofline(prof, N, fp32, peak, peak_kind, vec_bytes=8):
    prof = by_precision(prof, fp32)
    ab = alg_bytes(N, fp32, vec_bytes)
    dom = max((k for k in prof if k in ab), key=lambda k: prof[k][1])
    dom_ms = prof[dom][1] / prof[dom][0]
    achieved = ab[dom] / (dom_ms * 1e-3) / 1e9
    conv_ms = sum(prof[k][1] for k in CONV_KERNELS if k in prof)
    n_eval = prof.get("z_phi_grad", (0, 0))[0] + prof.get("z_phi_energy", (0, 0))[0]
    conv_gbs = ab["eval_model"] * n_eval / (conv_ms * 1e-3) / 1e9 if conv_ms else None
    traffic = None
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tp):
        try:
            with open(tp) as fh:
                traffic = json.load(fh).get(f"{'fp32' if fp32 else 'fp64'}_{N}_{dom}")
        except Exception:
            traffic = None
    # every kernel of the evaluation and the Hessian-vector product with its
    # algorithmic bytes per launch against its mean event time
    by_kernel = {}
    for k, (nl, ms) in sorted(prof.items(), key=lambda kv: -kv[1][1]):
        if k in ab and nl:
            us = 1e3 * ms / nl
            gbs = ab[k] / (us * 1e-6) / 1e9
            by_kernel[k] = {"us_per_launch": round(us, 2), "alg_MB": round(ab[k] / 1e6, 1),
                            "GB_s": round(gbs, 1), "frac": round(gbs / peak, 3)}
    return {
        "bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
        "frac": achieved / peak, "traffic": traffic, "alg_bytes_per_launch": ab[dom],
        "avg_launch_ms": dom_ms, "by_kernel": by_kernel,
        "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
        else "fallback 6.8 TB/s",
        "conv_hbm_gbs": conv_gbs, "conv_frac": conv_gbs / peak if conv_gbs else None,
    }


def get_network(args, N, dev, log):
    """The warm-start network: --weights, or trained here on --train-count
    solves of the same family (training seed, disjoint from the held-out seed)."""
    from deft_gb300.warmstart import FourierOperator, make_dataset, train
    from deft_gb300.workloads import walls_solutes_set
    if args.weights != "train":
        net = FourierOperator.load(args.weights, device=dev)
        bundled = os.path.basename(args.weights) == os.path.basename(BUNDLED_WEIGHTS)
        return net, {"source": os.path.relpath(args.weights, ROOT),
                     "trained_on": "2000 converged solves (mixed, refined on the FP64 gradient "
                                   "to |grad F| < 1e-9) of seeded wall + solute problems, "
                                   f"training seed {TRAIN_SEED}, 3 epochs (python -m "
                                   "deft_gb300.warmstart --count 2000 --epochs 3)"
                     if bundled else "given with --weights"}
    t0 = time.perf_counter()
    ds = make_dataset(walls_solutes_set(args.train_count, TRAIN_SEED, N=N), device=dev,
                      workers=args.train_workers)
    t_data = time.perf_counter() - t0
    net = FourierOperator(N, 16, 12, 4, seed=TRAIN_SEED, device=dev)
    t0 = time.perf_counter()
    losses = train(net, ds, epochs=args.train_epochs, lr=1e-3, lr_final=1e-4, seed=TRAIN_SEED)
    info = {"source": f"trained in this run on {len(ds)} converged solves "
                      f"(seed {TRAIN_SEED}), {args.train_epochs} epochs",
            "data_s": t_data, "train_s": time.perf_counter() - t0,
            "loss_first_epoch": float(np.mean(losses[:len(ds)])),
            "loss_last_epoch": float(np.mean(losses[-len(ds):]))}
    del ds
    log(f"network: {info}")
    return net, info


def cufft_comparison(N, dev):
    """One 3-D r2c of an N^3 FP64 field: this library's FFT against cuFFT
    (through torch.fft), both on device data, CUDA-event timed."""
    import torch
    from deft_gb300 import _lib
    L = _lib.load()
    x = torch.randn(N, N, N, dtype=torch.float64, device=f"cuda:{dev}")
    out = torch.empty(N, N, N // 2 + 1, dtype=torch.complex128, device=f"cuda:{dev}")
    h = ctypes.c_void_p()
    _lib.check(L.deft_ctx_create(dev, ctypes.byref(h)))
    ctx = h
    lat = np.ascontiguousarray(np.diag([0.2 * N] * 3).reshape(9))
    h = ctypes.c_void_p()
    _lib.check(L.deft_grid_create(ctx, lat.ctypes.data, N, N, N, ctypes.byref(h)))
    grid = h
    stream = torch.cuda.ExternalStream(L.deft_ctx_stream(ctx), device=f"cuda:{dev}")
    reps = 20
    for _ in range(3):
        _lib.check(L.deft_grid_fft(grid, x.data_ptr(), out.data_ptr(), 1))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        _lib.check(L.deft_grid_fft(grid, x.data_ptr(), out.data_ptr(), 1))
    e1.record(stream)
    e1.synchronize()
    ours = e0.elapsed_time(e1) / reps
    ref = torch.fft.rfftn(x) * (0.2 ** 3)
    err = float((out - ref).abs().max() / ref.abs().max())
    for _ in range(3):
        torch.fft.rfftn(x)
    torch.cuda.synchronize()
    c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    c0.record()
    for _ in range(reps):
        torch.fft.rfftn(x)
    c1.record()
    c1.synchronize()
    cu = c0.elapsed_time(c1) / reps
    L.deft_grid_destroy(grid)
    L.deft_ctx_destroy(ctx)
    return {"what": f"one {N}^3 FP64 r2c (x dV for ours), device data", "ours_ms": ours,
            "cufft_ms": cu, "max_rel_diff": err, "note": "cuFFT timed only as a comparison"}


def max_over_ranks(ms, world, device):
    """A barrier-bracketed step time reduced to its maximum over the ranks
    (each rank an independent replica on its own GPU: the only exchange is
    this scalar); with one rank ms is returned unchanged."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(ms)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_ours(args, rank, world):
    import torch
    from deft_gb300 import _lib, autotune
    from deft_gb300.warmstart import Solver

    def log(m):
        if args.verbose:
            print(m, file=sys.stderr, flush=True)

    L = _lib.load()
    N = args.N
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    tuned = autotune.load(args.tuning, device=dev) if args.tuning else autotune.load(device=dev)
    peak, peak_kind = measured_peaks()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    net, net_info = get_network(args, N, dev, log)
    probs = held_out(N, args.steps + args.warmup)
    sv = Solver(probs[0].shape, probs[0].lat, device=dev, gtol=GTOL)
    stream = torch.cuda.ExternalStream(L.deft_ctx_stream(sv.ctx), device=f"cuda:{dev}")
    dd = f"cuda:{dev}"
    # inputs resident in HBM before the timed region
    masks = [torch.tensor(s.mask.reshape(-1), device=dd) for s in probs]
    bulks = [torch.tensor(s.n0.reshape(-1), device=dd) for s in probs]
    n_ws = torch.empty_like(masks[0])
    MIXED, FP64 = _lib.PRECISION_MIXED, _lib.PRECISION_FP64
    global MIXED_GTOL
    MIXED_GTOL = (args.gtol_mixed if args.gtol_mixed else
                  MIXED_GTOL_PC["none" if args.no_precond else args.pc])
    PC = (_lib.PC_NONE if args.no_precond else
          _lib.PC_STRUCTURE if args.pc == "structure" else _lib.PC_DENSITY)
    # mixed solves driven from the host (one graph replay and sync per
    # evaluation; measured 0.3 ms per solve faster at 128^3 than the
    # device-driven graph) unless --device-driven (needs the preconditioner)
    DEVICE = PC in (_lib.PC_DENSITY, _lib.PC_STRUCTURE) and args.device_driven
    # FP32 stage exit |grad| < SWITCH x the bulk start's |grad|: with the
    # preconditioner, 1e-5 was the fastest of 1e-5, 3e-5, 3e-4 and the
    # relative rule on 30 held-out problems (python -m deft_gb300.warmstart
    # --count 256 --epochs 2 --held 30 --fp64-held 0 --switch 1e-5,3e-5,3e-4)
    # (structure preconditioner: 3e-6 against 1e-5 and 3e-5 in one call on
    # 20 held-out problems, 15.0 / 15.3 / 16.1 ms, fewer FP64 evaluations)
    SWITCH = args.switch if args.switch else {_lib.PC_NONE: 1e-4, _lib.PC_DENSITY: 1e-5,
                                              _lib.PC_STRUCTURE: 3e-6}[PC]
    timed_idx = [args.warmup + k for k in range(args.steps)]

    # The profile condition's reference: each timed problem solved in FP64
    # (density preconditioner) to |grad F| < 1e-12, before any timing.
    t0 = time.perf_counter()
    refs, ref_stats = {}, []
    for i in timed_idx:
        sv.set_problem(probs[i], masks[i].data_ptr())
        st, _ = sv.solve(FP64, bulks[i].data_ptr(), preconditioned=_lib.PC_DENSITY, gtol=REF_GTOL)
        if not (st.converged and st.status == 0 and st.gnorm < REF_GTOL):
            raise RuntimeError(f"FP64 reference solve of problem {i} did not converge "
                               f"(status {st.status}, |grad| {st.gnorm:.3e})")
        refs[i] = torch.empty_like(masks[0])
        _lib.check(L.deft_cg_get_x(sv.cg[FP64], refs[i].data_ptr(), 1))
        ref_stats.append((st.iter, st.evals))
    ref_s = time.perf_counter() - t0
    outs = {i: torch.empty_like(masks[0]) for i in timed_idx}  # each timed step's profile

    def profile_errors(i, x):
        d = float((x - refs[i]).abs().max())
        return d, d / float(refs[i].abs().max())

    phases = {"network_s": [], "cg_s": []}
    bulk_gn = {}

    def warm_step(i, device=None):
        s = probs[i]
        sv.set_problem(s, masks[i].data_ptr())
        t0 = time.perf_counter()
        used, _, gb = net.initial_density(sv.fmt[MIXED], masks[i].data_ptr(), s.eta, s.nb,
                                          n_ws.data_ptr(), bulk_gnorm=True)
        bulk_gn[i] = gb
        t1 = time.perf_counter()
        st, _ = sv.solve(MIXED, n_ws.data_ptr(), refine_abs=SWITCH * gb, preconditioned=PC,
                         gtol=MIXED_GTOL,
                         device=DEVICE if device is None else device)
        if i in outs:
            _lib.check(L.deft_cg_get_x(sv.cg[MIXED], outs[i].data_ptr(), 1))
        phases["network_s"].append(t1 - t0)
        phases["cg_s"].append(time.perf_counter() - t1)
        return st, used

    def fp64_step(i, pc=_lib.PC_NONE):
        sv.set_problem(probs[i], masks[i].data_ptr())
        st, _ = sv.solve(FP64, bulks[i].data_ptr(), preconditioned=pc)
        if i in outs:
            _lib.check(L.deft_cg_get_x(sv.cg[FP64], outs[i].data_ptr(), 1))
        return st, True

    def mixed_bulk_step(i):
        sv.set_problem(probs[i], masks[i].data_ptr())
        st, _ = sv.solve(MIXED, bulks[i].data_ptr(), refine_abs=SWITCH * bulk_gn[i],
                         preconditioned=PC, gtol=MIXED_GTOL, device=DEVICE)
        if i in outs:
            _lib.check(L.deft_cg_get_x(sv.cg[MIXED], outs[i].data_ptr(), 1))
        return st, True

    def timed(step, label, warmup=True, clocked=True, gtol=GTOL):
        if warmup:
            for i in range(args.warmup):
                step(i)
        clocks = Clocks(dev)
        if clocked:
            clocks.start()
        barrier()
        torch.cuda.synchronize()
        _lib.check(L.deft_ctx_sync(sv.ctx))
        launches0 = sum(v[0] for v in kernel_profile(L, sv.grid).values())
        fno0 = L.deft_fno_launches(net.h)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        stats = [step(i) for i in timed_idx]
        e1.record(stream)
        e1.synchronize()
        torch.cuda.synchronize()
        barrier()
        ck = clocks.stop() if clocked else None
        ms = max_over_ranks(e0.elapsed_time(e1), world, dd)
        nl = (sum(v[0] for v in kernel_profile(L, sv.grid).values()) - launches0
              + L.deft_fno_launches(net.h) - fno0)
        bad = [k for k, (st, _) in enumerate(stats) if not (st.converged and st.status == 0
                                                              and st.gnorm < gtol)]
        if bad:
            raise RuntimeError(f"{label}: steps {bad} did not converge")
        errs = [profile_errors(i, outs[i]) for i in timed_idx]
        return ms / args.steps, stats, ck, nl, errs

    def err_summary(errs, gate):
        worst_abs = max(e[0] for e in errs)
        worst_rel = max(e[1] for e in errs)
        out = {"max_abs_dn": worst_abs, "max_dn_rel_to_max_n": worst_rel,
               "per_step_max_abs_dn": [float(f"{e[0]:.3e}") for e in errs],
               "within_1e-8": bool(worst_abs <= PROFILE_TOL and worst_rel <= PROFILE_TOL)}
        if gate and not out["within_1e-8"]:
            raise RuntimeError(f"profile condition failed: max |dn| {worst_abs:.3e}, "
                               f"relative {worst_rel:.3e} (limit {PROFILE_TOL:g})")
        return out

    _lib.check(L.deft_grid_profile(sv.grid, 0))
    ms_w, st_w, ck_w, nl_w, err_w = timed(warm_step, "warm start + mixed", gtol=MIXED_GTOL)
    prof_err_w = err_summary(err_w, gate=True)
    phase_means = {k: float(np.mean(v[-args.steps:])) for k, v in phases.items()}
    ms_64, st_64, ck_64, nl_64, err_64 = timed(fp64_step, "plain FP64")
    prof_err_64 = err_summary(err_64, gate=False)
    avg = lambda sts, k: sum(getattr(x[0], k) for x in sts) / len(sts)  # noqa: E731
    # the speed-up's parts: preconditioner (FP64 with it, from the bulk
    # start), precision (mixed with it, from the bulk start), network
    PC_ARM = _lib.PC_DENSITY if PC == _lib.PC_NONE else PC
    pc_name = "structure" if PC_ARM == _lib.PC_STRUCTURE else "density"
    ms_pc, st_pc, _, _, err_pc = timed(lambda i: fp64_step(i, PC_ARM),
                                       f"FP64 + {pc_name} preconditioner", clocked=False)
    ms_mb, st_mb, _, _, err_mb = timed(mixed_bulk_step, "mixed from the bulk start",
                                       warmup=False, clocked=False, gtol=MIXED_GTOL)
    prof_err_mb = err_summary(err_mb, gate=True)
    decomposition = {
        "fp64_bulk_s": ms_64 / 1e3, "fp64_precond_bulk_s": ms_pc / 1e3,
        "mixed_precond_bulk_s": ms_mb / 1e3, "warm_mixed_s": ms_w / 1e3,
        "preconditioner_x": ms_64 / ms_pc, "precision_x": ms_pc / ms_mb,
        "network_x": ms_mb / ms_w,
        "fp64_precond_bulk": {"iters": avg(st_pc, "iter"), "evals": avg(st_pc, "evals"),
                              "profile_vs_fp64_solution": err_summary(err_pc, gate=False)},
        "mixed_precond_bulk": {"iters": avg(st_mb, "iter"), "evals": avg(st_mb, "evals"),
                               "evals_fp64": avg(st_mb, "evals_fp64"), "hvps": avg(st_mb, "hvps"),
                               "profile_vs_fp64_solution": prof_err_mb},
        "note": "same held-out problems, CUDA-event timed like the headline: plain FP64 (no "
                f"preconditioner) / FP64 with the {pc_name} preconditioner / mixed with it, "
                "both from the bulk start / mixed from the checked warm start",
    }

    # Profiled passes (per-kernel CUDA events; launches go out one by one):
    # the headline's timed problems again, for the kernel table, the roofline
    # and the host time between kernels.  (NVTX range "warm_mixed_step"
    # around the first: an ncu launch list of that one solve is
    # `ncu --nvtx --nvtx-include "warm_mixed_step/" --metrics gpu__time_duration.sum`)
    _lib.check(L.deft_grid_profile(sv.grid, 1))
    torch.cuda.nvtx.range_push("warm_mixed_step")
    warm_step(timed_idx[0], device=False)
    torch.cuda.nvtx.range_pop()
    for i in timed_idx[1:]:
        warm_step(i, device=False)
    prof_w = kernel_profile(L, sv.grid)
    _lib.check(L.deft_grid_profile(sv.grid, 1))
    fp64_step(timed_idx[0])
    prof_64 = kernel_profile(L, sv.grid)
    _lib.check(L.deft_grid_profile(sv.grid, 0))
    engine_ms_step = sum(v[1] for v in prof_w.values()) / len(timed_idx)
    prof_w1 = {k: (v[0] / len(timed_idx), v[1] / len(timed_idx)) for k, v in prof_w.items()}
    fwd_ms = network_forward_ms(L, net, masks[timed_idx[0]], probs[timed_idx[0]], n_ws, stream)
    host_gap = {"timed_ms_per_step": ms_w, "engine_kernels_ms_per_step": engine_ms_step,
                "network_forward_ms": fwd_ms,
                "gap_ms_per_step": ms_w - engine_ms_step - fwd_ms,
                "note": "timed step minus the summed per-kernel CUDA-event times of the same "
                        "problems' solves (engine) and the wall time of the network's forward "
                        "pass: the time the GPU waits on the host (line-search decisions, "
                        "scalar reads); the forward pass's own launch gaps are not counted "
                        "in it"}

    # end to end through the public API with host buffers: the problem's mask
    # goes in, the converged profile comes out, every step
    mask_host = [torch.tensor(s.mask.reshape(-1)).pin_memory() for s in probs]
    out_host = {i: torch.empty(probs[0].size, dtype=torch.float64).pin_memory()
                for i in timed_idx}
    mask_dev = torch.empty_like(masks[0])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in timed_idx:
        s = probs[i]
        mask_dev.copy_(mask_host[i], non_blocking=True)
        torch.cuda.current_stream().synchronize()
        sv.set_problem(s, mask_dev.data_ptr())
        used, _, gb = net.initial_density(sv.fmt[MIXED], mask_dev.data_ptr(), s.eta, s.nb,
                                          n_ws.data_ptr(), bulk_gnorm=True)
        st, _ = sv.solve(MIXED, n_ws.data_ptr(), refine_abs=SWITCH * gb, preconditioned=PC,
                         gtol=MIXED_GTOL, device=DEVICE)
        _lib.check(L.deft_cg_get_x(sv.cg[MIXED], out_host[i].data_ptr(), 0))
    e2e_s = (time.perf_counter() - t0) / len(timed_idx)
    err_e2e = [profile_errors(i, out_host[i].to(dd)) for i in timed_idx]
    e2e = {"value": e2e_s, "unit": UNIT, "h2d_bytes_per_step": 8 * probs[0].size,
           "d2h_bytes_per_step": 8 * probs[0].size,
           "api": "pinned host mask -> device, FourierOperator.initial_density "
                  "(deft_fno_initial_density), deft_cg_set_x + deft_cg_solve, deft_cg_get_x "
                  "to a pinned host buffer",
           "profile_vs_fp64_solution": err_summary(err_e2e, gate=True)}

    used_net = sum(1 for _, u in st_w if u)
    result = {
        "metric": METRIC,
        "value": ms_w / 1e3,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_w,
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 FFT/phi + f64 reductions and refinement (network: bf16 weights, "
                 "f32 accumulate)",
        "data": "synthetic (seeded wall + solute problems, see config)",
        "config": config(N, {
            "parallelism": "replicas only" if world > 1 else "single GPU",
            "form": "checked learned warm start, FP32 CG stage" +
                    ("" if args.no_precond else
                     " (bulk structure-factor preconditioner s F^-1[F[s r] / H_b(k)], "
                     "s = sqrt(n / n_b), in the FP32 stage and the Newton step's linear CG)"
                     if PC == _lib.PC_STRUCTURE else
                     " (density-variable diagonal preconditioner n/(kT dV))") +
                    ", Newton refinement on the FP64 gradient (FP32 stage "
                    f"left at {SWITCH:g} of the bulk start's gradient norm); "
                    + ("device-driven: each solve is one CUDA graph launch (conditional "
                       "WHILE/SWITCH/IF nodes, every decision in a kernel)" if DEVICE
                       else "host-driven (one graph replay and sync per evaluation)"),
            "gtol_mixed": MIXED_GTOL,
            "profile_condition": f"max |n - n_FP64| <= {PROFILE_TOL:g} (absolute and relative "
                                 f"to max n) against the FP64 solution of the same problem "
                                 f"converged to |grad F| < {REF_GTOL:g} (density-preconditioned "
                                 f"FP64 CG, {ref_s:.1f} s for the {len(timed_idx)} problems, "
                                 f"outside the timed region); checked on every timed step",
            "warm_mixed": {"solve_s": ms_w / 1e3, "iters": avg(st_w, "iter"),
                           "evals": avg(st_w, "evals"), "evals_fp64": avg(st_w, "evals_fp64"),
                           "hvps": avg(st_w, "hvps"), "network_used": used_net,
                           "max_final_gnorm_fp64": max(x[0].gnorm for x in st_w),
                           "profile_vs_fp64_solution": prof_err_w,
                           "host_wall_split_s": dict(phase_means,
                                                     note="host wall time per timed step: "
                                                          "checked warm start (network "
                                                          "forward + energy checks) and CG")},
            "fp64_bulk": {"solve_s": ms_64 / 1e3, "iters": avg(st_64, "iter"),
                          "evals": avg(st_64, "evals"), "max_final_gnorm":
                              max(x[0].gnorm for x in st_64),
                          "gpu_launches": nl_64,
                          "profile_vs_fp64_solution": prof_err_64,
                          "note": "plain FP64 CG stopped at |grad F| < 1e-9, the same rule "
                                  "as the reference's drivers; its profile is not held to "
                                  "the 1e-8 condition (reported), so this denominator is the "
                                  "faster, looser solve"},
            "speedup_warm_mixed_vs_fp64": ms_64 / ms_w,
            "decomposition": decomposition,
            "host_gap": host_gap,
            "network": net_info,
            "tuning_entries_loaded": tuned,
            "cuda_graphs": "evaluations and Hessian-vector products replayed as graphs in the "
                           "timed steps; the profiled step launches kernel by kernel",
        }),
        "e2e": e2e,
        "gpu_launches": nl_w,
        "clocks": ck_w,
        "clocks_fp64": ck_64,
        # the profiled solve's FP32 launches run on FP32 vectors, all but the
        # warm start's two checks (bulk start and estimate, FP64 at their
        # boundary) and the Hessian set-up at the FP64 iterate
        "roofline": roofline(prof_w1, N, True, peak, peak_kind,
                             vec_bytes=4 if f32_vectors(N, PC == _lib.PC_NONE) else 8),
        "roofline_fp64": dict(roofline(prof_64, N, False, peak, peak_kind),
                              note="FP64 form: bound by the FP64 pipe (measured 1.0 TFLOP/s "
                                   "FMA on this GB300), not by HBM"),
        "kernels": kernel_table(prof_w1),
        "kernels_fp64": kernel_table(prof_64),
    }
    if not args.no_extra:
        result["cufft_comparison"] = cufft_comparison(N, dev)
        result["batched_sweep"] = batched_sweep()
    if rank == 0 and world == 1 and not args.no_cpu:
        result["cpu_baseline"] = cpu_baseline(N, probs[args.warmup], avg(st_64, "evals"),
                                              budget_s=args.cpu_budget)
    net.close()
    sv.close()
    return result


def network_forward_ms(L, net, mask, s, n_out, stream, reps=5):
    """Wall time of the network's forward pass alone (deft_fno_warm_start on
    the problem's mask, which runs on the network's own stream and
    synchronises it before returning), median of `reps`, in ms."""
    import torch
    from deft_gb300 import _lib
    times = []
    for k in range(reps + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _lib.check(L.deft_fno_warm_start(net.h, mask.data_ptr(), s.eta, s.nb, 1e-3,
                                         n_out.data_ptr()))
        torch.cuda.synchronize()
        if k:
            times.append(1e3 * (time.perf_counter() - t0))
    return float(statistics.median(times))


def batched_sweep(count=64, seed=3):
    """The batched sweep (64 slits, eta in [0.05, 0.45], grids from
    {32,48,64,96,128}^3, dx = 0.2, slit widths 3-10): mixed form with the
    structure preconditioner (the density one on the 48^3 and 96^3 grids,
    which it does not take), solved (1) as one graph launch of 64
    device-driven solves (deft_batch_solve_device; the time includes each
    problem's grid set-up and the graph's capture), (2) by deft_batch_solve
    on 8 host threads and streams, (3) one after another on one stream.  The
    device batch's profiles are checked against the 8-stream ones."""
    import numpy as np
    from deft_gb300 import _lib
    from deft_gb300.warmstart import solve_batch
    from deft_gb300.workloads import batch_sweep
    probs = batch_sweep(count=count, seed=seed)
    PCD = _lib.PC_STRUCTURE
    solve_batch(probs[:8], workers=8, preconditioned=PCD)  # warm-up: module, plans
    solve_batch(probs[:8], preconditioned=PCD, device_driven=True)
    t0 = time.perf_counter()
    code_d, st_d, x_d = solve_batch(probs, preconditioned=PCD, device_driven=True)
    t_dev = time.perf_counter() - t0
    phases = np.zeros(3)
    _lib.check(_lib.load().deft_batch_device_times(phases.ctypes.data))
    t0 = time.perf_counter()
    code, st, x_h = solve_batch(probs, workers=8, preconditioned=PCD)
    t_conc = time.perf_counter() - t0
    t0 = time.perf_counter()
    code1, _, _ = solve_batch(probs, workers=1, preconditioned=PCD)
    t_seq = time.perf_counter() - t0
    conv = sum(1 for x in st if x.converged and x.gnorm < GTOL)
    conv_d = sum(1 for x in st_d if x.converged and x.gnorm < GTOL)
    dn = max(float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)) for a, b in zip(x_d, x_h))
    return {"problems": count, "converged_device": conv_d, "converged_8_streams": conv,
            "status": code_d or code or code1,
            "seconds_one_launch": t_dev,
            "one_launch_phases_s": {"set_up": float(phases[0]), "graph_build": float(phases[1]),
                                    "solve": float(phases[2])},
            "seconds_8_streams": t_conc, "seconds_1_stream": t_seq,
            "solves_per_s": count / t_dev, "solves_per_s_8_streams": count / t_conc,
            "max_profile_rel_diff_device_vs_streams": dn,
            "grid_points": int(sum(p.size for p in probs)),
            "form": "mixed (FP32 CG stage + FP64-residual Newton refinement), structure "
                    "preconditioner (density on 48^3 and 96^3), |grad F|<1e-9"}


def cpu_eval_seconds(s, budget_s, max_evals=8):
    """Seconds per energy+gradient evaluation of the oracle port on problem
    s, timed on up to max_evals evaluations within about budget_s."""
    from oracle import oracle as O
    O.build()
    P = O.Problem(s.lat, s.shape, mu=s.mu, terms=O.HS | O.IDEAL | O.MU, mask=s.mask.reshape(-1))
    n = s.n0.reshape(-1)
    t0 = time.perf_counter()
    k = 0
    while k < max_evals:
        P.energy_grad(n)
        k += 1
        if time.perf_counter() - t0 > budget_s:
            break
    return (time.perf_counter() - t0) / k, k


def cpu_baseline(N, s, evals_per_solve, budget_s=20.0):
    sec, k = cpu_eval_seconds(s, budget_s)
    return {"value": sec * evals_per_solve, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{k} energy+gradient evaluations of a held-out {N}^3 problem by the "
                      f"oracle port ({sec:.3f} s each, 1 thread), scaled by the "
                      f"{evals_per_solve:.0f} evaluations the plain FP64 solve takes with the "
                      f"same CG"}


# ---------------------------------------------------------------------------
# reference arm

def _port_warm(task):
    """Worker warm-up: loads the oracle port and runs one evaluation."""
    N, i = task
    from oracle import oracle as O
    s = held_out(N, i + 1)[i]
    P = O.Problem(s.lat, s.shape, mu=s.mu, terms=O.HS | O.IDEAL | O.MU, mask=s.mask.reshape(-1))
    P.energy_grad(s.n0.reshape(-1))
    return i


def _port_solve(task):
    """One converged solve by the oracle port (the plain-C restatement of the
    reference path: White Bear + ideal gas + mu + hard-wall constraint, the
    same secant-search PR-CG from the bulk start as the plain FP64 GPU arm)
    in a worker process on one core: (index, seconds, evaluations, iterations,
    final |grad F|)."""
    N, i, gtol = task
    from oracle import oracle as O
    s = held_out(N, i + 1)[i]
    P = O.Problem(s.lat, s.shape, mu=s.mu, terms=O.HS | O.IDEAL | O.MU, mask=s.mask.reshape(-1))
    n0 = s.n0.reshape(-1)
    t0 = time.perf_counter()
    _, info = P.cg_solve(n0, gtol=gtol, maxiter=20000)
    return i, time.perf_counter() - t0, info["evals"], info["iters"], info["gnorm"]


def run_reference(args, rank, world):
    """The reference's CPU path on the host cores: every timed step is one
    full converged solve (|grad F| < 1e-9) of that step's held-out problem by
    the oracle port, single-threaded as the reference is; the steps run
    concurrently, one per core, in a spawned process pool.  value = mean
    seconds per solve.  Warm-up: one evaluation per worker."""
    if rank != 0:
        return None
    import multiprocessing as mp
    from oracle import oracle as O
    O.build()
    N = args.N
    timed_idx = [args.warmup + k for k in range(args.steps)]
    cores = os.cpu_count() or 1
    workers = max(1, min(len(timed_idx), cores))
    ctx = mp.get_context("spawn")
    with ctx.Pool(workers) as pool:
        pool.map(_port_warm, [(N, args.warmup)] * workers, chunksize=1)
        t0 = time.perf_counter()
        res = list(pool.imap_unordered(_port_solve, [(N, i, GTOL) for i in timed_idx],
                                       chunksize=1))
        wall = time.perf_counter() - t0
    res.sort()
    bad = [r[0] for r in res if not r[4] < GTOL]
    if bad:
        raise RuntimeError(f"oracle port solves of problems {bad} did not converge")
    secs = [r[1] for r in res]
    evals = [r[2] for r in res]
    v = sum(secs) / len(secs)
    s_per_eval = sum(secs) / sum(evals)
    sample = (f"{len(res)} full converged solves (|grad F| < {GTOL:g}) of the timed held-out "
              f"{N}^3 problems by the oracle port (plain-C restatement of the reference path, "
              f"single-threaded like the reference), {workers} at a time on {workers} of "
              f"{cores} host cores; mean {statistics.mean(evals):.1f} evaluations per solve, "
              f"{s_per_eval:.3f} s per evaluation")
    return {
        "impl": "reference",
        "metric": METRIC,
        "value": v,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": wall / len(res) * 1e3,
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded wall + solute problems, see config)",
        "config": config(N, {"parallelism": f"one single-threaded solve per core, {workers} "
                                            f"concurrent (the reference has no threading)",
                             "per_step_s": [round(x, 2) for x in secs],
                             "per_step_evals": evals,
                             "wall_s_all_steps": wall,
                             "value_vs_ms_per_step": "value is the mean time of one "
                             "single-threaded solve (the metric's latency); ms_per_step is the "
                             "wall time of all timed steps over their count, the solves "
                             "running concurrently"}),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": workers, "kind": "port",
                         "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def kernel_case(precision, N, problem="slit", evals=3, tuning=None):
    """A small fixed case for kernel profiling: `evals` energy+gradient
    evaluations (and, in the mixed form, one Hessian-vector product) of the
    N^3 hard-wall slit (dx = 0.2, eta = 0.3) or of the first timed held-out
    wall + solute problem, about 0.5 GB on the device at 128^3; per-kernel
    event times of the evaluations are returned."""
    import torch
    from deft_gb300 import _lib
    from deft_gb300.workloads import Slit
    from deft_gb300 import autotune
    L = _lib.load()
    autotune.load(tuning) if tuning else autotune.load()
    s = Slit(N=N, dx=0.2, eta=0.3, seed=1) if problem == "slit" else held_out(N, 4)[3]
    h = ctypes.c_void_p()
    _lib.check(L.deft_ctx_create(0, ctypes.byref(h)))
    ctx = h
    lat = np.ascontiguousarray(s.lat.reshape(9))
    h = ctypes.c_void_p()
    _lib.check(L.deft_grid_create(ctx, lat.ctypes.data, *s.shape, ctypes.byref(h)))
    grid = h
    p = _lib.FmtParams(1.0, 1.0, s.mu, _lib.TERM_HS | _lib.TERM_IDEAL | _lib.TERM_MU |
                       _lib.TERM_MASK, precision)
    h = ctypes.c_void_p()
    _lib.check(L.deft_fmt_create(grid, ctypes.byref(p), ctypes.byref(h)))
    f = h
    mask = torch.tensor(s.mask.reshape(-1), device="cuda:0")
    _lib.check(L.deft_fmt_set_mask(f, mask.data_ptr(), 1))
    n = torch.tensor(s.n0.reshape(-1), device="cuda:0")
    g = torch.empty_like(n)
    E = ctypes.c_double()
    for _ in range(evals):
        _lib.check(L.deft_fmt_energy_grad(f, n.data_ptr(), 1, ctypes.addressof(E), g.data_ptr(),
                                          None))
    if precision == _lib.PRECISION_MIXED:
        _lib.check(L.deft_fmt_hessian_vector(f, n.data_ptr(), g.data_ptr(), 1, g.data_ptr()))
    # host wall time of one synchronous call (graph replay, energy read back)
    reps = 20
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        _lib.check(L.deft_fmt_energy_grad(f, n.data_ptr(), 1, ctypes.addressof(E), g.data_ptr(),
                                          None))
    wall_eval = (time.perf_counter() - t0) / reps
    _lib.check(L.deft_grid_profile(grid, 1))
    for _ in range(evals):
        _lib.check(L.deft_fmt_energy_grad(f, n.data_ptr(), 1, ctypes.addressof(E), g.data_ptr(),
                                          None))
    prof = kernel_profile(L, grid)
    hvp = {}
    if precision == _lib.PRECISION_MIXED:
        # the Newton refinement's Hessian-vector products
        hv = torch.empty_like(n)
        _lib.check(L.deft_grid_profile(grid, 1))
        for _ in range(evals):
            _lib.check(L.deft_fmt_hessian_vector(f, n.data_ptr(), g.data_ptr(), 1, hv.data_ptr()))
        hvp = kernel_profile(L, grid)
    torch.cuda.synchronize()
    L.deft_fmt_destroy(f)
    L.deft_grid_destroy(grid)
    L.deft_ctx_destroy(ctx)
    out = {"kernel_case": "mixed" if precision else "fp64", "problem": problem, "N": N,
           "evals": evals, "energy": E.value,
           "wall_us_per_eval_call": round(1e6 * wall_eval, 1),
           "kernel_us_per_eval": round(1e3 * sum(v[1] for v in prof.values()) / evals, 1),
           "us_per_launch": {k: round(1e3 * v[1] / v[0], 2) for k, v in prof.items()}}
    if hvp:
        out["hvp_kernel_us_per_product"] = round(1e3 * sum(v[1] for v in hvp.values()) / evals, 1)
        out["hvp_us_per_launch"] = {k: round(1e3 * v[1] / v[0], 2) for k, v in hvp.items()}
    return out


def fno_case(N=128, reps=5):
    """The warm-start network's forward pass at the timed configuration
    (N^3 grid, 16 channels, 12 modes, 4 Fourier layers; seeded random
    weights): `reps` passes of deft_fno_warm_start on a slit mask, each
    timed on the host around a device synchronisation."""
    import torch
    from deft_gb300 import _lib
    from deft_gb300.warmstart import FourierOperator
    L = _lib.load()
    net = FourierOperator(N, 16, 12, 4, seed=TRAIN_SEED, device=0)
    z = np.arange(N) * 0.2
    mask1 = ((z > 0) & (z < 0.35 * N * 0.2)).astype(np.float64)
    mask = torch.tensor(np.broadcast_to(mask1, (N, N, N)).reshape(-1).copy(), device="cuda:0")
    n = torch.empty_like(mask)
    nb = 0.3 / (4 * math.pi / 3)
    times = []
    try:
        for k in range(reps + 2):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            _lib.check(L.deft_fno_warm_start(net.h, mask.data_ptr(), 0.3, nb, 1e-3, n.data_ptr()))
            torch.cuda.synchronize()
            if k >= 2:
                times.append(time.perf_counter() - t0)
        launches = int(L.deft_fno_launches(net.h))
    finally:
        net.close()
    return {"fno_case": {"N": N, "channels": 16, "modes": 12, "layers": 4},
            "ms_per_forward": round(1e3 * statistics.median(times), 3),
            "launches_per_forward": launches // (reps + 2)}


def pc_case(N=128, reps=20):
    """The structure preconditioner (DEFT_PC_STRUCTURE) applied to a
    gradient-sized vector on a held-out N^3 wall + solute problem at its bulk
    start: `reps` applications through deft_fmt_precondition on device
    buffers (FP64 vectors, FP32 transforms), timed with CUDA events on the
    library's stream after warm-up; per-application kernel events from the
    grid's profile."""
    import torch
    from deft_gb300 import _lib
    from deft_gb300.warmstart import Solver
    L = _lib.load()
    s = held_out(N, 1)[0]
    sv = Solver(s.shape, s.lat, device=0, gtol=GTOL)
    try:
        mask = torch.tensor(s.mask.reshape(-1), device="cuda:0")
        sv.set_problem(s, mask.data_ptr())
        h = sv.fmt[_lib.PRECISION_MIXED]
        n = torch.tensor(s.n0.reshape(-1), device="cuda:0")
        r = torch.randn(n.numel(), dtype=torch.float64, device="cuda:0",
                        generator=torch.Generator(device="cuda:0").manual_seed(1)) * mask
        z = torch.empty_like(n)
        stream = torch.cuda.ExternalStream(L.deft_ctx_stream(sv.ctx), device="cuda:0")
        nb = ctypes.c_double()
        for _ in range(3):
            _lib.check(L.deft_fmt_precondition(h, n.data_ptr(), r.data_ptr(), 1, z.data_ptr(),
                                               ctypes.addressof(nb)))
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            _lib.check(L.deft_fmt_precondition(h, n.data_ptr(), r.data_ptr(), 1, z.data_ptr(),
                                               None))
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        _lib.check(L.deft_grid_profile(sv.grid, 1))
        _lib.check(L.deft_fmt_precondition(h, n.data_ptr(), r.data_ptr(), 1, z.data_ptr(), None))
        prof = kernel_profile(L, sv.grid)
        _lib.check(L.deft_grid_profile(sv.grid, 0))
    finally:
        sv.close()
    return {"pc_case": {"N": N, "eta": s.eta, "bulk_density": nb.value},
            "us_per_application": round(1e3 * ms, 2),
            "kernels_us": {k: round(1e3 * v[1] / v[0], 2) for k, v in prof.items()},
            "launches": {k: v[0] for k, v in prof.items()}}


def solute_case(N=256, reps=5):
    """The hard-sphere solute workload at 256^3 (dx = 0.1, eta = 0.35, centre
    exclusion radius 3, smoothed-noise start with seed 2;
    papers/contact/figs/sphere.cpp:90-105 geometry): plain FP64 solve and the
    mixed solve (FP32 CG stage with the density preconditioner, Newton
    refinement on the FP64 gradient), both from the same start and timed
    with CUDA events, and the mixed form's errors against FP64: one
    evaluation at the start (free energy, gradient) and the converged
    profile against the FP64 solution converged to |grad F| < 1e-12."""
    import torch
    from deft_gb300 import _lib
    from deft_gb300.warmstart import Solver
    from deft_gb300.workloads import Solute
    s = Solute(N=N, dx=0.1, eta=0.35, r_excl=3.0, seed=2)
    dd = "cuda:0"
    mask = torch.tensor(s.mask.reshape(-1), device=dd)
    n0 = torch.tensor(s.n0.reshape(-1), device=dd)
    sv = Solver(s.shape, s.lat, device=0, gtol=GTOL)
    stream = torch.cuda.ExternalStream(sv.L.deft_ctx_stream(sv.ctx), device=dd)
    MIXED, FP64 = _lib.PRECISION_MIXED, _lib.PRECISION_FP64
    L = sv.L
    try:
        sv.set_problem(s, mask.data_ptr())
        # one evaluation at the start in both forms
        E = {}
        g = {}
        for prec in (FP64, MIXED):
            e = ctypes.c_double()
            g[prec] = torch.empty_like(n0)
            _lib.check(L.deft_fmt_energy_grad(sv.fmt[prec], n0.data_ptr(), 1, ctypes.addressof(e),
                                              g[prec].data_ptr(), None))
            E[prec] = e.value
        eval_err = {"dF_rel": abs(E[MIXED] / E[FP64] - 1),
                    "max_dg_rel_to_max_g": float((g[MIXED] - g[FP64]).abs().max()
                                                 / g[FP64].abs().max())}
        # the FP64 solution to 1e-12 (the profile reference)
        st, _ = sv.solve(FP64, n0.data_ptr(), preconditioned=_lib.PC_DENSITY, gtol=REF_GTOL)
        if not (st.converged and st.gnorm < REF_GTOL):
            raise RuntimeError("FP64 reference solve did not converge")
        x_ref = torch.empty_like(n0)
        _lib.check(L.deft_cg_get_x(sv.cg[FP64], x_ref.data_ptr(), 1))
        x = torch.empty_like(n0)

        def timed(prec, pc, gtol):
            times, sts = [], []
            for k in range(reps + 1):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                st, _ = sv.solve(prec, n0.data_ptr(), preconditioned=pc, gtol=gtol)
                e1.record(stream)
                e1.synchronize()
                if k:
                    times.append(e0.elapsed_time(e1) / 1e3)
                    sts.append(st)
            if not all(t.converged and t.status == 0 and t.gnorm < gtol for t in sts):
                raise RuntimeError("solute solve did not converge")
            _lib.check(L.deft_cg_get_x(sv.cg[prec], x.data_ptr(), 1))
            d = float((x - x_ref).abs().max())
            st = sts[-1]
            return {"seconds": statistics.median(times), "iters": st.iter, "evals": st.evals,
                    "evals_fp64": st.evals_fp64, "hvps": st.hvps, "gnorm": st.gnorm,
                    "max_abs_dn_vs_fp64_solution": d,
                    "max_dn_rel_to_max_n": d / float(x_ref.abs().max())}

        fp64 = timed(FP64, _lib.PC_NONE, GTOL)
        fp64_pc = timed(FP64, _lib.PC_DENSITY, GTOL)
        mixed = timed(MIXED, _lib.PC_DENSITY, MIXED_GTOL_PC["density"])
    finally:
        sv.close()
    return {"solute_case": f"White Bear + ideal gas + mu, {N}^3 periodic, dx = 0.1, eta = 0.35, "
                           "hard-sphere solute (centre exclusion radius 3, n = 0 and frozen "
                           "inside), smoothed-noise start (seed 2)",
            "fp64_plain": fp64, "fp64_density_preconditioned": fp64_pc, "mixed": mixed,
            "speedup_mixed_vs_fp64_plain": fp64["seconds"] / mixed["seconds"],
            "mixed_single_evaluation_errors": eval_err,
            "timing": f"median of {reps} solves from the start, CUDA events"}


def saft_case(N=128, dx=0.2, evals=10, gtol=1e-11):
    """The water SAFT workload (WaterSaft with hughes_water_prop,
    src/water-constants.cpp:22-40; atomic units): N^3 grid of spacing dx bohr,
    liquid density 4.9388942e-3 bohr^-3 around a hard-sphere solute whose
    centre-exclusion radius is 3 Angstrom = 5.669 bohr (the density inside it
    floored at 1e-5 of the liquid's), mu of the homogeneous liquid.  In the
    FP64 form and in the mixed form (every transform in FP32, refinement by
    FP64 CG): energy+gradient evaluations timed with CUDA events, the mixed
    evaluation's errors against FP64, and one converged solve each
    (density-preconditioned CG to |grad F| < gtol) with the two profiles
    compared."""
    import torch
    from deft_gb300 import _lib
    L = _lib.load()
    kB, ang = 3.16681539628059e-6, 1.8897261
    R, kT, nl = 3.03420 * ang / 2, 298.15 * kB, 4.9388942e-3
    sp = np.array([1400.0 * kB, 0.0381876 * (3.03420 * ang) ** 3, 250.0 * kB, 1.78890, 0.353])
    terms = _lib.TERM_HS | _lib.TERM_IDEAL | _lib.TERM_MU | _lib.TERM_SAFT

    def fmt(grid, mu, mask=None, precision=0):
        h = ctypes.c_void_p()
        p = _lib.FmtParams(R, kT, mu, terms | (_lib.TERM_MASK if mask is not None else 0),
                           precision, 0)
        _lib.check(L.deft_fmt_create(grid, ctypes.byref(p), ctypes.byref(h)))
        _lib.check(L.deft_fmt_set_saft(h, sp.ctypes.data))
        if mask is not None:
            _lib.check(L.deft_fmt_set_mask(h, mask.data_ptr(), 1))
        return h

    h = ctypes.c_void_p()
    _lib.check(L.deft_ctx_create(0, ctypes.byref(h)))
    ctx = h
    # chemical potential of the homogeneous liquid: -dF/dN on a small cell
    cell = 8 * dx
    lat8 = np.ascontiguousarray(np.diag([cell] * 3).reshape(9))
    h = ctypes.c_void_p()
    _lib.check(L.deft_grid_create(ctx, lat8.ctypes.data, 8, 8, 8, ctypes.byref(h)))
    g8 = h
    f8 = fmt(g8, 0.0)
    E = ctypes.c_double()
    dn = 1e-7 * nl
    Es = []
    for v in (nl + dn, nl - dn):
        u = np.full(512, v)
        _lib.check(L.deft_fmt_energy(f8, u.ctypes.data, 0, ctypes.addressof(E), None))
        Es.append(E.value)
    mu = -(Es[0] - Es[1]) / (2 * dn * cell ** 3)
    L.deft_fmt_destroy(f8)
    L.deft_grid_destroy(g8)
    lat = np.ascontiguousarray(np.diag([N * dx] * 3).reshape(9))
    h = ctypes.c_void_p()
    _lib.check(L.deft_grid_create(ctx, lat.ctypes.data, N, N, N, ctypes.byref(h)))
    grid = h
    x = (np.arange(N) - N / 2) * dx
    r = np.sqrt(x[:, None, None] ** 2 + x[None, :, None] ** 2 + x[None, None, :] ** 2)
    mask_h = (r > 3 * ang).astype(np.float64).reshape(-1)
    mask = torch.tensor(mask_h, device="cuda:0")
    n0 = torch.tensor(np.where(mask_h > 0, nl, 1e-5 * nl), device="cuda:0")
    stream = torch.cuda.ExternalStream(L.deft_ctx_stream(ctx))
    out = {}
    res = {}
    for prec, name in ((0, "fp64"), (1, "mixed")):
        f = fmt(grid, mu, mask, prec)
        gbuf = torch.empty_like(n0)
        for _ in range(3):
            _lib.check(L.deft_fmt_energy_grad(f, n0.data_ptr(), 1, ctypes.addressof(E),
                                              gbuf.data_ptr(), None))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(evals):
            _lib.check(L.deft_fmt_energy_grad(f, n0.data_ptr(), 1, ctypes.addressof(E),
                                              gbuf.data_ptr(), None))
        e1.record(stream)
        e1.synchronize()
        ms_eval = e0.elapsed_time(e1) / evals
        E0 = E.value
        cp = _lib.CgParams(_lib.LS_SECANT, gtol, 20000, 1.0, 0.0, 0.0, _lib.PC_DENSITY, 0.0)
        h = ctypes.c_void_p()
        _lib.check(L.deft_cg_create(f, ctypes.byref(cp), ctypes.byref(h)))
        cg = h
        _lib.check(L.deft_cg_set_x(cg, n0.data_ptr(), 1))
        st = _lib.CgStatus()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        code = L.deft_cg_solve(cg, ctypes.byref(st))
        torch.cuda.synchronize()
        t_solve = time.perf_counter() - t0
        xs = torch.empty_like(n0)
        _lib.check(L.deft_cg_get_x(cg, xs.data_ptr(), 1))
        res[name] = (E0, gbuf.clone(), xs)
        L.deft_cg_destroy(cg)
        L.deft_fmt_destroy(f)
        out[name] = {"ms_per_energy_grad": ms_eval,
                     "solve": {"status": code, "converged": bool(st.converged),
                               "seconds": t_solve, "iters": st.iter, "evals": st.evals,
                               "evals_fp64": st.evals_fp64, "gnorm": st.gnorm, "gtol": gtol,
                               "energy_hartree": st.energy}}
    L.deft_grid_destroy(grid)
    L.deft_ctx_destroy(ctx)
    (Ed, gd, xd), (Em, gm, xm) = res["fp64"], res["mixed"]
    out["mixed"]["evaluation_errors_vs_fp64"] = {
        "dF_rel": abs(Em / Ed - 1),
        "max_dg_rel_to_max_g": float((gm - gd).abs().max() / gd.abs().max())}
    out["mixed"]["profile_vs_fp64_solve"] = float((xm - xd).abs().max() / xd.abs().max())
    return {"saft_case": "water SAFT (WaterSaft, hughes_water_prop), hard-sphere solute "
                         "of exclusion radius 3 Angstrom in liquid water; FP64 and mixed "
                         "(transforms in FP32, refinement by FP64 CG)",
            "N": N, "dx_bohr": dx, "mu_hartree": mu, **out,
            "speedup_mixed_vs_fp64_solve": out["fp64"]["solve"]["seconds"]
            / out["mixed"]["solve"]["seconds"]}

def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--N", type=int, default=128)
    ap.add_argument("--weights", default=None,
                    help="warm-start network weight file (default: the bundled 2000-solve "
                         "network when present), or 'train' to train one in the run on "
                         "--train-count solves")
    ap.add_argument("--train-count", type=int, default=256)
    ap.add_argument("--train-epochs", type=int, default=2)
    ap.add_argument("--train-workers", type=int, default=8,
                    help="concurrent streams generating the training solves")
    ap.add_argument("--tuning", default=None,
                    help="tuning file to register instead of the bundled one")
    ap.add_argument("--no-precond", action="store_true",
                    help="mixed solve without a preconditioner")
    ap.add_argument("--pc", choices=("density", "structure"), default="structure",
                    help="preconditioner of the warm-started mixed solve: the density-variable "
                         "diagonal or the bulk structure-factor one (DEFT_PC_STRUCTURE)")
    ap.add_argument("--gtol-mixed", type=float, default=None,
                    help="stop test |grad F| of the timed mixed solves (default 3e-10 with the "
                         "structure preconditioner, 5e-10 otherwise)")
    ap.add_argument("--switch", type=float, default=None,
                    help="FP32-stage exit as a fraction of the bulk start's gradient norm "
                         "(default 1e-5 with the preconditioner, 1e-4 without)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip cuFFT and batched sweep")
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--verbose", action="store_true")
    ap.add_argument("--kernel-case", default=None, choices=["mixed", "fp64"],
                    help="only run the small kernel-profiling case and exit")
    ap.add_argument("--case-problem", default="slit", choices=["slit", "solutes"])
    ap.add_argument("--saft-case", action="store_true",
                    help="only time the water SAFT workload (FP64) and exit")
    ap.add_argument("--device-driven", action="store_true",
                    help="run the timed mixed solves device-driven (deft_cg_solve_device, one "
                         "graph launch each) instead of host-driven (deft_cg_solve)")
    ap.add_argument("--solute-case", action="store_true",
                    help="only run the 256^3 hard-sphere solute workload (FP64 vs mixed) and exit")
    ap.add_argument("--fno-case", action="store_true",
                    help="only time the warm-start network's forward pass and exit")
    ap.add_argument("--pc-case", action="store_true",
                    help="only time the structure preconditioner's application and exit")
    args = ap.parse_args()
    if args.weights is None:
        args.weights = BUNDLED_WEIGHTS if os.path.exists(BUNDLED_WEIGHTS) else "train"
    if args.saft_case:
        print(json.dumps(saft_case(args.N)))
        return
    if args.solute_case:
        print(json.dumps(solute_case()))
        return
    if args.fno_case:
        print(json.dumps(fno_case(args.N)))
        return
    if args.pc_case:
        print(json.dumps(pc_case(args.N)))
        return
    if args.kernel_case:
        print(json.dumps(kernel_case(1 if args.kernel_case == "mixed" else 0, args.N,
                                     args.case_problem, tuning=args.tuning)))
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1 and args.impl == "ours":
        import torch.distributed as dist
        dist.init_process_group("nccl")
    if args.impl == "reference":
        res = run_reference(args, rank, world)
    else:
        res = run_ours(args, rank, world)
    if rank == 0 and res is not None:
        print(json.dumps(res))
    if world > 1 and args.impl == "ours":
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
