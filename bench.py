"""Benchmark: converged FMT solve at 128^3 on one GB300.

Workload (named in the JSON line's config): White Bear hard spheres R = 1,
kT = 1, ideal gas + mu at bulk packing eta = 0.3, periodic 128^3 grid with
dx = 0.2 (edge 25.6), hard walls (n = 0, frozen by the constraint mask)
outside the slit 0 < z < 12.8, initial density bulk x (1 + 0.05 smoothed
seeded noise).  One step = one converged solve: CG with the derivative
line search from the device-resident initial density to |grad F|_2 < 1e-9.

Our arm (default): FP64 evaluator + CG on the GPU; value = seconds per
converged solve (lower is better).  Also reported: per-kernel event timings
(roofline of the dominant kernel and the whole-evaluation "conv HBM GB/s"),
the same solve end to end through the C ABI with host buffers, and a CPU
baseline (the oracle port, one core, on a bounded sample).

--impl reference: the reference's CPU path (the plain-C restatement of it,
since the reference sources are not present where this runs), bounded
sample per step, scaled to the same metric.
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

METRIC = "converged-solve s at 128^3 (mixed form; plain FP64 GPU beside it), |grad F|<1e-9"
UNIT = "s"
GTOL = 1e-9
# Energy+gradient evaluations one converged FP64 solve of this workload takes
# with the derivative-line-search CG (118 at 128^3, measured on GB300 with
# seed 1; the same algorithm on the CPU takes the same count).  The reference
# arm scales its per-evaluation time by it.
SOLVE_EVALS = {128: 118}
HBM_FALLBACK_GBS = 6800.0


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return HBM_FALLBACK_GBS, "fallback"


def workload(N):
    from deft_gb300.workloads import Slit
    return Slit(N=N, dx=0.2, eta=0.3, seed=1)


def config(N, extra=None):
    c = {
        "workload": f"White Bear FMT hard-wall slit, {N}^3, dx=0.2, eta=0.3, R=1, kT=1, "
                    f"CG (secant line search) to |grad F|<1e-9 from seeded noisy bulk",
        "grid": [N, N, N],
        "dx": 0.2,
        "eta": 0.3,
        "gtol": GTOL,
        "l2": "working set (~0.2 GB of fields per solve) larger than the 129 MB L2; "
              "each evaluation streams every field",
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
                 "--format=csv,noheader,nounits", "-lms", "200"],
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

def alg_bytes(N, fp32):
    """Algorithmic bytes per launch of each kernel: the compulsory field reads
    and writes of the stage (nothing for the analytic weights).  Real fields
    at the boundary (n, mask, gradient) are FP64 (R = 8 N^3); spectra are
    C = 16 N^2 (N/2+1) in the FP64 form and 8 N^2 (N/2+1) in the mixed form."""
    NR = N ** 3
    NC = N * N * (N // 2 + 1)
    R, C = 8 * NR, (8 if fp32 else 16) * NC
    return {
        "z_r2c": R + C,
        "y_fft_1field": 2 * C,
        "y_fft_5fields": 10 * C,
        "x_conv_fwd": C + 5 * C,
        "z_phi_grad": 5 * C + R + 5 * C,
        "z_phi_energy": 5 * C + R,
        "x_conv_adj": 5 * C + C,
        "z_grad": C + 3 * R,
        "z_hess": 5 * C + R + 44 * NR,
        "z_jac": 5 * C + 40 * NR + 5 * C,
        "z_hvp_out": C + 4 * NR + 3 * R,
        "eval_model": 4 * R + 24 * C,  # one energy+gradient evaluation
    }


CONV_KERNELS = ("z_r2c", "y_fft_1field", "y_fft_5fields", "x_conv_fwd", "z_phi_grad",
                "z_phi_energy", "x_conv_adj", "z_grad")


def run_ours(args, rank, world):
    import torch
    from deft_gb300 import _lib
    from tests.capi import CG, Ctx, Fmt, Grid

    L = _lib.load()
    N = args.N
    s = workload(N)
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    ctx = Ctx(dev)
    g = Grid(ctx, s.lat, s.shape)
    terms = _lib.TERM_HS | _lib.TERM_IDEAL | _lib.TERM_MU | _lib.TERM_MASK
    n0_dev = torch.tensor(s.n0.reshape(-1), dtype=torch.float64, device=f"cuda:{dev}")
    torch.cuda.synchronize()
    stream = torch.cuda.ExternalStream(L.deft_ctx_stream(ctx.h), device=f"cuda:{dev}")
    peak, peak_kind = measured_peaks()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    def timed(precision):
        f = Fmt(g, R=s.R, kT=s.kT, mu=s.mu, terms=terms, mask=s.mask.reshape(-1),
                precision=precision)
        cg = CG(f, linesearch=_lib.LS_SECANT, gtol=GTOL, maxiter=20000, step=1.0)

        def solve():
            _lib.check(L.deft_cg_set_x(cg.h, n0_dev.data_ptr(), 1))
            st = _lib.CgStatus()
            _lib.check(L.deft_cg_solve(cg.h, ctypes.byref(st)))
            return st

        for _ in range(args.warmup):
            st = solve()
        if not (st.converged and st.gnorm < GTOL):
            raise RuntimeError(f"warm-up solve did not converge: {st.gnorm}")
        _lib.check(L.deft_grid_profile(g.h, 1))
        clocks = Clocks(dev)
        clocks.start()
        barrier()
        torch.cuda.synchronize()
        _lib.check(L.deft_ctx_sync(ctx.h))
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        stats = [solve() for _ in range(args.steps)]
        e1.record(stream)
        e1.synchronize()
        torch.cuda.synchronize()
        barrier()
        ck = clocks.stop()
        ms = e0.elapsed_time(e1)
        if world > 1:
            import torch.distributed as dist
            t = torch.tensor([ms], device=f"cuda:{dev}")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        prof = {}
        name = ctypes.c_char_p()
        launches = ctypes.c_longlong()
        tot = ctypes.c_double()
        for i in range(L.deft_grid_profile_count(g.h)):
            _lib.check(L.deft_grid_profile_entry(g.h, i, ctypes.byref(name),
                                                 ctypes.addressof(launches), ctypes.addressof(tot)))
            if launches.value:
                prof[name.value.decode()] = (launches.value, tot.value)
        _lib.check(L.deft_grid_profile(g.h, 0))
        return f, cg, ms / args.steps, stats, prof, ck

    def kernel_table(prof):
        total = sum(v[1] for v in prof.values())
        return {k: {"launches": v[0], "ms_total": round(v[1], 3), "share": round(v[1] / total, 4)}
                for k, v in sorted(prof.items(), key=lambda kv: -kv[1][1])}

    def roofline(prof, fp32):
        ab = alg_bytes(N, fp32)
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
        return {
            "bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": traffic, "alg_bytes_per_launch": ab[dom],
            "avg_launch_ms": dom_ms,
            "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
            else "fallback 6.8 TB/s",
            "conv_hbm_gbs": conv_gbs, "conv_frac": conv_gbs / peak if conv_gbs else None,
        }

    f64, cg64, ms64, st64, prof64, ck64 = timed(_lib.PRECISION_FP64)
    fmx, cgmx, msmx, stmx, profmx, ckmx = timed(_lib.PRECISION_MIXED)
    avg = lambda sts, k: sum(getattr(x, k) for x in sts) / len(sts)  # noqa: E731

    # end to end through the C ABI with host buffers: mask + initial density
    # in, converged profile out, every step (mixed form, the headline)
    n0_host = torch.tensor(s.n0.reshape(-1), dtype=torch.float64).pin_memory()
    mask_host = torch.tensor(s.mask.reshape(-1), dtype=torch.float64).pin_memory()
    out_host = torch.empty(s.size, dtype=torch.float64).pin_memory()
    K2 = max(1, min(args.steps, 3))
    t0 = time.perf_counter()
    for _ in range(K2):
        _lib.check(L.deft_fmt_set_mask(fmx.h, mask_host.data_ptr(), 0))
        _lib.check(L.deft_cg_set_x(cgmx.h, n0_host.data_ptr(), 0))
        st = _lib.CgStatus()
        _lib.check(L.deft_cg_solve(cgmx.h, ctypes.byref(st)))
        _lib.check(L.deft_cg_get_x(cgmx.h, out_host.data_ptr(), 0))
    e2e_s = (time.perf_counter() - t0) / K2
    e2e = {"value": e2e_s, "unit": UNIT, "h2d_bytes_per_step": 2 * 8 * s.size,
           "d2h_bytes_per_step": 8 * s.size,
           "api": "C ABI: deft_fmt_set_mask + deft_cg_set_x + deft_cg_solve + deft_cg_get_x "
                  "with pinned host buffers (mixed form)"}

    result = {
        "metric": METRIC,
        "value": msmx / 1e3,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": msmx,
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 FFT/phi + f64 reductions and refinement",
        "data": "synthetic (seeded smoothed-noise slit, see config)",
        "config": config(N, {
            "parallelism": "replicas only" if world > 1 else "single GPU",
            "form": "mixed: FP32 CG stage, then Newton refinement on the FP64 gradient",
            "mixed": {"solve_s": msmx / 1e3, "iters": avg(stmx, "iter"),
                      "evals": avg(stmx, "evals"), "evals_fp64": avg(stmx, "evals_fp64"),
                      "hvps": avg(stmx, "hvps"), "final_gnorm_fp64": stmx[-1].gnorm},
            "fp64": {"solve_s": ms64 / 1e3, "iters": avg(st64, "iter"),
                     "evals": avg(st64, "evals"), "final_gnorm": st64[-1].gnorm},
            "speedup_mixed_vs_fp64": ms64 / msmx,
        }),
        "e2e": e2e,
        "gpu_launches": sum(v[0] for v in profmx.values()),
        "clocks": ckmx,
        "roofline": roofline(profmx, True),
        "roofline_fp64": dict(roofline(prof64, False),
                              note="FP64 form: bound by the FP64 pipe (measured 1.0 TFLOP/s "
                                   "FMA on this GB300), not by HBM"),
        "clocks_fp64": ck64,
        "kernels": kernel_table(profmx),
        "kernels_fp64": kernel_table(prof64),
    }
    if not args.no_sweep:
        result["batched_sweep"] = batched_sweep()
    if rank == 0 and world == 1 and not args.no_cpu:
        result["cpu_baseline"] = cpu_baseline(N, avg(st64, "evals"), budget_s=args.cpu_budget)
    for obj in (cg64, cgmx, f64, fmx):
        obj.close()
    g.close()
    ctx.close()
    return result


def batched_sweep(count=64, seed=3):
    """The batched sweep (64 slits, eta in [0.05, 0.45], grids from
    {32,48,64,96,128}^3, dx = 0.2, slit widths 3-10): mixed form, solved by
    deft_batch_solve with 8 concurrent streams, against the same problems one
    after another on one stream."""
    from deft_gb300.workloads import batch_sweep
    from tests.capi import batch_solve
    probs = batch_sweep(count=count, seed=seed)
    batch_solve(probs[:8], precision=1, workers=8)  # warm-up: plans and tables
    t0 = time.perf_counter()
    code, st, _ = batch_solve(probs, precision=1, workers=8)
    t_conc = time.perf_counter() - t0
    t0 = time.perf_counter()
    code1, _, _ = batch_solve(probs, precision=1, workers=1)
    t_seq = time.perf_counter() - t0
    conv = sum(1 for x in st if x.converged and x.gnorm < GTOL)
    return {"problems": count, "converged": conv, "status": code or code1,
            "seconds_8_streams": t_conc, "seconds_1_stream": t_seq,
            "solves_per_s": count / t_conc, "grid_points": int(sum(p.size for p in probs)),
            "form": "mixed (FP32 CG stage + FP64-residual Newton refinement), |grad F|<1e-9"}


def cpu_eval_seconds(N, budget_s, max_evals=8):
    """Seconds per energy+gradient evaluation of the oracle port at N^3,
    timed on up to max_evals evaluations within about budget_s."""
    from oracle import oracle as O
    O.build()
    s = workload(N)
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


def cpu_baseline(N, evals_per_solve, budget_s=20.0):
    sec, k = cpu_eval_seconds(N, budget_s)
    return {"value": sec * evals_per_solve, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{k} energy+gradient evaluations of the {N}^3 slit by the oracle port "
                      f"({sec:.3f} s each, 1 thread), scaled by the {evals_per_solve:.0f} "
                      f"evaluations the converged solve takes with the same CG"}


# ---------------------------------------------------------------------------
# reference arm

def run_reference(args, rank, world):
    if rank != 0:
        return None
    N = args.N
    evals = SOLVE_EVALS.get(N, 118)
    for _ in range(args.warmup):
        cpu_eval_seconds(N, budget_s=0.0, max_evals=1)
    samples = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        sec, _k = cpu_eval_seconds(N, budget_s=0.0, max_evals=1)
        samples.append(sec * evals)
    wall = time.perf_counter() - t0
    v = sum(samples) / len(samples)
    return {
        "impl": "reference",
        "metric": METRIC,
        "value": v,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": wall / args.steps * 1e3,
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded smoothed-noise slit, see config)",
        "config": config(N, {"parallelism": "single thread (the reference has no threading)"}),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": 1, "kind": "port",
                         "sample": f"per step: one energy+gradient evaluation of the {N}^3 slit "
                                   f"by the oracle port (plain-C restatement of the reference "
                                   f"path), scaled by the {evals} evaluations of a converged "
                                   f"solve"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--N", type=int, default=128)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-sweep", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1 and args.impl == "ours":
        import torch.distributed as dist
        dist.init_process_group("nccl" if args.impl == "ours" else "gloo")
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
