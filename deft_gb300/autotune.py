"""Autotuner for the evaluator's launch shapes and FFT radix orders.

For one grid shape and precision it times the kernels of an energy+gradient
evaluation (and, for the mixed form, of a Hessian-vector product) with the
engine's per-kernel CUDA-event accounting (deft_grid_profile), then picks,
one parameter at a time, the tile width that minimises the time of the
kernels that parameter shapes, and after that the radix order of each axis.
Choices change results only by rounding.

Results are cached in a JSON file keyed by GPU name, grid shape and
precision; ``load`` registers a file's entries for the current GPU with
``deft_tuning_set``, so every grid created afterwards (including the grids
of ``deft_batch_solve``) starts from them.

    python -m deft_gb300.autotune --N 32 48 64 96 128 --out tuning.json
"""
import ctypes
import itertools
import json
import os
import time

import numpy as np

from . import _lib
from ._lib import check

PARAMS = ("By", "Bx", "Bxf", "Bxc", "Pz", "Pphi")
# kernels each tile width shapes (names of deft_grid_profile_entry)
KERNELS = {
    "By": ("y_fft_1field", "y_fft_5fields"),
    "Bx": ("x_fft",),
    "Bxf": ("x_conv_fwd",),
    "Bxc": ("x_conv_adj",),
    "Pz": ("z_r2c", "z_grad", "z_hvp_out"),
    "Pphi": ("z_phi_grad", "z_phi_energy", "z_hess", "z_jac"),
}
# tile widths that shape each axis's transforms (x, y, z)
AXIS_PARAMS = (("Bxf", "Bxc"), ("By",), ("Pz", "Pphi"))
AXIS_KERNELS = (
    ("x_fft", "x_conv_fwd", "x_conv_adj"),
    ("y_fft_1field", "y_fft_5fields"),
    ("z_r2c", "z_phi_grad", "z_phi_energy", "z_grad", "z_hess", "z_jac", "z_hvp_out"),
)
# tile widths tried per parameter (those that do not fit in shared memory are
# refused by deft_grid_set_tiles and skipped)
CANDIDATES = tuple(range(1, 17)) + (20, 24, 28, 32, 40, 48, 64)
BUNDLED = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning_gb300.json")


def radix_orders(n, limit=12):
    """Orderings of factorizations of n into the hand-written radices."""
    out = set()

    def rec(m, acc):
        if len(out) > 200:
            return
        if m == 1:
            out.add(tuple(acc))
            return
        for r in (8, 4, 2, 3, 5):
            if m % r == 0 and len(acc) < 8:
                rec(m // r, acc + [r])

    rec(n, [])
    if not out:
        return []
    # prefer few passes, then all orderings of those multisets
    fewest = min(len(o) for o in out)
    cands = sorted({p for o in out if len(o) <= fewest + 1
                    for p in itertools.permutations(o)}, key=lambda o: (len(o), o))
    return [list(o) for o in cands[:limit]]


def _device_name(device):
    import torch
    return torch.cuda.get_device_name(device)


class _Bench:
    """A grid with a slit problem of the given shape and precision."""

    def __init__(self, shape, precision, device=0):
        import torch
        from .workloads import Slit
        L = self.L = _lib.load()
        self.precision = precision
        if shape[0] != shape[1]:
            raise ValueError("shapes other than (M, M, N) are not tuned by this driver")
        s = Slit(N=shape[2], dx=0.2, eta=0.3, seed=1, Nxy=shape[0])
        h = ctypes.c_void_p()
        check(L.deft_ctx_create(device, ctypes.byref(h)))
        self.ctx = h
        lat9 = np.ascontiguousarray(s.lat.reshape(9))
        h = ctypes.c_void_p()
        check(L.deft_grid_create(self.ctx, lat9.ctypes.data, *shape, ctypes.byref(h)))
        self.grid = h
        terms = _lib.TERM_HS | _lib.TERM_IDEAL | _lib.TERM_MU | _lib.TERM_MASK
        p = _lib.FmtParams(s.R, s.kT, s.mu, terms, precision)
        h = ctypes.c_void_p()
        check(L.deft_fmt_create(self.grid, ctypes.byref(p), ctypes.byref(h)))
        self.fmt = h
        dev = f"cuda:{device}"
        self.mask = torch.tensor(s.mask.reshape(-1), device=dev)
        check(L.deft_fmt_set_mask(self.fmt, self.mask.data_ptr(), 1))
        self.n = torch.tensor(s.n0.reshape(-1), device=dev)
        self.g = torch.empty_like(self.n)
        self.dx = torch.tensor(0.01 * s.nb * s.mask.reshape(-1), device=dev)

    def tiles(self):
        t = np.zeros(6, dtype=np.int32)
        r = np.zeros(24, dtype=np.int32)
        check(self.L.deft_grid_get_tiles(self.grid, self.precision, t.ctypes.data, r.ctypes.data))
        return t, r

    def set(self, t, r):
        t = np.ascontiguousarray(t, dtype=np.int32)
        r = np.ascontiguousarray(r, dtype=np.int32)
        return self.L.deft_grid_set_tiles(self.grid, self.precision, t.ctypes.data,
                                          r.ctypes.data) == 0

    def measure(self, repeats):
        """Per-kernel milliseconds summed over `repeats` workloads."""
        L = self.L
        E = ctypes.c_double()
        for _ in range(1):  # warm-up
            check(L.deft_fmt_energy_grad(self.fmt, self.n.data_ptr(), 1, ctypes.addressof(E),
                                         self.g.data_ptr(), None))
        check(L.deft_grid_profile(self.grid, 1))
        for _ in range(repeats):
            check(L.deft_fmt_energy_grad(self.fmt, self.n.data_ptr(), 1, ctypes.addressof(E),
                                         self.g.data_ptr(), None))
            if self.precision == _lib.PRECISION_MIXED:
                check(L.deft_fmt_hessian_vector(self.fmt, self.n.data_ptr(), self.dx.data_ptr(),
                                                1, self.g.data_ptr()))
        out = {}
        name = ctypes.c_char_p()
        launches = ctypes.c_longlong()
        tot = ctypes.c_double()
        for i in range(L.deft_grid_profile_count(self.grid)):
            check(L.deft_grid_profile_entry(self.grid, i, ctypes.byref(name),
                                            ctypes.addressof(launches), ctypes.addressof(tot)))
            nm = name.value.decode()
            # FP32 launches carry "_f32" in the engine's accounting
            if launches.value and nm.endswith("_f32") == (self.precision == _lib.PRECISION_MIXED):
                out[nm[:-4] if nm.endswith("_f32") else nm] = tot.value
        check(L.deft_grid_profile(self.grid, 0))
        return out

    def close(self):
        self.L.deft_fmt_destroy(self.fmt)
        self.L.deft_grid_destroy(self.grid)
        self.L.deft_ctx_destroy(self.ctx)


def tune(shape, precision=_lib.PRECISION_MIXED, device=0, repeats=4, trials=2, log=None):
    """Returns the tuned entry for one shape and precision."""
    b = _Bench(shape, precision, device)
    try:
        t0 = time.perf_counter()
        tiles, radix = b.tiles()
        base_t, base_r = tiles.copy(), radix.copy()

        def cost(kernels):
            best = None
            for _ in range(trials):
                m = b.measure(repeats)
                v = sum(m.get(k, 0.0) for k in kernels)
                best = v if best is None else min(best, v)
            return best

        before = b.measure(repeats)
        for pi, p in enumerate(PARAMS):
            if p == "Bx":
                continue  # plain x FFTs only serve deft_grid_fft / ifft
            kern = KERNELS[p]
            best_v, best_c = int(tiles[pi]), cost(kern)
            for v in CANDIDATES:
                if v == best_v:
                    continue
                cand = tiles.copy()
                cand[pi] = v
                if not b.set(cand, radix):
                    continue
                c = cost(kern)
                if c < best_c * 0.98:
                    best_v, best_c = v, c
            tiles[pi] = best_v
            b.set(tiles, radix)
            if log:
                log(f"{shape} prec {precision}: {p} = {best_v} ({best_c / repeats:.4f} ms)")
        N = shape
        for a in range(3):
            orders = radix_orders(N[a])
            if precision == _lib.PRECISION_MIXED and N[a] in (32, 64, 128, 256):
                orders = [[16, N[a] // 16]] + orders  # register-resident transform
            if len(orders) < 2:
                continue
            cur = [int(v) for v in radix[8 * a:8 * a + 8] if v]
            best_o, best_c = cur, cost(AXIS_KERNELS[a])
            for o in orders:
                if o == cur:
                    continue
                cand = radix.copy()
                cand[8 * a:8 * a + 8] = 0
                cand[8 * a:8 * a + len(o)] = o
                if not b.set(tiles, cand):
                    continue
                c = cost(AXIS_KERNELS[a])
                if c < best_c * 0.98:
                    best_o, best_c = o, c
            radix[8 * a:8 * a + 8] = 0
            radix[8 * a:8 * a + len(best_o)] = best_o
            b.set(tiles, radix)
            if log:
                log(f"{shape} prec {precision}: axis {a} radix {best_o}")
        if precision == _lib.PRECISION_MIXED:
            # The register-resident transform (M = N/16 threads a line) fills
            # a block only with enough lines per tile, which the Stockham
            # tiles chosen above need not give: try it jointly with a sweep
            # of that axis's tile widths.
            for a in range(3):
                if N[a] not in (32, 64, 128, 256):
                    continue
                reg = [16, N[a] // 16]
                cur = [int(v) for v in radix[8 * a:8 * a + 8] if v]
                if cur == reg:
                    continue
                cand_r = radix.copy()
                cand_r[8 * a:8 * a + 8] = 0
                cand_r[8 * a:8 * a + 2] = reg
                base_c = cost(AXIS_KERNELS[a])
                cand_t = tiles.copy()
                for p in AXIS_PARAMS[a]:
                    pi = PARAMS.index(p)
                    best_v, best_pc = None, None
                    for v in CANDIDATES:
                        t2 = cand_t.copy()
                        t2[pi] = v
                        if not b.set(t2, cand_r):
                            continue
                        c = cost(KERNELS[p])
                        if best_pc is None or c < best_pc:
                            best_v, best_pc = v, c
                    if best_v is not None:
                        cand_t[pi] = best_v
                if b.set(cand_t, cand_r) and cost(AXIS_KERNELS[a]) < base_c * 0.98:
                    tiles, radix = cand_t, cand_r
                    if log:
                        log(f"{shape} prec {precision}: axis {a} register transform, tiles "
                            f"{[int(v) for v in tiles]}")
                b.set(tiles, radix)
        after = b.measure(repeats)
        return {
            "N": list(shape), "precision": int(precision),
            "tiles": [int(v) for v in tiles], "radix": [int(v) for v in radix],
            "default_tiles": [int(v) for v in base_t], "default_radix": [int(v) for v in base_r],
            "ms_per_workload_before": sum(before.values()) / repeats,
            "ms_per_workload_after": sum(after.values()) / repeats,
            "kernels_before_ms": {k: v / repeats for k, v in before.items()},
            "kernels_after_ms": {k: v / repeats for k, v in after.items()},
            "workload": "one energy+gradient" + (" and one Hessian-vector product"
                                                 if precision == _lib.PRECISION_MIXED else ""),
            "tuning_s": time.perf_counter() - t0,
        }
    finally:
        b.close()


def save(entries, path, device=0):
    name = _device_name(device)
    data = {"format": "deft_gb300 tuning", "entries": []}
    if os.path.exists(path):
        with open(path) as f:
            data = json.load(f)
    keep = [e for e in data["entries"]
            if not any(e["device"] == name and e["N"] == n["N"] and e["precision"] == n["precision"]
                       for n in entries)]
    data["entries"] = keep + [dict(e, device=name) for e in entries]
    with open(path, "w") as f:
        json.dump(data, f, indent=1)


def load(path=BUNDLED, device=0):
    """Registers the file's entries for this GPU; returns how many."""
    if not os.path.exists(path):
        return 0
    with open(path) as f:
        data = json.load(f)
    name = _device_name(device)
    L = _lib.load()
    k = 0
    for e in data.get("entries", []):
        if e.get("device") != name:
            continue
        N = np.array(e["N"], dtype=np.int32)
        t = np.array(e["tiles"], dtype=np.int32)
        r = np.array(e["radix"], dtype=np.int32)
        check(L.deft_tuning_set(N.ctypes.data, int(e["precision"]), t.ctypes.data, r.ctypes.data))
        k += 1
    return k


def main(argv=None):
    import argparse
    import sys
    ap = argparse.ArgumentParser(description="tune launch shapes and radix orders")
    ap.add_argument("--N", type=int, nargs="+", default=[32, 48, 64, 96, 128])
    ap.add_argument("--precision", nargs="+", default=["mixed", "fp64"],
                    choices=["mixed", "fp64"])
    ap.add_argument("--out", default=BUNDLED)
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args(argv)
    prec = {"mixed": _lib.PRECISION_MIXED, "fp64": _lib.PRECISION_FP64}
    entries = []
    for p in a.precision:
        for N in a.N:
            e = tune((N, N, N), prec[p], a.device,
                     log=lambda m: print(m, file=sys.stderr, flush=True))
            entries.append(e)
            print(json.dumps({k: e[k] for k in ("N", "precision", "tiles", "ms_per_workload_before",
                                                "ms_per_workload_after")}), flush=True)
    save(entries, a.out, a.device)
    return entries


if __name__ == "__main__":
    main()
