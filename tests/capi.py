"""Thin test-side helpers that call the C ABI (include/deft_gb300.h) directly
through ctypes with numpy buffers."""
import ctypes

import numpy as np

from deft_gb300 import _lib
from deft_gb300._lib import check


class Ctx:
    def __init__(self, device=0):
        self.L = _lib.load()
        h = ctypes.c_void_p()
        check(self.L.deft_ctx_create(device, ctypes.byref(h)))
        self.h = h

    def close(self):
        self.L.deft_ctx_destroy(self.h)


class Grid:
    def __init__(self, ctx, lat, N):
        self.L = ctx.L
        self.N = tuple(int(v) for v in N)
        self.size = int(np.prod(self.N))
        lat9 = np.ascontiguousarray(np.asarray(lat, dtype=np.float64).reshape(9))
        h = ctypes.c_void_p()
        check(self.L.deft_grid_create(ctx.h, lat9.ctypes.data, *self.N, ctypes.byref(h)))
        self.h = h

    def fft(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = np.empty((self.N[0], self.N[1], self.N[2] // 2 + 1), dtype=np.complex128)
        check(self.L.deft_grid_fft(self.h, x.ctypes.data, out.ctypes.data, 0))
        return out

    def ifft(self, c):
        c = np.ascontiguousarray(c, dtype=np.complex128)
        out = np.empty(self.N)
        check(self.L.deft_grid_ifft(self.h, c.ctypes.data, out.ctypes.data, 0))
        return out

    def info(self):
        dV = ctypes.c_double()
        vol = ctypes.c_double()
        sb = ctypes.c_double()
        check(self.L.deft_grid_info(self.h, None, ctypes.addressof(dV), ctypes.addressof(vol),
                                    ctypes.addressof(sb)))
        return dV.value, vol.value, sb.value

    def close(self):
        self.L.deft_grid_destroy(self.h)


class Fmt:
    def __init__(self, grid, R=1.0, kT=1.0, mu=0.0, terms=7, V=None, mask=None, precision=0,
                 functional=0):
        self.L = grid.L
        self.grid = grid
        p = _lib.FmtParams(R, kT, mu, terms, precision, functional)
        h = ctypes.c_void_p()
        check(self.L.deft_fmt_create(grid.h, ctypes.byref(p), ctypes.byref(h)))
        self.h = h
        if V is not None:
            V = np.ascontiguousarray(V, dtype=np.float64)
            check(self.L.deft_fmt_set_vext(h, V.ctypes.data, 0))
        if mask is not None:
            m = np.ascontiguousarray(mask, dtype=np.float64)
            check(self.L.deft_fmt_set_mask(h, m.ctypes.data, 0))

    def energy(self, n):
        n = np.ascontiguousarray(n, dtype=np.float64)
        E = ctypes.c_double()
        t = np.zeros(_lib.NTERMS)
        check(self.L.deft_fmt_energy(self.h, n.ctypes.data, 0, ctypes.addressof(E), t.ctypes.data))
        return E.value, t

    def energy_grad(self, n):
        n = np.ascontiguousarray(n, dtype=np.float64)
        E = ctypes.c_double()
        t = np.zeros(_lib.NTERMS)
        g = np.empty(self.grid.size)
        check(self.L.deft_fmt_energy_grad(self.h, n.ctypes.data, 0, ctypes.addressof(E),
                                          g.ctypes.data, t.ctypes.data))
        return E.value, g, t

    def energy_grad_pgrad(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        E = ctypes.c_double()
        g = np.empty(self.grid.size)
        pg = np.empty(self.grid.size)
        check(self.L.deft_fmt_energy_grad_pgrad(self.h, x.ctypes.data, 0, ctypes.addressof(E),
                                                g.ctypes.data, pg.ctypes.data, None))
        return E.value, g, pg

    def hessian_vector(self, n, dx):
        n = np.ascontiguousarray(n, dtype=np.float64)
        dx = np.ascontiguousarray(dx, dtype=np.float64)
        out = np.empty(self.grid.size)
        check(self.L.deft_fmt_hessian_vector(self.h, n.ctypes.data, dx.ctypes.data, 0,
                                             out.ctypes.data))
        return out

    def weighted(self, n):
        n = np.ascontiguousarray(n, dtype=np.float64)
        out = np.empty(5 * self.grid.size)
        check(self.L.deft_fmt_weighted(self.h, n.ctypes.data, 0, out.ctypes.data))
        return out.reshape(5, -1)

    def close(self):
        self.L.deft_fmt_destroy(self.h)


class CG:
    def __init__(self, fmt, linesearch=_lib.LS_SECANT, gtol=1e-9, maxiter=0, step=1.0,
                 precision=0.0, refine_rel=0.0, preconditioned=0, refine_abs=0.0,
                 relative_precision=0.0, miniter=0, device_loops=0):
        self.L = fmt.L
        self.size = fmt.grid.size
        p = _lib.CgParams(linesearch, gtol, maxiter, step, precision, refine_rel, preconditioned,
                          refine_abs, relative_precision, miniter, device_loops)
        h = ctypes.c_void_p()
        check(self.L.deft_cg_create(fmt.h, ctypes.byref(p), ctypes.byref(h)))
        self.h = h
        self.st = _lib.CgStatus()

    def set_x(self, n):
        n = np.ascontiguousarray(n, dtype=np.float64)
        check(self.L.deft_cg_set_x(self.h, n.ctypes.data, 0))

    def get_x(self):
        out = np.empty(self.size)
        check(self.L.deft_cg_get_x(self.h, out.ctypes.data, 0))
        return out

    def step(self):
        s = self.L.deft_cg_step(self.h, ctypes.byref(self.st))
        return s, self.st

    def solve(self):
        s = self.L.deft_cg_solve(self.h, ctypes.byref(self.st))
        return s, self.st

    def solve_device(self):
        s = self.L.deft_cg_solve_device(self.h, ctypes.byref(self.st))
        return s, self.st

    def close(self):
        self.L.deft_cg_destroy(self.h)


def batch_solve(problems, precision=0, workers=4, gtol=1e-9, device=0, preconditioned=0,
                device_driven=False):
    """Runs deft_batch_solve (or, device_driven, deft_batch_solve_device with
    the density preconditioner, or the structure one when asked) on
    workloads.Slit-like problems (host
    arrays); returns (status code, list of CgStatus, list of converged
    profiles)."""
    keep = []
    arr = (_lib.BatchProblem * len(problems))()
    outs = []
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
    st = (_lib.CgStatus * len(problems))()
    if device_driven:
        pc = preconditioned if preconditioned == _lib.PC_STRUCTURE else _lib.PC_DENSITY
        cp = _lib.CgParams(_lib.LS_SECANT, gtol, 20000, 1.0, 0.0, 0.0, pc)
        code = _lib.load().deft_batch_solve_device(device, len(problems), arr, ctypes.byref(cp),
                                                   st)
    else:
        bp = _lib.BatchParams(workers, _lib.CgParams(_lib.LS_SECANT, gtol, 20000, 1.0, 0.0, 0.0,
                                                     preconditioned))
        code = _lib.load().deft_batch_solve(device, len(problems), arr, ctypes.byref(bp), st)
    return code, list(st), outs
