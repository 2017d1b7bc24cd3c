"""ctypes bindings for the oracle -- TEST INFRASTRUCTURE ONLY.

Two CPU libraries live under oracle/:

* ``liboracle.so`` -- the plain-C restatement of the FMT + CG hot path
  (``deft_oracle.c``), built everywhere by ``make -C oracle liboracle``;
* ``_ref/libdeft_ref.so`` -- the unmodified reference sources plus the
  project's FFTW3-API shim, built only where the reference checkout exists
  (``make -C oracle ref``).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline /
reference arm may import this module, as the checker.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libdeft_ref.so")

HS, IDEAL, MU, VEXT, MASK, VEFF = 1, 2, 4, 8, 16, 32
HS_WB, HS_RF, HS_M2, HS_WBT, HS_TZ = 0, 1, 2, 3, 4  # hard-sphere kinds (oracle_params.hs)
# contact fields (oracle_contact)
CONTACT_GSIGMA_S, CONTACT_GSIGMA_A, CONTACT_GROSS, CONTACT_YUWU, CONTACT_YUWU_S = 0, 1, 2, 3, 4
NTERMS = 6
TERM_NAMES = ("phi3", "phi1", "phi2", "ideal_gas", "chemical_potential", "external_potential")

_dp = ctypes.POINTER(ctypes.c_double)


def _ptr(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


class _Params(ctypes.Structure):
    _fields_ = [
        ("Nx", ctypes.c_int), ("Ny", ctypes.c_int), ("Nz", ctypes.c_int),
        ("lat", ctypes.c_double * 9),
        ("R", ctypes.c_double), ("kT", ctypes.c_double), ("mu", ctypes.c_double),
        ("terms", ctypes.c_int), ("hs", ctypes.c_int),
        ("saft_on", ctypes.c_int), ("saft", ctypes.c_double * 5),
    ]


def build(ref=False):
    """Compile liboracle.so (and, if ref and the checkout exists, the reference)."""
    import subprocess
    targets = ["liboracle"]
    if ref:
        targets.append("ref")
    subprocess.check_call(["make", "-s", "-C", HERE] + targets)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build()
        L = ctypes.CDLL(ORACLE_SO)
        P = ctypes.POINTER(_Params)
        L.oracle_dvolume.restype = ctypes.c_double
        L.oracle_dvolume.argtypes = [P]
        L.oracle_weighted.argtypes = [P, _dp, _dp]
        L.oracle_energy.restype = ctypes.c_double
        L.oracle_energy.argtypes = [P, _dp, _dp, _dp, _dp]
        L.oracle_energy_grad.restype = ctypes.c_double
        L.oracle_energy_grad.argtypes = [P, _dp, _dp, _dp, _dp, _dp]
        L.oracle_find_mu.restype = ctypes.c_double
        L.oracle_find_mu.argtypes = [ctypes.c_double] * 3
        L.oracle_homogeneous.restype = ctypes.c_double
        L.oracle_homogeneous.argtypes = [ctypes.c_double] * 4
        L.oracle_cg_quadratic.restype = ctypes.c_int
        L.oracle_cg_quadratic.argtypes = [P, _dp, _dp, _dp, ctypes.c_int, ctypes.c_double, _dp]
        L.oracle_cg_solve.restype = ctypes.c_int
        L.oracle_cg_solve.argtypes = [P, _dp, _dp, _dp, ctypes.c_double, ctypes.c_int,
                                      ctypes.c_double, _dp]
        L.oracle_cg_solve_pc.restype = ctypes.c_int
        L.oracle_cg_solve_pc.argtypes = [P, _dp, _dp, _dp, ctypes.c_double, ctypes.c_int,
                                         ctypes.c_double, ctypes.c_int, _dp]
        L.oracle_energy_grad_pgrad.restype = ctypes.c_double
        L.oracle_energy_grad_pgrad.argtypes = [P, _dp, _dp, _dp, _dp, _dp, _dp]
        L.oracle_pcg_quadratic.restype = ctypes.c_int
        L.oracle_pcg_quadratic.argtypes = [P, _dp, _dp, _dp, ctypes.c_int, ctypes.c_double, _dp]
        L.oracle_fft_count.restype = ctypes.c_longlong
        L.oracle_contact.argtypes = [P, _dp, ctypes.c_int, _dp]
        L.oracle_new_minimize.restype = ctypes.c_int
        L.oracle_new_minimize.argtypes = [P, _dp, _dp, _dp, ctypes.c_int, ctypes.c_double,
                                          ctypes.c_double, _dp]
        L.oracle_saft.restype = ctypes.c_double
        L.oracle_saft.argtypes = [P, _dp, _dp, _dp, _dp]
        L.offt_r2c_3d.argtypes = [ctypes.c_int] * 3 + [_dp, _dp]
        L.offt_c2r_3d.argtypes = [ctypes.c_int] * 3 + [_dp, _dp]
        _lib = L
    return _lib


def ref_available():
    return os.path.exists(REF_SO)


def ref():
    """The unmodified reference build (only where it was compiled)."""
    global _ref
    if _ref is None:
        L = ctypes.CDLL(REF_SO)
        L.ref_eval.restype = ctypes.c_int
        L.ref_eval.argtypes = [_dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                               ctypes.c_double, ctypes.c_double, ctypes.c_int, _dp, _dp, _dp,
                               _dp, _dp, _dp]
        L.ref_weighted.argtypes = [_dp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_double, _dp, _dp]
        L.ref_find_mu.restype = ctypes.c_double
        L.ref_find_mu.argtypes = [ctypes.c_double] * 3
        L.ref_homogeneous.restype = ctypes.c_double
        L.ref_homogeneous.argtypes = [ctypes.c_double] * 4
        L.ref_cg.restype = ctypes.c_int
        L.ref_cg.argtypes = [_dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                             ctypes.c_double, ctypes.c_double, ctypes.c_int, _dp, _dp, _dp,
                             ctypes.c_int, ctypes.c_double, _dp]
        L.ref_fd_test.restype = ctypes.c_int
        L.ref_fd_test.argtypes = [_dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                  ctypes.c_double, ctypes.c_double, ctypes.c_int, _dp, _dp]
        L.ref_eval_veff.argtypes = [_dp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_int, _dp, _dp, _dp, _dp, _dp, _dp]
        L.ref_pcg.restype = ctypes.c_int
        L.ref_pcg.argtypes = [_dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                              ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int, _dp,
                              _dp, _dp, ctypes.c_int, ctypes.c_double, _dp]
        L.ref_pcg_precision.restype = ctypes.c_int
        L.ref_pcg_precision.argtypes = [_dp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, ctypes.c_int,
                                        ctypes.c_double, ctypes.c_double, _dp]
        L.ref_fft_count.restype = ctypes.c_longlong
        L.ref_set_hs.argtypes = [ctypes.c_int]
        L.ref_new_minimize.restype = ctypes.c_int
        L.ref_new_minimize.argtypes = ([_dp] + [ctypes.c_int] * 3 + [ctypes.c_double] * 3 +
                                       [ctypes.c_int, _dp, _dp, _dp, ctypes.c_int, ctypes.c_double,
                                        ctypes.c_double, _dp])
        L.ref_saft.restype = ctypes.c_double
        L.ref_saft.argtypes = [_dp] + [ctypes.c_int] * 3 + [ctypes.c_double] * 8 + [_dp, _dp, _dp]
        L.ref_contact.argtypes = [_dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                  ctypes.c_int, _dp, _dp]
        _ref = L
    return _ref


class Problem:
    """One evaluation setting: lattice (rows a1, a2, a3), grid, R, kT, mu, terms."""

    def __init__(self, lat, N, R=1.0, kT=1.0, mu=0.0, terms=HS | IDEAL | MU, V=None, mask=None,
                 hs=0, saft=None):
        self.hs = int(hs)  # HS_WB, HS_RF, HS_M2, HS_WBT or HS_TZ
        # water SAFT terms: (eps_a, kappa_a, eps_d, lambda_d, length_scaling) or None
        self.saft_params = None if saft is None else tuple(float(v) for v in saft)
        self.lat = np.ascontiguousarray(np.asarray(lat, dtype=np.float64).reshape(9))
        self.N = tuple(int(v) for v in N)
        self.R, self.kT, self.mu, self.terms = float(R), float(kT), float(mu), int(terms)
        self.V = None if V is None else np.ascontiguousarray(V, dtype=np.float64).reshape(-1)
        self.mask = None if mask is None else np.ascontiguousarray(mask, dtype=np.float64).reshape(-1)
        if self.V is not None:
            self.terms |= VEXT
        if self.mask is not None:
            self.terms |= MASK

    @property
    def size(self):
        return self.N[0] * self.N[1] * self.N[2]

    def params(self):
        p = _Params()
        p.Nx, p.Ny, p.Nz = self.N
        for i in range(9):
            p.lat[i] = self.lat[i]
        p.R, p.kT, p.mu, p.terms, p.hs = self.R, self.kT, self.mu, self.terms, self.hs
        if self.saft_params is not None:
            p.saft_on = 1
            for i, v in enumerate(self.saft_params):
                p.saft[i] = v
        return p

    # -- restatement -------------------------------------------------------
    def dvolume(self):
        return lib().oracle_dvolume(ctypes.byref(self.params()))

    def weighted(self, n):
        n = np.ascontiguousarray(n, dtype=np.float64).reshape(-1)
        out = np.empty(5 * self.size)
        lib().oracle_weighted(ctypes.byref(self.params()), _ptr(n), _ptr(out))
        return out.reshape(5, -1)

    def energy(self, n, terms=False):
        n = np.ascontiguousarray(n, dtype=np.float64).reshape(-1)
        t = np.zeros(NTERMS)
        E = lib().oracle_energy(ctypes.byref(self.params()), _ptr(n), _ptr(self.V),
                                _ptr(self.mask), _ptr(t))
        return (E, t) if terms else E

    def energy_grad(self, n, terms=False):
        n = np.ascontiguousarray(n, dtype=np.float64).reshape(-1)
        g = np.empty(self.size)
        t = np.zeros(NTERMS)
        E = lib().oracle_energy_grad(ctypes.byref(self.params()), _ptr(n), _ptr(self.V),
                                     _ptr(self.mask), _ptr(g), _ptr(t))
        return (E, g, t) if terms else (E, g)

    def energy_grad_pgrad(self, x):
        """Energy, gradient and preconditioned gradient at the variable x
        (the effective potential when VEFF is in terms)."""
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1)
        g = np.empty(self.size)
        pg = np.empty(self.size)
        E = lib().oracle_energy_grad_pgrad(ctypes.byref(self.params()), _ptr(x), _ptr(self.V),
                                           _ptr(self.mask), _ptr(g), _ptr(pg), None)
        return E, g, pg

    def pcg_quadratic(self, x, iters, step=0.1):
        x = np.array(x, dtype=np.float64).reshape(-1)
        e = np.zeros(iters)
        k = lib().oracle_pcg_quadratic(ctypes.byref(self.params()), _ptr(self.V), _ptr(self.mask),
                                       _ptr(x), iters, step, _ptr(e))
        return x, e[:k]

    def cg_quadratic(self, n, iters, step=0.1):
        x = np.array(n, dtype=np.float64).reshape(-1)
        e = np.zeros(iters)
        k = lib().oracle_cg_quadratic(ctypes.byref(self.params()), _ptr(self.V), _ptr(self.mask),
                                      _ptr(x), iters, step, _ptr(e))
        return x, e[:k]

    def cg_solve(self, n, gtol=1e-9, maxiter=10000, step=1.0, preconditioned=False):
        x = np.array(n, dtype=np.float64).reshape(-1)
        out = np.zeros(3)
        it = lib().oracle_cg_solve_pc(ctypes.byref(self.params()), _ptr(self.V), _ptr(self.mask),
                                      _ptr(x), gtol, maxiter, step, int(preconditioned),
                                      _ptr(out))
        return x, {"iters": it, "energy": out[0], "gnorm": out[1], "evals": int(out[2])}

    def new_minimize(self, x, iters, precision=0.0, relative_precision=1e-15):
        """The restated "new" API Minimize from x: (x after, energies)."""
        x = np.array(x, dtype=np.float64).reshape(-1)
        e = np.zeros(iters)
        k = lib().oracle_new_minimize(ctypes.byref(self.params()), _ptr(self.V), _ptr(self.mask),
                                      _ptr(x), iters, precision, relative_precision, _ptr(e))
        return x, e[:k]

    def saft(self, n, saft_params, grad=True):
        """Water SAFT association + dispersion energy and (unmasked) gradient
        at n; saft_params = (eps_a, kappa_a, eps_d, lambda_d, length_scaling)."""
        n = np.ascontiguousarray(n, dtype=np.float64).reshape(-1)
        sp = np.ascontiguousarray(saft_params, dtype=np.float64)
        g = np.empty(self.size) if grad else None
        out2 = np.zeros(2)
        E = lib().oracle_saft(ctypes.byref(self.params()), _ptr(sp), _ptr(n), _ptr(g), _ptr(out2))
        return E, g, out2

    def contact(self, n, which):
        """Contact field `which` (CONTACT_*) at the density n."""
        n = np.ascontiguousarray(n, dtype=np.float64).reshape(-1)
        out = np.empty(self.size)
        lib().oracle_contact(ctypes.byref(self.params()), _ptr(n), int(which), _ptr(out))
        return out

    # -- unmodified reference ---------------------------------------------
    def _ref(self):
        """The reference build, set to this problem's hard-sphere functional."""
        L = ref()
        L.ref_set_hs(self.hs)
        return L

    def ref_energy_grad(self, n, grad=True):
        n = np.ascontiguousarray(n, dtype=np.float64).reshape(-1)
        E = ctypes.c_double(0)
        t = np.zeros(8)
        g = np.empty(self.size) if grad else None
        nt = self._ref().ref_eval(_ptr(self.lat), *self.N, self.R, self.kT, self.mu, self.terms,
                            _ptr(n), _ptr(self.V), _ptr(self.mask), ctypes.byref(E), _ptr(t), _ptr(g))
        return E.value, g, t[:nt]

    def ref_saft(self, n, saft_params, grad=True):
        """The reference's WaterSaft (all terms, mu included) energy and
        integralgrad (constrained by this problem's mask)."""
        n = np.ascontiguousarray(n, dtype=np.float64).reshape(-1)
        g = np.empty(self.size) if grad else None
        E = ref().ref_saft(_ptr(self.lat), *self.N, self.R, *[float(v) for v in saft_params],
                           self.mu, self.kT, _ptr(n), _ptr(self.mask), _ptr(g))
        return E, g

    def ref_new_minimize(self, x, iters, precision=0.0, relative_precision=1e-15):
        """The reference's "new" API Minimize (src/new/Minimize.cpp) from x:
        (x after, energies after each improve_energy call)."""
        x = np.array(x, dtype=np.float64).reshape(-1)
        e = np.zeros(iters)
        k = self._ref().ref_new_minimize(_ptr(self.lat), *self.N, self.R, self.kT, self.mu,
                                         self.terms, _ptr(self.V), _ptr(self.mask), _ptr(x), iters,
                                         precision, relative_precision, _ptr(e))
        return x, e[:k]

    def ref_contact(self, n, which):
        n = np.ascontiguousarray(n, dtype=np.float64).reshape(-1)
        out = np.empty(self.size)
        self._ref().ref_contact(_ptr(self.lat), *self.N, self.R, int(which), _ptr(n), _ptr(out))
        return out

    def ref_weighted(self, n):
        n = np.ascontiguousarray(n, dtype=np.float64).reshape(-1)
        out = np.empty(5 * self.size)
        self._ref().ref_weighted(_ptr(self.lat), *self.N, self.R, _ptr(n), _ptr(out))
        return out.reshape(5, -1)

    def ref_eval_veff(self, x):
        """The unmodified reference's constrain(mask, OfEffectivePotential(sum)):
        energy, integralgrad and pgrad at the effective potential x."""
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1)
        E = ctypes.c_double(0)
        g = np.empty(self.size)
        pg = np.empty(self.size)
        self._ref().ref_eval_veff(_ptr(self.lat), *self.N, self.R, self.kT, self.mu, self.terms,
                            _ptr(x), _ptr(self.V), _ptr(self.mask), ctypes.byref(E), _ptr(g),
                            _ptr(pg))
        return E.value, g, pg

    def ref_pcg(self, x, iters, step=0.1):
        x = np.array(x, dtype=np.float64).reshape(-1)
        e = np.zeros(iters)
        k = self._ref().ref_pcg(_ptr(self.lat), *self.N, self.R, self.kT, self.mu, self.terms,
                          int(bool(self.terms & VEFF)), _ptr(self.V), _ptr(self.mask), _ptr(x),
                          iters, step, _ptr(e))
        return x, e[:k]

    def ref_pcg_precision(self, x, iters, step, precision):
        """Precision(precision, PreconditionedConjugateGradient(...)) of the
        reference: (x after, energies after each improve_energy() call, the
        last call being the one that returned false, if any)."""
        x = np.array(x, dtype=np.float64).reshape(-1)
        e = np.zeros(iters)
        k = self._ref().ref_pcg_precision(_ptr(self.lat), *self.N, self.R, self.kT, self.mu,
                                          self.terms, int(bool(self.terms & VEFF)), _ptr(self.V),
                                          _ptr(self.mask), _ptr(x), iters, step, precision,
                                          _ptr(e))
        return x, e[:k]

    def ref_cg(self, n, iters, step=0.1):
        x = np.array(n, dtype=np.float64).reshape(-1)
        e = np.zeros(iters)
        k = self._ref().ref_cg(_ptr(self.lat), *self.N, self.R, self.kT, self.mu, self.terms,
                         _ptr(self.V), _ptr(self.mask), _ptr(x), iters, step, _ptr(e))
        return x, e[:k]


def find_mu(R, kT, nb):
    return lib().oracle_find_mu(R, kT, nb)


def homogeneous(R, kT, mu, nb):
    return lib().oracle_homogeneous(R, kT, mu, nb)


def r2c_3d(x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    Nx, Ny, Nz = x.shape
    out = np.empty((Nx, Ny, Nz // 2 + 1), dtype=np.complex128)
    lib().offt_r2c_3d(Nx, Ny, Nz, _ptr(x), out.ctypes.data_as(_dp))
    return out


def c2r_3d(c, Nz):
    c = np.ascontiguousarray(c, dtype=np.complex128)
    Nx, Ny, _ = c.shape
    out = np.empty((Nx, Ny, Nz))
    lib().offt_c2r_3d(Nx, Ny, Nz, c.ctypes.data_as(_dp), _ptr(out))
    return out
