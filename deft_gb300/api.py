"""Python mirror of deft's Functional / Grid / GridDescription / Minimizer API
over the C ABI (include/deft_gb300.h).

Names, argument meaning and return conventions follow the reference:

* ``Lattice(a1, a2, a3)``                       src/lattice.h:79-113
* ``GridDescription(lat, Nx, Ny, Nz)`` / ``(lat, dx)``  src/GridDescription.cpp:6-48
* ``Grid(gd[, values])``, ``grid(x, y, z)``, ``Set(f)``  src/Grid.h:22-72
* ``HardSpheresWBnotensor(R)``, ``IdealGas()``, ``ChemicalPotential(mu)``,
  ``ExternalPotential(V)``, ``constrain(mask, f)``, ``+``  (src/HardSpheres.cpp,
  src/IdealGas.cpp, src/ChemicalPotential.cpp, src/ExternalPotential.cpp,
  src/Functional.cpp:834-838, src/Functional.h:88-103)
* ``f.integral(kT, grid)``, ``f.integralgrad(kT, gd, x, g)``  src/Functional.h:125-149
* ``OfEffectivePotential(f)``, ``EffectivePotentialToDensity()``
  src/EffectivePotentialToDensity.cpp:20-91
* ``PreconditionedConjugateGradient(f, gd, kT, x, lm, step)``
  src/ConjugateGradient.cpp:115-174
* ``ConjugateGradient(f, gd, kT, x, QuadraticLineMinimizer, step)``,
  ``Precision(eps, m)``, ``MaxIter(n, m)``, ``m.improve_energy()``,
  ``m.energy()``, ``m.grad()``  src/LineMinimizer.h:18-19, src/Minimizer.h:13-60
* ``find_chemical_potential(f, kT, n)``          src/equation-of-state.cpp:189-192
* the "new" API: ``NewFunctional(f, gd, kT, x)``, ``Minimize(newf)`` with
  ``set_precision``, ``set_relative_precision``, ``set_maxiter``,
  ``set_miniter``, ``precondition``, ``improve_energy``  src/new/Minimize.h
* ``WaterSaft(R, epsAB, kappaAB, eps_d, lambda_d, length_scaling, mu)``
  src/OptimizedFunctionals.h:13-15 (src/haskell/WaterSaft.hs)
* ``HardSpheresRF(R)`` src/HardSpheres.cpp:69-88; ``WhiteBearMarkII(R)``
  src/haskell/WhiteBear.hs:140-159; ``HardSpheresWB(R)`` (tensor, also
  ``HardSpheres``) and ``HardSpheresTarazona(R)`` src/HardSpheres.cpp:90-135
* ``gSigmaS(R)``, ``gSigmaA(R)``, ``gSigmaSm2(R)``, ``gSigmaAm2(R)``,
  ``CorrelationGrossCorrect(R)``, ``YuWuCorrelation(R)``,
  ``YuWuCorrelation_S(R)``, each called as ``f(kT, gd, density)``
  (src/ContactDensity.h, papers/contact/figs/walls.cpp:118-129)

Everything is evaluated by the sm_103a kernels; there is no CPU path.  The
functional composition is recognised (White Bear + ideal gas + mu + V_ext,
optionally constrained) and sent to one fused GPU evaluator.
"""
import ctypes
import math

import numpy as np

from . import _lib
from ._lib import check

QuadraticLineMinimizer = "quadratic"   # src/QuadraticLineMinimizer.cpp:207-214
SecantLineMinimizer = "secant"         # derivative search (converges to |grad| ~ 1e-12)


# ---------------------------------------------------------------------------
# Context

class Context:
    """One GPU and one CUDA stream (deft_ctx)."""

    def __init__(self, device=0):
        L = _lib.load()
        h = ctypes.c_void_p()
        check(L.deft_ctx_create(device, ctypes.byref(h)))
        self.handle = h
        self.device = device

    def sync(self):
        check(_lib.load().deft_ctx_sync(self.handle))

    def close(self):
        if self.handle:
            _lib.load().deft_ctx_destroy(self.handle)
            self.handle = None


_default_ctx = None


def default_context():
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


# ---------------------------------------------------------------------------
# Geometry

class Lattice:
    def __init__(self, a1, a2, a3):
        self.R = np.array([a1, a2, a3], dtype=np.float64)  # rows a1, a2, a3

    def a1(self):
        return self.R[0].copy()

    def a2(self):
        return self.R[1].copy()

    def a3(self):
        return self.R[2].copy()

    def volume(self):
        return float(np.linalg.det(self.R.T))

    def flat(self):
        return np.ascontiguousarray(self.R.reshape(9))


def grid_size_from_dx(lat, dx):
    """N_i = 1 + int(e/100 + |a_i|/dx), the rule of GridDescription(lat, dx)
    (src/GridDescription.cpp:27-29)."""
    R = lat.R if isinstance(lat, Lattice) else np.asarray(lat, dtype=np.float64).reshape(3, 3)
    return [1 + int(math.e / 100 + np.linalg.norm(R[i]) / dx) for i in range(3)]


class GridDescription:
    """GridDescription(lat, Nx, Ny, Nz) or GridDescription(lat, dx)."""

    def __init__(self, lat, nx, ny=None, nz=None, ctx=None):
        self.Lat = lat
        if ny is None:
            N = grid_size_from_dx(lat, float(nx))
        else:
            N = [int(nx), int(ny), int(nz)]
        self.Nx, self.Ny, self.Nz = N
        self.NyNz = self.Ny * self.Nz
        self.NxNyNz = self.Nx * self.NyNz
        self.NzOver2 = self.Nz // 2 + 1
        self.NyNzOver2 = self.Ny * self.NzOver2
        self.NxNyNzOver2 = self.Nx * self.NyNzOver2
        self.dx, self.dy, self.dz = 1.0 / self.Nx, 1.0 / self.Ny, 1.0 / self.Nz
        self.ctx = ctx or default_context()
        h = ctypes.c_void_p()
        lat9 = lat.flat()
        check(_lib.load().deft_grid_create(self.ctx.handle, lat9.ctypes.data, self.Nx, self.Ny,
                                           self.Nz, ctypes.byref(h)))
        self.handle = h
        dV = ctypes.c_double()
        vol = ctypes.c_double()
        check(_lib.load().deft_grid_info(h, None, ctypes.addressof(dV), ctypes.addressof(vol), None))
        self.dvolume = dV.value
        self.volume = vol.value

    @property
    def shape(self):
        return (self.Nx, self.Ny, self.Nz)

    def fft(self, v):
        """fft(gd, v): r2c times dV (src/Grid.cpp:470-478)."""
        v = _host_f64(v, self.NxNyNz)
        out = np.empty((self.Nx, self.Ny, self.NzOver2), dtype=np.complex128)
        check(_lib.load().deft_grid_fft(self.handle, v.ctypes.data, out.ctypes.data, 0))
        return out

    def ifft(self, c):
        """ifft(gd, c): c2r times 1/V (src/ReciprocalGrid.cpp:42-66)."""
        c = np.ascontiguousarray(c, dtype=np.complex128)
        assert c.size == self.NxNyNzOver2
        out = np.empty(self.NxNyNz)
        check(_lib.load().deft_grid_ifft(self.handle, c.ctypes.data, out.ctypes.data, 0))
        return out

    def close(self):
        if self.handle:
            _lib.load().deft_grid_destroy(self.handle)
            self.handle = None


def _host_f64(v, n):
    a = np.ascontiguousarray(np.asarray(v, dtype=np.float64).reshape(-1))
    if a.size != n:
        raise ValueError(f"field has {a.size} values, grid has {n}")
    return a


class Grid(np.ndarray):
    """A real field on a GridDescription (row-major x, y, z; src/Grid.h:37-42)."""

    def __new__(cls, gd, values=None):
        if values is None:
            a = np.zeros(gd.NxNyNz)
        else:
            a = np.array(values, dtype=np.float64).reshape(-1).copy()
            if a.size != gd.NxNyNz:
                raise ValueError("size mismatch")
        obj = a.view(cls)
        obj.gd = gd
        return obj

    def __array_finalize__(self, obj):
        self.gd = getattr(obj, "gd", None)

    def description(self):
        return self.gd

    def __call__(self, x, y, z):
        return float(self[(x * self.gd.Ny + y) * self.gd.Nz + z])

    def Set(self, f):
        """Grid::Set (src/Grid.cpp:43-52) without the Wigner-Seitz wrap."""
        gd = self.gd
        for x in range(gd.Nx):
            for y in range(gd.Ny):
                for z in range(gd.Nz):
                    r = gd.Lat.R.T @ np.array([x * gd.dx, y * gd.dy, z * gd.dz])
                    self[(x * gd.Ny + y) * gd.Nz + z] = f(r)

    def integrate(self):
        return float(np.asarray(self).sum() * self.gd.dvolume)


# ---------------------------------------------------------------------------
# Functionals

class Functional:
    """A sum of the recognised terms, optionally wrapped in constrain(mask, .)."""

    def __init__(self, R=None, ideal=False, mu=None, V=None, mask=None, names=(), veff=False,
                 hs=_lib.HS_WB_NOTENSOR, saft=None):
        self.R = R
        self.hs = hs  # hard-sphere kind (White Bear, Rosenfeld, mark II, tensor kinds)
        self.saft = saft  # water SAFT parameters (5 values) or None
        self.ideal = ideal
        self.mu = mu
        self.V = V
        self.mask = mask
        self.veff = veff  # OfEffectivePotential: the variable is Veff, n = exp(-Veff/kT)
        self.names = tuple(names)
        self._fmt = {}
        self.last_energy = {}

    def __add__(self, o):
        if self.mask is not None or o.mask is not None:
            raise NotImplementedError("add terms before constrain()")
        if self.veff or o.veff:
            raise NotImplementedError("add terms inside OfEffectivePotential()")
        def pick(a, b, what):
            if a is not None and b is not None and a is not b:
                raise NotImplementedError(f"two {what} terms")
            return a if a is not None else b
        return Functional(R=pick(self.R, o.R, "hard-sphere"), ideal=self.ideal or o.ideal,
                          mu=pick(self.mu, o.mu, "chemical-potential"),
                          V=pick(self.V, o.V, "external-potential"),
                          names=self.names + o.names,
                          hs=self.hs if self.R is not None else o.hs,
                          saft=pick(self.saft, o.saft, "SAFT"))

    def terms(self):
        t = 0
        if self.R is not None:
            t |= _lib.TERM_HS
        if self.ideal:
            t |= _lib.TERM_IDEAL
        if self.mu is not None:
            t |= _lib.TERM_MU
        if self.V is not None:
            t |= _lib.TERM_VEXT
        if self.mask is not None:
            t |= _lib.TERM_MASK
        if self.veff:
            t |= _lib.TERM_VEFF
        if self.saft is not None:
            t |= _lib.TERM_SAFT
        return t

    def fmt(self, gd, kT):
        """The deft_fmt handle for this grid (created on first use)."""
        key = id(gd)
        L = _lib.load()
        p = _lib.FmtParams(self.R if self.R is not None else 1.0, kT,
                           self.mu if self.mu is not None else 0.0, self.terms(), 0, self.hs)
        if key not in self._fmt:
            h = ctypes.c_void_p()
            check(L.deft_fmt_create(gd.handle, ctypes.byref(p), ctypes.byref(h)))
            if self.V is not None:
                V = _host_f64(self.V, gd.NxNyNz)
                check(L.deft_fmt_set_vext(h, V.ctypes.data, 0))
            if self.mask is not None:
                m = _host_f64(self.mask, gd.NxNyNz)
                check(L.deft_fmt_set_mask(h, m.ctypes.data, 0))
            if self.saft is not None:
                sp = np.ascontiguousarray(self.saft, dtype=np.float64)
                check(L.deft_fmt_set_saft(h, sp.ctypes.data))
            self._fmt[key] = (gd, h)
        else:
            check(L.deft_fmt_set_params(self._fmt[key][1], ctypes.byref(p)))
        return self._fmt[key][1]

    def _gd_data(self, a, b, c):
        # integral(kT, grid) | integral(kT, gd, data) | integral(gd, kT, data)
        if c is None:
            return b.description(), b
        if isinstance(a, GridDescription):
            return a, c
        return b, c

    def integral(self, a, b, c=None):
        kT = a if not isinstance(a, GridDescription) else b
        gd, x = self._gd_data(a, b, c)
        E, terms = self.energy_terms(gd, kT, x)
        return E

    def energy_terms(self, gd, kT, x):
        h = self.fmt(gd, kT)
        x = _host_f64(x, gd.NxNyNz)
        E = ctypes.c_double()
        t = np.zeros(_lib.NTERMS)
        check(_lib.load().deft_fmt_energy(h, x.ctypes.data, 0, ctypes.addressof(E), t.ctypes.data))
        self.last_energy = dict(zip(("phi3", "phi1", "phi2", "ideal_gas", "chemical_potential",
                                     "external_potential"), t))
        return E.value, t

    def integralgrad(self, kT, gd, x=None, g=None, pg=None):
        """Accumulates dF/dx (dV included, mask applied) into g (and pg)."""
        if x is None or isinstance(x, np.ndarray) and g is None:
            # integralgrad(kT, grid, g)
            x, g = gd, x
            gd = x.description()
        h = self.fmt(gd, kT)
        xs = _host_f64(x, gd.NxNyNz)
        out = np.empty(gd.NxNyNz)
        pout = np.empty(gd.NxNyNz) if pg is not None else None
        E = ctypes.c_double()
        check(_lib.load().deft_fmt_energy_grad_pgrad(
            h, xs.ctypes.data, 0, ctypes.addressof(E), out.ctypes.data,
            pout.ctypes.data if pout is not None else None, None))
        g += out.reshape(g.shape)
        if pg is not None:
            pg += pout.reshape(pg.shape)
        return E.value

    def integralpgrad(self, kT, gd, x, pg):
        """Accumulates the preconditioned gradient (src/Functional.h:150-155)."""
        g = np.zeros(gd.NxNyNz)
        return self.integralgrad(kT, gd, x, g, pg)

    def weighted(self, gd, x):
        h = self.fmt(gd, 1.0)
        xs = _host_f64(x, gd.NxNyNz)
        out = np.empty(5 * gd.NxNyNz)
        check(_lib.load().deft_fmt_weighted(h, xs.ctypes.data, 0, out.ctypes.data))
        return out.reshape(5, -1)

    def close(self):
        for gd, h in self._fmt.values():
            _lib.load().deft_fmt_destroy(h)
        self._fmt = {}


def HardSpheresWBnotensor(R):
    return Functional(R=float(R), names=("phi3", "phi1", "phi2"))


def HardSpheresRF(R):
    """Rosenfeld's functional (src/HardSpheres.cpp:69-88)."""
    return Functional(R=float(R), names=("phi3", "phi1", "phi2"), hs=_lib.HS_RF)


def HardSpheresWB(R):
    """White Bear with the tensor third term (src/HardSpheres.cpp:113-135)."""
    return Functional(R=float(R), names=("phi3", "phi1", "phi2"), hs=_lib.HS_WB_TENSOR)


def HardSpheresTarazona(R):
    """Tarazona's tensor functional (src/HardSpheres.cpp:90-111)."""
    return Functional(R=float(R), names=("phi3", "phi1", "phi2"), hs=_lib.HS_TARAZONA)


HardSpheres = HardSpheresWB  # src/HardSpheres.cpp:185-187


# ---------------------------------------------------------------------------
# The "new" API (src/new/NewFunctional.h, src/new/Minimize.h)

class NewFunctional:
    """A functional bound to its input, as the new API's NewFunctional holds
    its data: (f, gd, kT, x); ``data`` is the current x (host array)."""

    def __init__(self, f, gd, kT, x):
        self.f, self.gd, self.kT = f, gd, float(kT)
        self.data = np.array(_host_f64(x, gd.NxNyNz))

    def energy(self):
        return self.f.integral(self.kT, self.gd, self.data)

    def grad(self):
        g = np.zeros(self.gd.NxNyNz)
        self.f.integralgrad(self.kT, self.gd, self.data, g)
        return g


class Minimize:
    """The new API's minimiser (src/new/Minimize.cpp:9-304), run by the C ABI
    (DEFT_LS_NEW_API): set_precision, set_relative_precision, set_maxiter,
    set_miniter, precondition, improve_energy, energy, get_iteration_count.
    The minimiser keeps its own copy of x and writes it back into
    ``newf.data`` after every improve_energy call."""

    def __init__(self, newf):
        self.nf = newf
        self.precision, self.relative_precision = 0.0, 1e-15
        self.maxiter, self.miniter = 10000000, 6
        self.use_preconditioning = False
        self._cg = None
        self._st = _lib.CgStatus()

    def set_precision(self, p):
        self.precision = float(p)
        self._cg = None

    def set_relative_precision(self, p):
        self.relative_precision = float(p)
        self._cg = None

    def set_maxiter(self, n):
        self.maxiter = int(n)
        self._cg = None

    def set_miniter(self, n):
        self.miniter = int(n)
        self._cg = None

    def precondition(self, u):
        self.use_preconditioning = bool(u)
        self._cg = None

    def _make(self):
        L = _lib.load()
        h = self.nf.f.fmt(self.nf.gd, self.nf.kT)
        pc = _lib.PC_FUNCTIONAL if (self.use_preconditioning and self.nf.f.veff) else _lib.PC_NONE
        p = _lib.CgParams(_lib.LS_NEW_API, 0.0, self.maxiter, 0.1, self.precision, 0.0, pc, 0.0,
                          self.relative_precision, self.miniter)
        c = ctypes.c_void_p()
        check(L.deft_cg_create(h, ctypes.byref(p), ctypes.byref(c)))
        check(L.deft_cg_set_x(c, self.nf.data.ctypes.data, 0))
        self._cg = c

    def improve_energy(self, verbose=False):
        if self._cg is None:
            self._make()
        L = _lib.load()
        check(L.deft_cg_step(self._cg, ctypes.byref(self._st)))
        check(L.deft_cg_get_x(self._cg, self.nf.data.ctypes.data, 0))
        if verbose:
            print(f"==== Iteration {self._st.iter} ====  total energy = {self._st.energy:.15g}")
        return not self._st.converged

    def energy(self):
        if self._cg is None:
            return self.nf.energy()
        return self._st.energy

    def get_iteration_count(self):
        return self._st.iter

    def close(self):
        if self._cg is not None:
            _lib.load().deft_cg_destroy(self._cg)
            self._cg = None


def WaterSaft(R, epsilon_association, kappa_association, epsilon_dispersion, lambda_dispersion,
              length_scaling, mu):
    """The water SAFT functional (src/OptimizedFunctionals.h:13-15,
    src/WaterSaftFast.cpp): ideal gas + White Bear + association +
    dispersion + mu N, in the reference's units (kT is the caller's)."""
    return Functional(R=float(R), ideal=True, mu=float(mu),
                      names=("phi3", "phi1", "phi2", "ideal_gas", "chemical_potential"),
                      saft=(float(epsilon_association), float(kappa_association),
                            float(epsilon_dispersion), float(lambda_dispersion),
                            float(length_scaling)))


def WhiteBearMarkII(R):
    """White Bear mark II (src/haskell/WhiteBear.hs:140-159)."""
    return Functional(R=float(R), names=("phi3", "phi1", "phi2"), hs=_lib.HS_WB_MARK2)


class _ContactField:
    """A transformation of the density into a contact field, called as the
    reference's Functional transformations are: f(kT, gd, density) -> Grid
    (papers/contact/figs/walls.cpp:120-129)."""

    def __init__(self, R, which, hs):
        self.f = Functional(R=float(R), hs=hs)
        self.which = which

    def __call__(self, kT, gd, x):
        h = self.f.fmt(gd, kT)
        xs = _host_f64(x, gd.NxNyNz)
        out = Grid(gd)
        check(_lib.load().deft_fmt_contact(h, xs.ctypes.data, 0, self.which, out.ctypes.data))
        return out

    def close(self):
        self.f.close()


def gSigmaS(R):
    return _ContactField(R, _lib.CONTACT_GSIGMA_S, _lib.HS_WB_NOTENSOR)


def gSigmaA(R):
    return _ContactField(R, _lib.CONTACT_GSIGMA_A, _lib.HS_WB_NOTENSOR)


def gSigmaSm2(R):
    return _ContactField(R, _lib.CONTACT_GSIGMA_S, _lib.HS_WB_MARK2)


def gSigmaAm2(R):
    return _ContactField(R, _lib.CONTACT_GSIGMA_A, _lib.HS_WB_MARK2)


def GrossCorrelation(R):
    return _ContactField(R, _lib.CONTACT_GROSS, _lib.HS_WB_NOTENSOR)


CorrelationGrossCorrect = GrossCorrelation


def YuWuCorrelation(R):
    return _ContactField(R, _lib.CONTACT_YUWU, _lib.HS_WB_NOTENSOR)


def YuWuCorrelation_S(R):
    return _ContactField(R, _lib.CONTACT_YUWU_S, _lib.HS_WB_NOTENSOR)


def IdealGas():
    return Functional(ideal=True, names=("ideal_gas",))


def ChemicalPotential(mu):
    return Functional(mu=float(mu), names=("chemical_potential",))


def ExternalPotential(V):
    return Functional(V=np.asarray(V, dtype=np.float64), names=("external potential",))


def constrain(mask, f):
    c = Functional(R=f.R, ideal=f.ideal, mu=f.mu, V=f.V, names=f.names, veff=f.veff)
    c.mask = np.asarray(mask, dtype=np.float64)
    return c


def OfEffectivePotential(f):
    """f of n = exp(-Veff/kT), as a functional of Veff
    (src/EffectivePotentialToDensity.cpp:28-91)."""
    if f.mask is not None:
        raise NotImplementedError("constrain() outside OfEffectivePotential(), as the drivers do")
    return Functional(R=f.R, ideal=f.ideal, mu=f.mu, V=f.V, names=f.names, veff=True)


def EffectivePotentialToDensity():
    """The map Veff -> n = exp(-Veff/kT) (src/EffectivePotentialToDensity.cpp:20-23),
    as a callable (kT, gd, Veff) -> n."""
    def to_density(kT, gd, V):
        return np.exp(-np.asarray(V, dtype=np.float64) / kT)
    return to_density


def find_chemical_potential(f, kT, n):
    """mu with n as the bulk density of f = HS(R) + IdealGas()."""
    if f.R is None or not f.ideal:
        raise NotImplementedError("find_chemical_potential needs HardSpheresWBnotensor + IdealGas")
    mu = ctypes.c_double()
    check(_lib.load().deft_find_chemical_potential(f.R, kT, n, ctypes.addressof(mu)))
    return mu.value


# ---------------------------------------------------------------------------
# Minimisers

class Minimizer:
    """ConjugateGradient(...) wrapped in optional Precision / MaxIter."""

    def __init__(self, f, gd, kT, x, linmin=QuadraticLineMinimizer, step=0.1, precision=0.0,
                 maxiter=0, gtol=0.0, preconditioned=False):
        self.f, self.gd, self.kT, self.x = f, gd, kT, x
        self.linmin, self.step = linmin, step
        self.preconditioned = preconditioned
        self.precision, self.maxiter, self.gtol = precision, maxiter, gtol
        self.handle = None
        self.status = _lib.CgStatus()

    def _make(self):
        if self.handle is not None:
            return
        L = _lib.load()
        p = _lib.CgParams(_lib.LS_SECANT if self.linmin == SecantLineMinimizer else
                          _lib.LS_QUADRATIC_REF, self.gtol, self.maxiter, self.step, self.precision,
                          0.0, int(bool(self.preconditioned)))
        h = ctypes.c_void_p()
        check(L.deft_cg_create(self.f.fmt(self.gd, self.kT), ctypes.byref(p), ctypes.byref(h)))
        self.handle = h
        xs = _host_f64(self.x, self.gd.NxNyNz)
        check(L.deft_cg_set_x(h, xs.ctypes.data, 0))

    def improve_energy(self, verbose=False):
        """One improve_energy() call; False once converged (src/Minimizer.h:44)."""
        self._make()
        s = _lib.load().deft_cg_step(self.handle, ctypes.byref(self.status))
        self._pull()
        if s == _lib.ERR_MAXITER:
            return False
        check(s)
        if verbose:
            print(f"iter {self.status.iter} energy {self.status.energy:.16g} "
                  f"|grad| {self.status.gnorm:g}")
        return not self.status.converged

    def solve(self):
        self._make()
        s = _lib.load().deft_cg_solve(self.handle, ctypes.byref(self.status))
        self._pull()
        check(s)
        return self.status

    def _pull(self):
        out = np.empty(self.gd.NxNyNz)
        check(_lib.load().deft_cg_get_x(self.handle, out.ctypes.data, 0))
        self.x[...] = out.reshape(self.x.shape)

    def energy(self):
        return self.f.integral(self.kT, self.gd, self.x)

    def grad(self):
        g = np.zeros(self.gd.NxNyNz)
        self.f.integralgrad(self.kT, self.gd, self.x, g)
        return g

    def close(self):
        if self.handle is not None:
            _lib.load().deft_cg_destroy(self.handle)
            self.handle = None


def ConjugateGradient(f, gd, kT, x, lm=QuadraticLineMinimizer, stepsize=0.1):
    return Minimizer(f, gd, kT, x, linmin=lm, step=stepsize)


def PreconditionedConjugateGradient(f, gd, kT, x, lm=QuadraticLineMinimizer, stepsize=0.1):
    """src/ConjugateGradient.cpp:115-160,171-174."""
    return Minimizer(f, gd, kT, x, linmin=lm, step=stepsize, preconditioned=True)


def Precision(eps, m):
    m.precision = float(eps)
    return m


def MaxIter(n, m):
    m.maxiter = int(n)
    return m
