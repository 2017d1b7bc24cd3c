"""Seeded synthetic inputs for the FMT hot path (host-side set-up only).

The reference's drivers build the same kinds of inputs by hand: hard walls
frozen by a constraint mask (papers/contact/figs/walls.cpp:30-37,93-101) and
hard-sphere solutes excluded from a cavity (papers/contact/figs/sphere.cpp:
28-33,93-105).  Here the walls hold n = 0 exactly and are frozen by the mask;
the initial density is the bulk density times (1 + amp * xi), xi seeded
Gaussian noise smoothed by exp(-k^2 sigma^2 / 2) and renormalised to unit RMS.
"""
import math

import numpy as np


def bulk_density(eta, R=1.0):
    return eta / (4 * math.pi / 3 * R ** 3)


def chemical_potential(R, kT, nb):
    """mu of HardSpheresWBnotensor(R) + IdealGas() at bulk density nb, the
    value find_chemical_potential returns (src/equation-of-state.cpp:189-192)."""
    n3 = nb * 4 * math.pi / 3 * R ** 3
    n2 = nb * 4 * math.pi * R ** 2
    omn3 = 1 - n3
    l = math.log(omn3)
    fpr, fpr2 = 4 * math.pi * R, 4 * math.pi * R * R
    g = n3 + omn3 * omn3 * l
    dg = n3 - 2 * omn3 * l
    S = g / n3 ** 2
    dS = (dg * n3 - 2 * g) / n3 ** 3
    f3 = S / (36 * math.pi * omn3 ** 2)
    df3 = (dS * omn3 + 2 * S) / (36 * math.pi * omn3 ** 3)
    d3 = n2 / (fpr2 * omn3) + n2 * n2 / (fpr * omn3 ** 2) + df3 * n2 ** 3
    d2 = -l / fpr2 + 2 * n2 / (fpr * omn3) + f3 * 3 * n2 * n2
    x = 18.01528 * 1822.8885 * kT / (2 * math.pi)
    nQ = x * math.sqrt(x)
    return -(kT * (d3 * 4 * math.pi / 3 * R ** 3 + d2 * 4 * math.pi * R ** 2) + kT * math.log(nb / nQ))


def smoothed_noise(shape, spacing, sigma, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    xi = rng.standard_normal(shape)
    k = [2 * np.pi * np.fft.fftfreq(n, d=h) for n, h in zip(shape, spacing)]
    kz = 2 * np.pi * np.fft.rfftfreq(shape[2], d=spacing[2])
    k2 = k[0][:, None, None] ** 2 + k[1][None, :, None] ** 2 + kz[None, None, :] ** 2
    xi = np.fft.irfftn(np.fft.rfftn(xi) * np.exp(-0.5 * k2 * sigma * sigma), s=shape,
                       axes=(0, 1, 2))
    rms = np.sqrt(np.mean(xi * xi))
    return xi / rms if rms > 0 else xi


class Slit:
    """Hard-wall slit: periodic N^3 box of edge N*dx; the fluid occupies
    0 < z < width (strict), the rest is wall with n = 0 and frozen DOF."""

    def __init__(self, N=64, dx=0.2, eta=0.3, width=None, R=1.0, kT=1.0, seed=1, amp=0.05,
                 sigma=0.4, Nxy=None):
        Nxy = N if Nxy is None else Nxy
        self.shape = (Nxy, Nxy, N)
        self.dx = dx
        self.L = N * dx
        self.lat = np.diag([Nxy * dx, Nxy * dx, N * dx])
        self.width = self.L / 2 if width is None else width
        self.R, self.kT, self.eta = R, kT, eta
        self.nb = bulk_density(eta, R)
        self.mu = chemical_potential(R, kT, self.nb)
        z = np.arange(N) * dx
        inside = ((z > 1e-12) & (z < self.width - 1e-12)).astype(np.float64)
        self.mask = np.broadcast_to(inside, self.shape).copy()
        xi = smoothed_noise(self.shape, (dx, dx, dx), sigma, seed)
        self.n0 = self.nb * (1 + amp * xi) * self.mask

    @property
    def size(self):
        return int(np.prod(self.shape))


class Solute:
    """Hard-sphere solute at the cell centre: n = 0 and frozen DOF within
    radius r_excl of the centre (papers/contact/figs/sphere.cpp:93-105)."""

    def __init__(self, N=256, dx=0.1, eta=0.35, r_excl=3.0, R=1.0, kT=1.0, seed=2, amp=0.05,
                 sigma=0.4):
        self.shape = (N, N, N)
        self.dx = dx
        self.L = N * dx
        self.lat = np.diag([self.L] * 3)
        self.R, self.kT, self.eta = R, kT, eta
        self.nb = bulk_density(eta, R)
        self.mu = chemical_potential(R, kT, self.nb)
        c = np.arange(N) * dx - self.L / 2
        r2 = c[:, None, None] ** 2 + c[None, :, None] ** 2 + c[None, None, :] ** 2
        self.mask = (r2 > r_excl * r_excl).astype(np.float64)
        xi = smoothed_noise(self.shape, (dx, dx, dx), sigma, seed)
        self.n0 = self.nb * (1 + amp * xi) * self.mask

    @property
    def size(self):
        return int(np.prod(self.shape))


def batch_sweep(count=64, seed=3, sizes=(32, 48, 64, 96, 128), dx=0.2, eta=(0.05, 0.45),
                width=(3.0, 10.0), R=1.0, kT=1.0):
    """The batched sweep: `count` independent hard-wall slits, packing
    fraction uniform in eta, grid edge drawn from `sizes` (cubic, spacing dx),
    slit width uniform in `width` but at most 0.7 of the cell edge (so a wall
    remains on small cells).  Returns a list of Slit problems."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for i in range(count):
        N = int(rng.choice(sizes))
        e = float(rng.uniform(*eta))
        w = min(float(rng.uniform(*width)), 0.7 * N * dx)
        out.append(Slit(N=N, dx=dx, eta=e, width=w, R=R, kT=kT, seed=seed * 1000 + i))
    return out


class WallsSolutes:
    """Hard-wall slit (fluid in 0 < z < width) holding hard-sphere solutes:
    n = 0 and frozen DOF in the walls and within radius Rs of each solute
    centre (periodic distances), as sphere.cpp excludes its cavity
    (papers/contact/figs/sphere.cpp:93-105).  The bulk start is nb on the free
    points (amp = 0) or nb (1 + amp xi) with the smoothed-noise recipe.  The
    mask and start are built on each access (a training set holds thousands
    of these)."""

    def __init__(self, N=128, dx=0.2, eta=0.3, width=6.0, solutes=(), R=1.0, kT=1.0, seed=0,
                 amp=0.0, sigma=0.4):
        self.shape = (N, N, N)
        self.dx = dx
        self.L = N * dx
        self.lat = np.diag([self.L] * 3)
        self.width = width
        self.solutes = tuple(tuple(float(v) for v in s) for s in solutes)
        self.R, self.kT, self.eta = R, kT, eta
        self.nb = bulk_density(eta, R)
        self.mu = chemical_potential(R, kT, self.nb)
        self.seed, self.amp, self.sigma = seed, amp, sigma

    @property
    def mask(self):
        N, dx = self.shape[0], self.dx
        c = np.arange(N) * dx
        inside = (c > 1e-12) & (c < self.width - 1e-12)
        mask = np.broadcast_to(inside[None, None, :], self.shape).copy()
        for (x0, y0, z0, rs) in self.solutes:
            d = [np.minimum(np.abs(c - a), self.L - np.abs(c - a)) for a in (x0, y0, z0)]
            r2 = d[0][:, None, None] ** 2 + d[1][None, :, None] ** 2 + d[2][None, None, :] ** 2
            mask &= r2 > rs * rs
        return mask.astype(np.float64)

    @property
    def n0(self):
        if self.amp:
            xi = smoothed_noise(self.shape, (self.dx,) * 3, self.sigma, self.seed)
            return self.nb * (1 + self.amp * xi) * self.mask
        return self.nb * self.mask

    @property
    def size(self):
        return int(np.prod(self.shape))


def walls_solutes_set(count, seed, N=128, dx=0.2, eta=(0.1, 0.4), width=(3.0, 10.0),
                      solutes=(1, 4), radius=(1.0, 4.0), R=1.0, kT=1.0):
    """`count` problems for the learned warm start: slit width uniform in
    `width` (at most 0.7 of the cell edge), 1-4 solutes with radius uniform in
    `radius`, centres uniform in x, y and in the slit's z range, packing
    fraction uniform in `eta`; every problem starts from the bulk density."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    L = N * dx
    for _ in range(count):
        e = float(rng.uniform(*eta))
        w = min(float(rng.uniform(*width)), 0.7 * L)
        k = int(rng.integers(solutes[0], solutes[1] + 1))
        sol = [(float(rng.uniform(0, L)), float(rng.uniform(0, L)), float(rng.uniform(0, w)),
                float(rng.uniform(*radius))) for _ in range(k)]
        out.append(WallsSolutes(N=N, dx=dx, eta=e, width=w, solutes=sol, R=R, kT=kT))
    return out
