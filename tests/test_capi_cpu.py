"""CPU tests of the boundary and the host logic (no GPU needed): the C ABI
library loads and exports every symbol include/deft_gb300.h declares, host-only
entry points agree with the oracle, and the set-up helpers behave."""
import ctypes
import math
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "deft_gb300.h")


def _declared():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(deft_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    from deft_gb300 import _lib
    L = _lib.load()
    declared = _declared()
    assert len(declared) >= 30
    for name in declared:
        assert hasattr(L, name), name
    assert set(declared) == set(_lib.EXPORTS)
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True,
                         text=True).stdout
    exported = set(re.findall(r" T (deft_[a-z0-9_]+)", out))
    assert set(declared) <= exported


def test_library_is_built_for_sm_103a():
    from deft_gb300 import _build
    assert "arch=compute_103a,code=sm_103a" in " ".join(_build.ARCH)


def test_strerror_and_null_arguments():
    from deft_gb300 import _lib
    L = _lib.load()
    assert L.deft_strerror(0) == b"ok"
    assert L.deft_strerror(_lib.ERR_NAN).startswith(b"energy")
    assert L.deft_ctx_create(0, None) == _lib.ERR_ARG
    assert L.deft_grid_create(None, None, 4, 4, 4, None) == _lib.ERR_ARG
    assert L.deft_fmt_energy(None, None, 0, None, None) == _lib.ERR_ARG
    assert L.deft_cg_step(None, None) == _lib.ERR_ARG


@pytest.mark.skipif(os.path.exists("/dev/nvidia0"), reason="checks the no-GPU error path")
def test_context_fails_cleanly_without_gpu():
    from deft_gb300 import _lib
    L = _lib.load()
    h = ctypes.c_void_p()
    s = L.deft_ctx_create(0, ctypes.byref(h))
    assert s in (_lib.ERR_CUDA, _lib.ERR_ARG)
    assert len(L.deft_last_error()) > 0


@pytest.mark.parametrize("eta", [0.05, 0.2, 0.3, 0.45])
def test_find_chemical_potential_matches_oracle(oracle_mod, eta):
    from deft_gb300 import _lib
    from deft_gb300.workloads import chemical_potential
    L = _lib.load()
    nb = eta / (4 * math.pi / 3)
    mu = ctypes.c_double()
    assert L.deft_find_chemical_potential(1.0, 1.0, nb, ctypes.addressof(mu)) == 0
    ref = oracle_mod.find_mu(1.0, 1.0, nb)
    assert abs(mu.value / ref - 1) < 1e-13
    assert abs(chemical_potential(1.0, 1.0, nb) / ref - 1) < 1e-13


@pytest.mark.parametrize("eta", [0.05, 0.2, 0.3, 0.45])
@pytest.mark.parametrize("kind", [0, 1, 2])
def test_bulk_density_inverts_the_chemical_potential(eta, kind):
    """deft_bulk_density (the structure preconditioner's n_b) against closed
    forms of the bulk chemical potential: White Bear and mark II give the
    Carnahan-Starling mu_ex (the reference's find_chemical_potential for
    White Bear), Rosenfeld the Percus-Yevick compressibility route,
    beta mu_ex = -ln(1-eta) + (14 eta - 13 eta^2 + 5 eta^3) / (2 (1-eta)^3)."""
    from deft_gb300 import _lib
    from deft_gb300.workloads import chemical_potential
    L = _lib.load()
    R, kT = 1.0, 1.0
    nb = eta / (4 * math.pi / 3)
    if kind == 1:
        x = 18.01528 * 1822.8885 * kT / (2 * math.pi)
        nQ = x * math.sqrt(x)
        mu_ex = -math.log(1 - eta) + (14 * eta - 13 * eta ** 2 + 5 * eta ** 3) / (2 * (1 - eta) ** 3)
        mu = -kT * (math.log(nb / nQ) + mu_ex)
    else:
        mu = chemical_potential(R, kT, nb)
    out = ctypes.c_double()
    assert L.deft_bulk_density(R, kT, mu, kind, ctypes.addressof(out)) == 0
    assert abs(out.value / nb - 1) < 1e-12
    # no solution for the tensor kinds; bad arguments refused
    assert L.deft_bulk_density(R, kT, mu, 3, ctypes.addressof(out)) == _lib.ERR_ARG
    assert L.deft_bulk_density(-1.0, kT, mu, kind, ctypes.addressof(out)) == _lib.ERR_ARG


def test_grid_size_from_dx_rule():
    """GridDescription(lat, dx): N = 1 + int(e/100 + |a|/dx) (src/GridDescription.cpp:27-29);
    L = 12.8, dx = 0.2 gives 65, not 64."""
    from deft_gb300.api import grid_size_from_dx
    assert grid_size_from_dx(np.diag([12.8, 12.8, 12.8]), 0.2) == [65, 65, 65]
    assert grid_size_from_dx(np.diag([1.0, 2.0, 3.0]), 0.5) == [3, 5, 7]


def test_slit_workload():
    from deft_gb300.workloads import Slit
    s = Slit(N=32, dx=0.2, eta=0.3, seed=1, Nxy=8)
    assert s.shape == (8, 8, 32)
    z = np.arange(32) * 0.2
    inside = (z > 0) & (z < 3.2 - 1e-9)
    assert np.array_equal(s.mask[0, 0] > 0, inside)
    assert np.all(s.n0[:, :, ~inside] == 0)
    assert np.all(s.n0[:, :, inside] > 0)
    rel = s.n0[:, :, inside] / s.nb - 1
    assert 0.02 < rel.std() < 0.08  # 5 % smoothed noise
    s2 = Slit(N=32, dx=0.2, eta=0.3, seed=1, Nxy=8)
    assert np.array_equal(s.n0, s2.n0)  # seeded
