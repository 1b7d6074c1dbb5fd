"""sgb_energy_grad_static, the gradient entry point that allocates no device memory,
against sgb_energy_grad on the same state (same tolerance as the gradient parity tests).
It serves hosts that may not call the CUDA allocator themselves (device memory owned by
their own pool, or a fixed budget), so the comparison covers every term the allocating
entry point evaluates, the dipole-dipole term included.

Collected last so that it also runs after every other GPU test in one process."""
import ctypes as C

import numpy as np
import pytest

from models import rich_dipole, rich_sun, sc_c1

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _grad(sg, sys_, fn, shape):
    lib = sys_._lib
    sys_._sync_to_device()
    out = np.zeros(shape)
    rc = getattr(lib, fn)(sys_.handle, sg._abi.dptr(out))
    assert rc == sg._abi.SGB_OK, (lib.sgb_last_error(sys_.handle) or b"").decode()
    return out


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_static_grad_dipole_two_calls(gpu, sg, precision):
    sys_ = rich_dipole(sg, precision=precision)
    shape = (sys_.nsites, 3)
    for _ in range(2):
        ref = _grad(sg, sys_, "sgb_energy_grad", shape)
        got = _grad(sg, sys_, "sgb_energy_grad_static", shape)
        assert rel(got, ref) < 1e-12
        sys_.randomize_spins()


def test_static_grad_sun_two_calls(gpu, sg):
    sys_ = rich_sun(sg, N=3)
    shape = (sys_.nsites, 3, 2)
    for _ in range(2):
        ref = _grad(sg, sys_, "sgb_energy_grad", shape)
        got = _grad(sg, sys_, "sgb_energy_grad_static", shape)
        assert rel(got, ref) < 1e-12
        sys_.randomize_spins()


def test_static_grad_shared_between_systems(gpu, sg):
    # two handles share the one static array: each call must see only its own system
    a = sc_c1(sg, L=8, seed=5)
    b = sc_c1(sg, L=6, seed=6)
    ga = _grad(sg, a, "sgb_energy_grad_static", (a.nsites, 3))
    gb = _grad(sg, b, "sgb_energy_grad_static", (b.nsites, 3))
    assert rel(ga, _grad(sg, a, "sgb_energy_grad", (a.nsites, 3))) < 1e-12
    assert rel(gb, _grad(sg, b, "sgb_energy_grad", (b.nsites, 3))) < 1e-12


def test_static_grad_rejects_oversize(gpu, sg):
    # 71^3 = 357,911 dipole sites need 1,073,733 doubles > 2^20
    sys_ = sg.System(sg.cubic_crystal(), [(1, sg.Moment(s=1, g=2))], "dipole", dims=(71, 71, 71),
                     precision="fp32", device=0)
    out = np.zeros((1, 3))
    rc = sys_._lib.sgb_energy_grad_static(sys_.handle, sg._abi.dptr(out))
    assert rc == sg._abi.SGB_ERR_ARG
    assert b"static scratch" in sys_._lib.sgb_last_error(sys_.handle)


@pytest.mark.parametrize("mode", ["dipole", "SUN"])
def test_static_grad_with_dipole_dipole_two_calls(gpu, sg, mode):
    # the long-range term runs on the transforms allocated when it was enabled
    sys_ = rich_dipole(sg) if mode == "dipole" else rich_sun(sg, N=3)
    sys_.enable_dipole_dipole(0.5)
    shape = (sys_.nsites, 3) if mode == "dipole" else (sys_.nsites, 3, 2)
    for _ in range(2):
        ref = _grad(sg, sys_, "sgb_energy_grad", shape)
        got = _grad(sg, sys_, "sgb_energy_grad_static", shape)
        assert rel(got, ref) < 1e-12
        sys_.randomize_spins()


def _current_device():
    for name in ("libcudart.so.13", "libcudart.so", "/usr/local/cuda/lib64/libcudart.so.13"):
        try:
            lib = C.CDLL(name)
        except OSError:
            continue
        d = C.c_int(-1)
        assert lib.cudaGetDevice(C.byref(d)) == 0
        return d.value
    pytest.skip("no CUDA runtime library")


def test_static_grad_keeps_the_current_device(gpu, sg):
    sys_ = sc_c1(sg, L=4, seed=2)
    before = _current_device()
    _grad(sg, sys_, "sgb_energy_grad_static", (sys_.nsites, 3))
    assert _current_device() == before
