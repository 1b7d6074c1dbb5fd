"""CPU tests: the C-ABI library exports every declared symbol, and host-side setup
(crystals, bond propagation, sampler parameters) matches the reference's conventions."""
import ctypes
import math
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    hdr = (ROOT / "include" / "sunny_gb300.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(sgb_\w+)\s*\(", hdr, re.M)))


def test_library_exports_every_declared_symbol(sg):
    lib_path = ROOT / "sunny.jl_gb300" / "libsunnygb300.so"
    if not lib_path.exists():
        pytest.skip("library not built")
    lib = ctypes.CDLL(str(lib_path))
    syms = declared_symbols()
    assert len(syms) >= 40
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    # every declared symbol has a ctypes signature in the binding
    from sunny_gb300 import _abi
    assert set(syms) == set(_abi.SIGNATURES)
    lib = sg.load_library()
    assert b"sm_103a" in lib.sgb_version()


def test_struct_layouts_match_header(sg):
    from sunny_gb300 import _abi
    assert ctypes.sizeof(_abi.BondC) == 4 * 5 + 4 + 8 + 72 + 4 + 4 + 200  # i,j,n[3], pad, scalar, bilin, kind, pad, biquad
    assert ctypes.sizeof(_abi.Desc) == 8 * 4
    assert _abi.CorrDesc.dt.offset == 40
    # sgb_proposal: int32 n, int32 kind[4], (pad), double weight[4], double magnitude[4]
    assert ctypes.sizeof(_abi.Proposal) == 88 and _abi.Proposal.weight.offset == 24


def test_create_without_gpu_fails_cleanly(sg):
    from sunny_gb300 import _abi
    lib = sg.load_library()
    n = ctypes.c_int(0)
    cudart = ctypes.CDLL("libcudart.so.13") if True else None
    if cudart.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0:
        pytest.skip("a GPU is present")
    d = _abi.Desc()
    d.dims[:] = (2, 2, 2)
    d.natoms, d.N, d.mode, d.precision, d.device = 1, 0, 0, 0, 0
    h = ctypes.c_void_p()
    rc = lib.sgb_create(ctypes.byref(d), ctypes.byref(h))
    assert rc == _abi.SGB_ERR_CUDA
    assert h.value is None
    assert lib.sgb_last_error(None)
    # argument validation happens before any CUDA call
    d.mode = 7
    assert lib.sgb_create(ctypes.byref(d), ctypes.byref(h)) == _abi.SGB_ERR_ARG
    assert b"Mode must be" in lib.sgb_last_error(None)


def test_cubic_and_pyrochlore_bond_shells(sg):
    c = sg.cubic_crystal()
    nn = c.bonds_at_distance(1.0)
    assert sorted(b.n for b in nn) == [(0, 0, 1), (0, 1, 0), (1, 0, 0)]
    p = sg.pyrochlore_crystal()
    assert p.natoms == 16
    d1 = math.sqrt(2) / 4
    d2 = math.sqrt(6) / 4
    assert len(p.bonds_at_distance(d1)) == 16 * 6 // 2
    assert len(p.bonds_at_distance(d2)) == 16 * 12 // 2
    for b in p.bonds_at_distance(d1):
        assert sg.bond_parity(b)


def test_triangular_anisotropic_propagation(sg):
    # J -> R J R^T under C3; reversed bonds carry J^T (AllowedCouplings.jl:121-123)
    tri = sg.triangular_crystal(a=4.05, c=6.75)
    J1 = np.array([[-0.24, 0, 0], [0, -0.24, 0.1], [0, 0.1, -0.24]])
    eq = tri.equivalent_bonds(sg.Bond(1, 1, [1, 0, 0]), J1)
    assert len(eq) == 3
    rots = []
    for k in range(3):
        th = 2 * math.pi * k / 3
        rots.append(np.array([[math.cos(th), -math.sin(th), 0], [math.sin(th), math.cos(th), 0], [0, 0, 1]]))
    used = set()
    for b, J in eq:
        # under the -3 group every copy is J1 rotated by a C3 power (inversion's proper part is 1)
        k = next(k for k, R in enumerate(rots) if np.allclose(J, R @ J1 @ R.T) or np.allclose(J, (R @ J1 @ R.T).T))
        used.add(k)
        assert abs(tri.distance(b) - 4.05) < 1e-9
    assert used == {0, 1, 2}
    with pytest.raises(ValueError):
        sg.cubic_crystal().equivalent_bonds(sg.Bond(1, 1, [1, 0, 0]), J1)


def test_sampler_parameters(sg):
    # SampledCorrelations.jl:152-173 for 16^3 pyrochlore: energies 0..6 meV in 200 bins, dt 0.025
    dt, mp = sg.adjusted_dt_and_downsampling_factor(0.025, 200, 6.0)
    assert mp == 21
    assert dt == pytest.approx(2 * math.pi / ((6.0 / 199) * 21 * 398))
    assert dt == pytest.approx(0.024933, abs=1e-6)


def test_host_only_system_and_bond_table(sg):
    sys_ = sg.System(sg.pyrochlore_crystal(), [(1, sg.Moment(s=1.5, g=2))], "dipole", dims=(2, 2, 2), device=None)
    sys_.set_exchange(1.0, sg.Bond(1, 2, [0, 0, 0]))
    sys_.set_exchange(0.05, sg.Bond(1, 6, [0, 0, 0]) if abs(sys_.crystal.distance(sg.Bond(1, 6, [0, 0, 0])) - math.sqrt(6) / 4) < 1e-9
                      else sg.Bond(*next((b.i, b.j, b.n) for b in sys_.crystal.bonds_at_distance(math.sqrt(6) / 4))))
    tab = sys_.bond_table()
    assert len(tab) == 48 + 96
    assert all(t.biquad_kind == 0 for t in tab)
    with pytest.raises(RuntimeError):
        sg.energy(sys_)
    with pytest.raises(ValueError, match="Bond must connect different atoms"):
        sys_.set_exchange(1.0, sg.Bond(1, 1, [0, 0, 0]))


def test_integrator_argument_errors(sg):
    with pytest.raises(ValueError, match="Use ImplicitMidpoint"):
        sg.Langevin(0.1, damping=0.0, kT=1.0)
    with pytest.raises(ValueError, match="Select positive dt"):
        sg.Langevin(-0.1, damping=0.1, kT=1.0)
    with pytest.raises(ValueError, match="not currently supported"):
        sg.ImplicitMidpoint(0.1, kT=0.5)
