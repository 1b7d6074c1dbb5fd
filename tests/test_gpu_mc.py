"""LocalSampler on the GPU (through the C ABI) against the FP64 oracle.

- local_energy_change: equal to the oracle's and to the difference of GPU energies, to
  1e-12 (test_energy_consistency.jl:58-76).
- Sweeps with caller-supplied random numbers: the GPU applies the updates colour class by
  colour class; the oracle applies the same updates sequentially in that order. FP64
  states agree to 1e-12; ΔE and ΔS agree with the oracle and with energy differences.
- The colouring is proper: no bond joins two sites of one class.
- Device random numbers: ΔE/ΔS bookkeeping against GPU energies, and known thermal
  averages: the classical Heisenberg ring ⟨S_i·S_(i+1)⟩ = coth(βJ) - 1/(βJ) (Fisher 1964),
  and an independent spin in E = D Sz², within 2 %.
"""
import math

import numpy as np
import pytest

from models import rich_dipole, sc_c1, oracle_of

pytestmark = pytest.mark.gpu


def _rand(rng, nsweeps, ns):
    return np.concatenate([rng.standard_normal((nsweeps, ns, 3)), rng.random((nsweeps, ns, 3))], axis=2)


def _neighbours(sys_):
    """Sites joined by a bond to each site (both directions), from the host bond list."""
    L1, L2, L3 = sys_.dims

    def idx(c1, c2, c3, a):   # 0-based cell and atom, Sunny's linear order
        return c1 + L1 * (c2 + L2 * (c3 + L3 * a))

    nb = [set() for _ in range(sys_.nsites)]
    for b in sys_.bond_table():   # 0-based atoms
        for c3 in range(L3):
            for c2 in range(L2):
                for c1 in range(L1):
                    i = idx(c1, c2, c3, b.i)
                    j = idx((c1 + b.n[0]) % L1, (c2 + b.n[1]) % L2, (c3 + b.n[2]) % L3, b.j)
                    nb[i].add(j)
                    nb[j].add(i)
    return nb


@pytest.mark.parametrize("builder", ["rich", "sc"])
def test_local_energy_change(gpu, sg, orc, builder):
    sys_ = rich_dipole(sg) if builder == "rich" else sc_c1(sg, L=5)
    o = oracle_of(orc, sys_)
    S = sys_.dipoles_flat()
    kap = np.asarray(sys_.kappas).reshape(-1)
    rng = np.random.default_rng(2)
    E0 = sg.energy(sys_)
    for _ in range(6):
        i = int(rng.integers(0, sys_.nsites))
        v = rng.standard_normal(3)
        Sn = kap[i] * v / np.linalg.norm(v)
        dE = sg.local_energy_change(sys_, i, Sn)
        assert dE == pytest.approx(o.local_energy_change(S, i, Sn), abs=1e-12 * max(1.0, abs(E0)))
        S1 = S.copy()
        S1[i] = Sn
        sys_.set_state_flat(dipoles=S1)
        assert dE == pytest.approx(sg.energy(sys_) - E0, abs=1e-11 * max(1.0, abs(E0)))
        sys_.set_state_flat(dipoles=S)


@pytest.mark.parametrize("builder", ["rich", "sc"])
def test_colouring_is_proper(gpu, sg, builder):
    sys_ = rich_dipole(sg) if builder == "rich" else sc_c1(sg, L=6)
    ncol, col = sg.local_colors(sys_)
    assert 2 <= ncol <= 64 and col.min() == 0 and col.max() == ncol - 1
    for i, nb in enumerate(_neighbours(sys_)):
        for j in nb:
            assert col[i] != col[j]


@pytest.mark.parametrize("kT,nsweeps", [(0.6, 3), (0.0, 2), (0.4, 2.5)])
def test_sweeps_match_oracle_injected(gpu, sg, orc, kT, nsweeps):
    sys_ = rich_dipole(sg)
    o = oracle_of(orc, sys_)
    S0 = sys_.dipoles_flat()
    ncol, col = sg.local_colors(sys_)
    order = np.lexsort((np.arange(sys_.nsites), col))     # class by class, ascending site
    total = math.ceil(nsweeps)
    rand = _rand(np.random.default_rng(3), total, sys_.nsites)
    prop = sg.mix_proposals(0.3, sg.propose_uniform, 0.2, sg.propose_flip, 0.5, sg.propose_delta(0.4))
    smp = sg.LocalSampler(kT=kT, nsweeps=nsweeps, propose=prop)
    sg.step(sys_, smp, 1, rand)
    frac = nsweeps - math.floor(nsweeps) if nsweeps != total else 1.0
    S_ref, dE_ref, dS_ref = o.local_sweeps(S0, kT, total, frac, order, prop.terms, rand)
    S_gpu = sys_.dipoles_flat()
    assert np.max(np.abs(S_gpu - S_ref)) < 1e-12 * np.max(np.abs(S_ref))
    assert not np.allclose(S_gpu, S0)
    assert smp.ΔE == pytest.approx(dE_ref, abs=1e-10)
    assert np.allclose(smp.ΔS, dS_ref, atol=1e-10)
    assert smp.ΔE == pytest.approx(o.energy(S_gpu) - o.energy(S0), abs=1e-10)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_device_rng_bookkeeping(gpu, sg, precision):
    sys_ = sc_c1(sg, L=8, precision=precision)
    sys_.set_field([0.0, 0.0, 0.3])
    E0, M0 = sg.energy(sys_), sg.magnetization(sys_)
    smp = sg.LocalSampler(kT=0.8, nsweeps=4, propose=sg.propose_delta(0.5))
    sg.step(sys_, smp, 3)
    E1, M1 = sg.energy(sys_), sg.magnetization(sys_)
    tol = 1e-9 if precision == "fp64" else 2e-4
    assert smp.ΔE == pytest.approx(E1 - E0, abs=tol * sys_.nsites)
    assert np.allclose(smp.ΔS, M1 - M0, atol=tol * sys_.nsites)
    assert sys_.mc_sweep == 12


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_heisenberg_ring_energy(gpu, sg, precision):
    # 64 independent periodic rings of 64 unit spins along x (an orthorhombic cell, so the
    # x bond has no symmetry partners), ferromagnetic J = -1
    J, kT = -1.0, 0.5
    cr = sg.Crystal(sg.lattice_vectors(1, 1.3, 1.7, 90, 90, 90), [[0, 0, 0]])
    sys_ = sg.System(cr, [(1, sg.Moment(s=1, g=2))], "dipole_uncorrected", dims=(64, 8, 8), seed=11,
                     precision=precision, device=0)
    sys_.set_exchange(J, sg.Bond(1, 1, [1, 0, 0]))
    sys_.randomize_spins()
    smp = sg.LocalSampler(kT=kT, propose=sg.propose_delta(0.6))
    sg.step(sys_, smp, 300)
    Es = []
    for _ in range(200):
        sg.step(sys_, smp, 5)
        Es.append(sg.energy_per_site(sys_))
    bj = abs(J) / kT
    exact = J * (1 / math.tanh(bj) - 1 / bj)
    assert np.mean(Es) == pytest.approx(exact, rel=0.02)


def test_single_ion_energy(gpu, sg):
    # independent unit spins, E = D Sz^2 + const: <Sz^2> = <x^2> under exp(-D x^2 / kT), x in [-1, 1]
    D, kT = 1.0, 0.5
    sys_ = sg.System(sg.cubic_crystal(), [(1, sg.Moment(s=1, g=2))], "dipole_uncorrected", dims=(16, 16, 16),
                     seed=12, device=0)
    c28 = np.zeros(28)
    c28[3] = D / 3            # (D/3) O20 = (D/3)(3 Sz^2 - |S|^2), classical Stevens, q = 0 slot of c2
    sys_.set_onsite_stevens(c28, 1)
    sys_.randomize_spins()
    smp = sg.LocalSampler(kT=kT, nsweeps=2.0)
    sg.step(sys_, smp, 50)
    sz2 = []
    for _ in range(100):
        sg.step(sys_, smp, 1)
        sz2.append(np.mean(sys_.dipoles_flat()[:, 2] ** 2))
    x = np.linspace(-1, 1, 200001)
    w = np.exp(-D * x * x / kT)
    exact = np.sum(x * x * w) / np.sum(w)
    assert np.mean(sz2) == pytest.approx(exact, rel=0.02)


def test_sun_local_energy_change(gpu, sg, orc):
    from models import rich_sun
    sys_ = rich_sun(sg, N=3)
    o = oracle_of(orc, sys_)
    Z = sys_.coherents_flat()
    S = o.expected_spin(Z)
    E0 = sg.energy(sys_)
    rng = np.random.default_rng(12)
    for _ in range(5):
        i = int(rng.integers(0, sys_.nsites))
        z = rng.standard_normal(3) + 1j * rng.standard_normal(3)
        z /= np.linalg.norm(z)
        dE = sg.local_energy_change(sys_, i, z)
        assert dE == pytest.approx(o.local_energy_change(S, i, z, Z), abs=1e-12 * max(1.0, abs(E0)))


@pytest.mark.parametrize("N", [3, 4])
def test_sun_sweeps_match_oracle_injected(gpu, sg, orc, N):
    from models import rich_sun
    sys_ = rich_sun(sg, N=N)
    o = oracle_of(orc, sys_)
    Z0 = sys_.coherents_flat()
    S0 = o.expected_spin(Z0)
    ncol, col = sg.local_colors(sys_)
    order = np.lexsort((np.arange(sys_.nsites), col))
    rng = np.random.default_rng(13)
    rand = np.concatenate([rng.standard_normal((2, sys_.nsites, 2 * N)) / np.sqrt(2), rng.random((2, sys_.nsites, 3))], axis=2)
    prop = sg.mix_proposals(0.3, sg.propose_uniform, 0.3, sg.propose_flip, 0.4, sg.propose_delta(0.5))
    smp = sg.LocalSampler(kT=0.7, nsweeps=2, propose=prop)
    sg.step(sys_, smp, 1, rand)
    S_ref, Z_ref, dE_ref, dS_ref = o.local_sweeps_sun(S0, Z0, 0.7, 2, 1.0, order, prop.terms, rand)
    Z_gpu = sys_.coherents_flat()
    assert np.max(np.abs(Z_gpu - Z_ref)) < 1e-12
    assert not np.allclose(Z_gpu, Z0)
    assert smp.ΔE == pytest.approx(dE_ref, abs=1e-10)
    assert np.allclose(smp.ΔS, dS_ref, atol=1e-10)
    assert np.allclose(sys_.dipoles_flat(), S_ref, atol=1e-12)


def test_sun_anisotropy_energy(gpu, sg):
    # SU(3) spins with Λ = D Sz², no couplings (test_samplers.jl:5-10, 61-80): the exact
    # thermal mean energy, here sampled by the LocalSampler
    D, kT = 1.0, 0.5
    sys_ = sg.System(sg.cubic_crystal(), [(1, sg.Moment(s=1, g=2))], "SUN", dims=(16, 16, 16), seed=14)
    sys_.set_onsite_coupling(lambda Sx, Sy, Sz: D * Sz @ Sz, 1)
    sys_.randomize_spins()
    smp = sg.LocalSampler(kT=kT)
    sg.step(sys_, smp, 50)
    Es = []
    for _ in range(100):
        sg.step(sys_, smp, 1)
        Es.append(sg.energy_per_site(sys_))
    a = D / kT
    exact = D * (2 - (2 + 2 * a + a * a) * math.exp(-a)) / (a * (1 - (1 + a) * math.exp(-a)))
    assert np.mean(Es) == pytest.approx(exact, rel=0.02)


def test_rejects_self_bonds(gpu, sg):
    d = sg.System(sg.cubic_crystal(), [(1, sg.Moment(s=1, g=2))], "dipole", dims=(1, 2, 2), seed=1, device=0)
    d.set_exchange(1.0, sg.Bond(1, 1, [1, 0, 0]))
    d.randomize_spins()
    with pytest.raises(sg.SunnyGPUError, match="self-interaction"):
        sg.step(d, sg.LocalSampler(kT=0.1))


@pytest.mark.parametrize("kind", ["local", "langevin"])
def test_parallel_tempering_over_clones(gpu, sg, kind):
    sys_ = sc_c1(sg, L=4, J=-1.0, D=0.3)
    kT = [1.0, 1.04, 1.08, 1.12]   # close enough for swaps of 64-spin replicas to be accepted
    smp = sg.LocalSampler(kT=1.0, propose=sg.propose_delta(0.5)) if kind == "local" else \
        sg.Langevin(0.02, damping=0.2, kT=1.0)
    pt = sg.ParallelTempering(sys_, smp, kT)
    assert isinstance(pt, sg.SystemParallelTempering)
    if kind == "local":
        for r in range(4):
            assert pt.samplers[r].ΔE == pytest.approx(sg.energy(pt.systems[r]), rel=1e-12)
    pt.step_ensemble(40, 5)
    assert pt.n_exch.sum() == 4 * 1 + 4 * 2   # 8 rounds alternating between 1 and 2 pairs
    assert sorted(pt.system_ids) == [0, 1, 2, 3]
    if kind == "local":
        # sampler bookkeeping follows the system now at its temperature (ParallelTempering.jl:64-66)
        for rank in range(4):
            s = pt.systems[pt.system_ids[rank]]
            assert pt.samplers[rank].ΔE == pytest.approx(sg.energy(s), abs=1e-9 * s.nsites)
            assert np.allclose(pt.samplers[rank].ΔS, sg.magnetization(s), atol=1e-9 * s.nsites)
    assert pt.n_accept.sum() > 0
    pt.close()
