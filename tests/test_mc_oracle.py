"""LocalSampler on the CPU: the oracle's local_energy_change against total-energy
differences (test_energy_consistency.jl:58-76 does the same check at atol 1e-12), the
sampler's ΔE/ΔS bookkeeping, and the host-side proposal mixture rules."""
import numpy as np
import pytest

from models import rich_dipole, sc_c1


def _systems(sg):
    yield rich_dipole(sg, device=None)
    yield sc_c1(sg, L=4, device=None)
    # an axis of length 2: a site meets the same neighbour through two bonds
    s = sg.System(sg.cubic_crystal(), [(1, sg.Moment(s=2, g=2))], "dipole", dims=(2, 3, 4), seed=5, device=None)
    s.set_bond_coupling(sg.Bond(1, 1, [1, 0, 0]), 0.2, np.array([[0.1, 0.2, 0.3], [0.0, -0.4, 0.5], [0.6, 0.0, 0.7]]),
                        0.3)
    s.set_exchange(-0.5, sg.Bond(1, 1, [0, 1, 1]))
    s.randomize_spins()
    yield s


def test_oracle_local_energy_change_is_energy_difference(sg, orc):
    rng = np.random.default_rng(0)
    for sys_ in _systems(sg):
        o = orc.OracleSystem.from_system(sys_)
        S = sys_.dipoles_flat()
        kap = sys_.kappas.reshape(-1) if hasattr(sys_.kappas, "reshape") else np.asarray(sys_.kappas)
        E0 = o.energy(S)
        for _ in range(5):
            i = int(rng.integers(0, sys_.nsites))
            v = rng.standard_normal(3)
            Sn = kap[i] * v / np.linalg.norm(v)
            dE = o.local_energy_change(S, i, Sn)
            S1 = S.copy()
            S1[i] = Sn
            assert dE == pytest.approx(o.energy(S1) - E0, abs=1e-12 * max(1.0, abs(E0)))


def test_oracle_local_sweeps_bookkeeping(sg, orc):
    sys_ = rich_dipole(sg, device=None)
    o = orc.OracleSystem.from_system(sys_)
    S0 = sys_.dipoles_flat()
    rng = np.random.default_rng(1)
    rand = np.concatenate([rng.standard_normal((3, sys_.nsites, 3)), rng.random((3, sys_.nsites, 3))], axis=2)
    prop = [(0, 0.3, 0.0), (1, 0.2, 0.0), (2, 0.5, 0.4)]
    S1, dE, dS = o.local_sweeps(S0, 0.7, 3, 0.5, np.arange(sys_.nsites), prop, rand)
    assert not np.allclose(S1, S0)
    assert dE == pytest.approx(o.energy(S1) - o.energy(S0), abs=1e-10)
    assert np.allclose(dS, S1.sum(0) - S0.sum(0), atol=1e-10)
    kap = np.asarray(sys_.kappas).reshape(-1)
    assert np.allclose(np.linalg.norm(S1, axis=1), kap, rtol=1e-13)


def test_proposal_mixture_rules(sg):
    m = sg.mix_proposals(0.4, sg.propose_flip, 0.6, sg.propose_delta(0.2))
    assert m.terms == [(1, 0.4, 0.0), (2, 0.6, 0.2)]
    with pytest.raises(ValueError, match="Alternate weights"):
        sg.mix_proposals(0.4, sg.propose_flip, 0.6)
    s = sg.LocalSampler(kT=0.2)
    assert s.nsweeps == 1.0 and s.propose is sg.propose_uniform and s.ΔE == 0.0
    c = s.copy()
    assert c.kT == 0.2 and c is not s


def test_exchange_round_matches_oracle(sg, orc):
    rng = np.random.default_rng(4)
    for trial in range(20):
        n = int(rng.integers(2, 9))
        E_sys = rng.normal(-10.0, 3.0, n)
        kT = np.sort(rng.uniform(0.1, 2.0, n))
        ids = list(rng.permutation(n))
        u = rng.random(n)
        for start in (1, 2):
            ref_ids, ref_acc = orc.replica_exchange(E_sys, kT, ids, start, u)
            got_ids, tried, acc = sg.exchange_round([E_sys[i] for i in ids], kT, ids, start, lambda k: u[k])
            assert got_ids == list(ref_ids)
            assert np.array_equal(acc, ref_acc)
            assert np.array_equal(tried, [(k >= start - 1 and (k - start + 1) % 2 == 0 and k < n - 1) for k in range(n)])


def test_clone_system_copies_couplings_and_state(sg, orc):
    s = rich_dipole(sg, device=None)
    c = sg.clone_system(s, seed=99)
    assert c.seed == 99 and c.dims == s.dims
    S = s.dipoles_flat()
    assert np.array_equal(c.dipoles_flat(), S)
    assert orc.OracleSystem.from_system(c).energy(S) == orc.OracleSystem.from_system(s).energy(S)
    c.set_state_flat(dipoles=-S)
    assert np.array_equal(s.dipoles_flat(), S)


def test_oracle_sun_local_energy_change_is_energy_difference(sg, orc):
    from models import rich_sun
    rng = np.random.default_rng(5)
    for N in (3, 4):   # rich_sun sets an onsite term, which spin 1/2 rejects
        sys_ = rich_sun(sg, N=N, device=None)
        o = orc.OracleSystem.from_system(sys_)
        Z = sys_.coherents_flat()
        S = o.expected_spin(Z)
        E0 = o.energy(S, Z)
        for _ in range(4):
            i = int(rng.integers(0, sys_.nsites))
            z = rng.standard_normal(N) + 1j * rng.standard_normal(N)
            z /= np.linalg.norm(z)
            dE = o.local_energy_change(S, i, z, Z)
            Z1 = Z.copy()
            Z1[i] = z
            assert dE == pytest.approx(o.energy(o.expected_spin(Z1), Z1) - E0, abs=1e-12 * max(1.0, abs(E0)))


def test_oracle_sun_local_sweeps_bookkeeping(sg, orc):
    from models import rich_sun
    sys_ = rich_sun(sg, N=3, device=None)
    o = orc.OracleSystem.from_system(sys_)
    Z0 = sys_.coherents_flat()
    S0 = o.expected_spin(Z0)
    rng = np.random.default_rng(6)
    ns, N = sys_.nsites, 3
    rand = np.concatenate([rng.standard_normal((2, ns, 2 * N)) / np.sqrt(2), rng.random((2, ns, 3))], axis=2)
    prop = [(0, 0.3, 0.0), (1, 0.3, 0.0), (2, 0.4, 0.5)]
    S1, Z1, dE, dS = o.local_sweeps_sun(S0, Z0, 0.8, 2, 1.0, np.arange(ns), prop, rand)
    assert not np.allclose(Z1, Z0)
    assert np.allclose(S1, o.expected_spin(Z1), atol=1e-13)
    assert dE == pytest.approx(o.energy(S1, Z1) - o.energy(S0, Z0), abs=1e-10)
    assert np.allclose(dS, S1.sum(0) - S0.sum(0), atol=1e-10)


def test_replica_group_needs_prototype_dims(sg):
    # with dipole-dipole interactions a ReplicaBatch is a group of clones of the prototype
    s = sc_c1(sg, L=4, device=None)
    s.enable_dipole_dipole(1.0)
    with pytest.raises(ValueError, match="prototype's dims"):
        sg.ReplicaBatch(s, [s.dims, (2, 2, 2)], kT=[0.1, 0.2])


def test_enable_dipole_dipole_host_settings(sg):
    s = sc_c1(sg, L=2, device=None)
    with pytest.warns(UserWarning, match="Deprecated"):
        s.enable_dipole_dipole()
    mu0, demag = s._ewald
    assert mu0 == pytest.approx(0.6745817653)
    assert np.allclose(demag, np.eye(3) / 3)
    s.enable_dipole_dipole(0.5, demag=np.diag([0.1, 0.2, 0.7]))
    c = sg.clone_system(s, seed=3)
    assert c._ewald[0] == 0.5 and np.allclose(c._ewald[1], np.diag([0.1, 0.2, 0.7]))
    assert c._ewald_dirty


def test_oracle_ewald_single_dipole_known_answer(orc):
    # test_ewald.jl:18-30: one dipole (g = 1, |S| = 1) in a unit cubic box, demag 0: E = -1/6
    A = orc.ewald_matrices((1, 1, 1), np.eye(3), [[0, 0, 0]], np.zeros((3, 3)), 1.0)
    mu = np.array([0.0, 0.0, -1.0])
    assert 0.5 * mu @ A[0, 0, 0] @ mu == pytest.approx(-1 / 6, abs=1e-13)
    A = orc.ewald_matrices((2, 3, 4), np.eye(3), [[0, 0, 0]], np.zeros((3, 3)), 1.0)
    E = 0.5 * sum(mu @ A[c, 0, 0] @ mu for c in range(24))
    assert E == pytest.approx(-1 / 6, abs=1e-13)


def test_minimization_result_text(sg):
    assert str(sg.MinimizationResult(True, 12, -1.0)) == "Converged in 12 iterations"
    assert str(sg.MinimizationResult(False, 1000, -1.0)) == "Non-converged after 1000 iterations"


def test_oracle_local_sweeps_heisenberg_ring(sg, orc):
    # the oracle's Metropolis restatement samples the classical Heisenberg ring:
    # <S_i · S_i+1> = coth(βJ) - 1/(βJ) for unit spins (Fisher 1964)
    import math
    J, kT = -1.0, 0.5
    cr = sg.Crystal(sg.lattice_vectors(1, 1.3, 1.7, 90, 90, 90), [[0, 0, 0]])
    n = 512
    s = sg.System(cr, [(1, sg.Moment(s=1, g=2))], "dipole_uncorrected", dims=(n, 1, 1), seed=3, device=None)
    s.set_exchange(J, sg.Bond(1, 1, [1, 0, 0]))
    s.randomize_spins()
    o = orc.OracleSystem.from_system(s)
    rng = np.random.default_rng(8)
    S = s.dipoles_flat()
    order = np.arange(n)
    prop = [(2, 1.0, 0.8)]
    Es = []
    for block in range(300):
        rand = np.concatenate([rng.standard_normal((10, n, 3)), rng.random((10, n, 3))], axis=2)
        S, _, _ = o.local_sweeps(S, kT, 10, 1.0, order, prop, rand)
        if block >= 50:
            Es.append(o.energy(S) / n)
    exact = J * (1 / math.tanh(abs(J) / kT) - kT / abs(J))
    assert np.mean(Es) == pytest.approx(exact, rel=0.02)


def test_oracle_sun_local_sweeps_anisotropy_energy(sg, orc):
    # SU(3) spins with Λ = D Sz², no couplings (test_samplers.jl:5-10): the oracle's
    # Metropolis sweeps reproduce the exact thermal mean energy
    import math
    D, kT, n = 1.0, 0.5, 512
    s = sg.System(sg.cubic_crystal(), [(1, sg.Moment(s=1, g=2))], "SUN", dims=(8, 8, 8), seed=4, device=None)
    s.set_onsite_coupling(lambda Sx, Sy, Sz: D * Sz @ Sz, 1)
    s.randomize_spins()
    o = orc.OracleSystem.from_system(s)
    rng = np.random.default_rng(12)
    Z = s.coherents_flat()
    S = o.expected_spin(Z)
    Es = []
    for block in range(120):
        rand = np.concatenate([rng.standard_normal((5, n, 6)) / np.sqrt(2), rng.random((5, n, 3))], axis=2)
        S, Z, _, _ = o.local_sweeps_sun(S, Z, kT, 5, 1.0, np.arange(n), [(0, 1.0, 0.0)], rand)
        if block >= 20:
            Es.append(o.energy(S, Z) / n)
    a = D / kT
    exact = D * (2 - (2 + 2 * a + a * a) * math.exp(-a)) / (a * (1 - (1 + a) * math.exp(-a)))
    assert np.mean(Es) == pytest.approx(exact, rel=0.02)


@pytest.mark.parametrize("mode", ["dipole", "SUN"])
def test_oracle_ewald_energy_delta_is_energy_difference(sg, orc, mode):
    # ewald_energy_delta (Ewald.jl:210-241) inside local_energy_change: the change of the
    # pairwise dipole-dipole energy ½ Σ S·∇E plus the short-range terms
    from models import oracle_of
    cr = sg.Crystal(sg.lattice_vectors(1.1, 0.9, 0.8, 92, 85, 95), [[0, 0.01, 0.01], [0.6, 0.4, 0.5]])
    N = 3
    s = sg.System(cr, [(1, sg.Moment(s=1, g=2))], mode, dims=(2, 2, 1), seed=3, device=None)
    s.set_bond_coupling(sg.Bond(1, 2, [0, 0, 0]), 0.0, 0.3, 0.0)
    s.randomize_spins()
    o = oracle_of(orc, s)
    rng = np.random.default_rng(2)
    demag = np.diag([0.1, 0.2, 0.3])
    pos = [cr.position(i) for i in (1, 2)]
    A = orc.ewald_matrices(s.dims, cr.latvecs, pos, demag, 0.7)
    o.set_ewald(A)
    g = s._g

    def energy(S, Z=None):
        return o.energy(S, Z) + 0.5 * np.sum(S * orc.ewald_pairwise_grad(A, s.dims, s.natoms, S, g))

    S = s.dipoles_flat()
    Z = s.coherents_flat() if mode == "SUN" else None
    for _ in range(4):
        i = int(rng.integers(0, s.nsites))
        if mode == "SUN":
            zn = rng.standard_normal(N) + 1j * rng.standard_normal(N)
            zn /= np.linalg.norm(zn)
            Z1 = Z.copy()
            Z1[i] = zn
            S1 = o.expected_spin(Z1)
            ref = energy(S1, Z1) - energy(S, Z)
            got = o.local_energy_change(S, i, zn, Z=Z)
        else:
            v = rng.standard_normal(3)
            Sn = v / np.linalg.norm(v)
            S1 = S.copy()
            S1[i] = Sn
            ref = energy(S1) - energy(S)
            got = o.local_energy_change(S, i, Sn)
        assert got == pytest.approx(ref, abs=1e-12)
