"""Dipole-dipole interactions (Ewald summation) on the GPU against the reference's known
answers (test_ewald.jl, test_optimization.jl:31-52) and the oracle's pairwise sums."""
import math

import numpy as np
import pytest

from models import oracle_of

pytestmark = pytest.mark.gpu


def _triclinic(sg, precision="fp64", dims=(1, 1, 1), seed=0):
    # a random box with three atoms of different spins and random g tensors (test_ewald.jl:29-47)
    rng = np.random.default_rng(seed)
    cr = sg.Crystal(sg.lattice_vectors(1.1, 0.9, 0.8, 92, 85, 95), [[0, 0.01, 0.01], [0.1, 0.01, 0.01], [0.6, 0.4, 0.5]])
    mom = [(1, sg.Moment(s=1, g=rng.random((3, 3)))), (2, sg.Moment(s=1.5, g=rng.random((3, 3)))),
           (3, sg.Moment(s=2, g=rng.random((3, 3))))]
    s = sg.System(cr, mom, "dipole", dims=dims, seed=seed + 1, precision=precision)
    s.randomize_spins()
    R = rng.standard_normal((3, 3))
    demag = R.T @ R
    s.enable_dipole_dipole(1.0, demag)
    return s, demag


def _reference_grad(orc, sys_, demag, mu0=1.0):
    o = oracle_of(orc, sys_)
    S = sys_.dipoles_flat()
    cr = sys_.crystal
    pos = [cr.position(i) for i in range(1, sys_.natoms + 1)]
    A = orc.ewald_matrices(sys_.dims, cr.latvecs, pos, demag, mu0)
    g = sys_._g
    gd = orc.ewald_pairwise_grad(A, sys_.dims, sys_.natoms, S, g)
    return o, S, gd, o.grad(S) + gd


def test_single_dipole_energy(gpu, sg):
    cr = sg.Crystal(sg.lattice_vectors(1, 1, 1, 90, 90, 90), [[0, 0, 0]])
    s = sg.System(cr, [(1, sg.Moment(s=1, g=1))], "dipole")
    s.enable_dipole_dipole(1.0, demag=0)
    assert sg.energy(s) == pytest.approx(-1 / 6, abs=1e-13)
    s2 = sg.System(cr, [(1, sg.Moment(s=1, g=1))], "dipole", dims=(2, 3, 4))
    s2.enable_dipole_dipole(1.0, demag=0)
    assert sg.energy_per_site(s2) == pytest.approx(-1 / 6, abs=1e-13)


@pytest.mark.parametrize("dims", [(1, 1, 1), (2, 3, 1)])
def test_energy_and_gradient_match_pairwise_sums(gpu, sg, orc, dims):
    sys_, demag = _triclinic(sg, dims=dims)
    o, S, gd, gtot = _reference_grad(orc, sys_, demag)
    g_gpu = sg.energy_grad(sys_)
    assert np.max(np.abs(g_gpu - gtot)) <= 1e-12 * np.max(np.abs(gtot))
    E_ref = o.energy(S) + 0.5 * np.sum(S * gd)
    assert sg.energy(sys_) == pytest.approx(E_ref, abs=1e-12 * max(1.0, abs(E_ref)))


def test_energy_per_site_independent_of_supercell(gpu, sg):
    a, _ = _triclinic(sg, dims=(1, 1, 1))
    b, _ = _triclinic(sg, dims=(2, 3, 1))
    Sa = a.dipoles_flat()
    b.set_state_flat(dipoles=np.repeat(Sa, 6, axis=0).reshape(3, 6, 3).reshape(-1, 3))   # same spin per atom
    assert sg.energy_per_site(a) == pytest.approx(sg.energy_per_site(b), abs=1e-12)


def _rhs(S, xi, g, dt, lam):
    # Integrators.jl:266-275
    return -np.cross(S, xi + dt * g - dt * lam * np.cross(S, g))


def _norm(S, kap):
    return S / np.linalg.norm(S, axis=1)[:, None] * kap[:, None]


def test_langevin_with_dipole_dipole_matches_restatement(gpu, sg, orc):
    sys_, demag = _triclinic(sg, dims=(2, 1, 1))
    kap = np.asarray(sys_.kappas, dtype=float)
    o = oracle_of(orc, sys_)
    cr = sys_.crystal
    A = orc.ewald_matrices(sys_.dims, cr.latvecs, [cr.position(i) for i in range(1, 4)], demag, 1.0)

    def grad(S):
        return o.grad(S) + orc.ewald_pairwise_grad(A, sys_.dims, sys_.natoms, S, sys_._g)

    dt, lam, kT = 0.01, 0.2, 0.3
    noise = np.random.default_rng(9).standard_normal((2, sys_.nsites, 3))
    S = sys_.dipoles_flat()
    for k in range(2):   # stochastic Heun (Integrators.jl:313-332) in FP64
        xi = noise[k] * math.sqrt(2 * dt * lam * kT)
        d1 = _rhs(S, xi, grad(S), dt, lam)
        P = _norm(S + d1, kap)
        d2 = _rhs(P, xi, grad(P), dt, lam)
        S = _norm(S + (d1 + d2) / 2, kap)
    sg.step(sys_, sg.Langevin(dt, damping=lam, kT=kT), 2, noise)
    assert np.max(np.abs(sys_.dipoles_flat() - S)) < 1e-12 * np.max(np.abs(S))


def test_midpoint_with_dipole_dipole(gpu, sg, orc):
    # exchange plus dipole-dipole on a cubic lattice (the random box's 0.1 Å pairs are too
    # stiff for the fixed-point iteration at a useful dt)
    cr = sg.Crystal(sg.lattice_vectors(2, 2, 2, 90, 90, 90), [[0, 0, 0]])
    sys_ = sg.System(cr, [(1, sg.Moment(s=1, g=2))], "dipole", dims=(3, 3, 2), seed=4)
    sys_.set_exchange(1.0, sg.Bond(1, 1, [1, 0, 0]))
    sys_.enable_dipole_dipole(0.5)
    sys_.randomize_spins()
    o = oracle_of(orc, sys_)
    A = orc.ewald_matrices(sys_.dims, cr.latvecs, [cr.position(1)], np.eye(3) / 3, 0.5)
    kap = np.asarray(sys_.kappas, dtype=float)

    def grad(S):
        return o.grad(S) + orc.ewald_pairwise_grad(A, sys_.dims, 1, S, sys_._g)

    dt, tol = 0.01, 1e-12
    atol2 = tol * tol * sys_.nsites
    S = sys_.dipoles_flat()
    E0 = sg.energy(sys_)
    for _ in range(3):   # spherical midpoint (Integrators.jl:379-413) in FP64
        Sp = S.copy()
        for _ in range(100):
            H = _norm((S + Sp) / 2, kap)
            Spp = S + _rhs(H, 0.0, grad(H), dt, 0.0)
            done = np.sum((Sp - Spp) ** 2) <= atol2
            Sp = Spp
            if done:
                break
        S = _norm(Sp, kap)
    sg.step(sys_, sg.ImplicitMidpoint(dt, tol=tol), 3)
    assert np.max(np.abs(sys_.dipoles_flat() - S)) < 1e-10
    sg.step(sys_, sg.ImplicitMidpoint(dt, tol=tol), 200)
    assert abs(sg.energy(sys_) - E0) <= 1e-3 * abs(E0)


@pytest.mark.parametrize("mode,jitter,ref", [("dipole", 0.0, 0.6327349993784377), ("dipole", 1e-8, -5.7060439873282),
                                             ("SUN", 0.0, -0.619368052000758), ("SUN", 1e-8, -5.7060439873282)])
def test_canted_afm_optimization(gpu, sg, mode, jitter, ref):
    # test_optimization.jl:31-52, both modes
    cr = sg.Crystal(sg.lattice_vectors(1, 1, 2, 90, 90, 90), [[0, 0, 0]])
    s = sg.System(cr, [(1, sg.Moment(s=1.5, g=2))], mode, dims=(4, 4, 1), seed=3)
    s.set_exchange(1.0, sg.Bond(1, 1, [1, 0, 0]))
    s.set_field([1.0, 0, 0])
    s.enable_dipole_dipole(1.0)
    s.polarize_spins([0, 0, 1])
    r = sg.minimize_energy(s, jitter=jitter)
    assert r.converged
    assert sg.energy_per_site(s) == pytest.approx(ref, rel=1e-9)


def _ewald_oracle(orc, sys_, demag, mu0):
    """Oracle of the system's short-range couplings with the pairwise dipole-dipole term
    included in its local energy changes; also returns the pair matrices A."""
    o = oracle_of(orc, sys_)
    cr = sys_.crystal
    A = orc.ewald_matrices(sys_.dims, cr.latvecs, [cr.position(i) for i in range(1, sys_.natoms + 1)], demag, mu0)
    o.set_ewald(A)
    return o, A


def _two_atom_box(sg, mode="dipole", precision="fp64", seed=5):
    # exchange plus dipole-dipole between two atoms of different spin and g tensor
    rng = np.random.default_rng(seed)
    cr = sg.Crystal(sg.lattice_vectors(2.0, 2.2, 2.5, 90, 90, 90), [[0, 0, 0], [0.5, 0.4, 0.3]])
    g2 = np.eye(3) * 2 + 0.2 * rng.standard_normal((3, 3))
    mom = [(1, sg.Moment(s=1, g=2)), (2, sg.Moment(s=1 if mode == "SUN" else 1.5, g=g2))]
    s = sg.System(cr, mom, mode, dims=(2, 2, 2), seed=seed + 1, precision=precision)
    s.set_exchange(0.5, sg.Bond(1, 2, [0, 0, 0]))
    if mode == "SUN":
        s.set_onsite_coupling(lambda Sx, Sy, Sz: -0.3 * Sz @ Sz, 1)
    s.randomize_spins()
    demag = np.diag([0.1, 0.2, 0.3])
    s.enable_dipole_dipole(0.4, demag)
    return s, demag


def test_local_energy_change_with_dipole_dipole(gpu, sg, orc):
    # ewald_energy_delta (Ewald.jl:210-241) inside local_energy_change (Interactions.jl:311-373)
    sys_, demag = _triclinic(sg, dims=(2, 1, 1))
    o, _ = _ewald_oracle(orc, sys_, demag, 1.0)
    S = sys_.dipoles_flat()
    kap = np.asarray(sys_.kappas, dtype=float).reshape(-1)
    rng = np.random.default_rng(4)
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


def test_sun_local_energy_change_with_dipole_dipole(gpu, sg, orc):
    sys_, demag = _two_atom_box(sg, "SUN")
    o, _ = _ewald_oracle(orc, sys_, demag, 0.4)
    Z = sys_.coherents_flat()
    S = o.expected_spin(Z)
    rng = np.random.default_rng(6)
    E0 = sg.energy(sys_)
    for _ in range(4):
        i = int(rng.integers(0, sys_.nsites))
        zn = rng.standard_normal(3) + 1j * rng.standard_normal(3)
        zn /= np.linalg.norm(zn)
        dE = sg.local_energy_change(sys_, i, zn)
        assert dE == pytest.approx(o.local_energy_change(S, i, zn, Z=Z), abs=1e-12 * max(1.0, abs(E0)))
        Z1 = Z.copy()
        Z1[i] = zn
        sys_.set_state_flat(coherents=Z1)
        assert dE == pytest.approx(sg.energy(sys_) - E0, abs=1e-11 * max(1.0, abs(E0)))
        sys_.set_state_flat(coherents=Z)


@pytest.mark.parametrize("kT,nsweeps", [(0.5, 2), (0.0, 1), (0.8, 1.5)])
def test_local_sweeps_with_dipole_dipole(gpu, sg, orc, kT, nsweeps):
    # LocalSampler with dipole-dipole: one block proposes the sites in sweep order and
    # updates every site's field after each accepted move; the oracle applies the same
    # proposals in the same order with the pairwise sum per proposal
    sys_, demag = _two_atom_box(sg)
    o, A = _ewald_oracle(orc, sys_, demag, 0.4)
    S0 = sys_.dipoles_flat()
    _, col = sg.local_colors(sys_)
    order = np.lexsort((np.arange(sys_.nsites), col))
    total = math.ceil(nsweeps)
    rng = np.random.default_rng(8)
    rand = np.concatenate([rng.standard_normal((total, sys_.nsites, 3)), rng.random((total, sys_.nsites, 3))], axis=2)
    prop = sg.mix_proposals(0.3, sg.propose_uniform, 0.2, sg.propose_flip, 0.5, sg.propose_delta(0.4))
    smp = sg.LocalSampler(kT=kT, nsweeps=nsweeps, propose=prop)
    E0 = sg.energy(sys_)
    sg.step(sys_, smp, 1, rand)
    frac = nsweeps - math.floor(nsweeps) if nsweeps != total else 1.0
    S_ref, dE_ref, dS_ref = o.local_sweeps(S0, kT, total, frac, order, prop.terms, rand)
    S_gpu = sys_.dipoles_flat()
    assert np.max(np.abs(S_gpu - S_ref)) < 1e-11 * np.max(np.abs(S_ref))
    assert not np.allclose(S_gpu, S0)
    assert smp.ΔE == pytest.approx(dE_ref, abs=1e-10 * max(1.0, abs(E0)))
    assert np.allclose(smp.ΔS, dS_ref, atol=1e-10)
    assert smp.ΔE == pytest.approx(sg.energy(sys_) - E0, abs=1e-10 * max(1.0, abs(E0)))


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_local_sweeps_with_dipole_dipole_device_rng(gpu, sg, precision):
    sys_, _ = _two_atom_box(sg, precision=precision)
    E0, M0 = sg.energy(sys_), sg.magnetization(sys_)
    smp = sg.LocalSampler(kT=0.6, nsweeps=3, propose=sg.propose_delta(0.5))
    sg.step(sys_, smp, 2)
    tol = 1e-9 if precision == "fp64" else 2e-4
    assert smp.ΔE == pytest.approx(sg.energy(sys_) - E0, abs=tol * sys_.nsites)
    assert np.allclose(smp.ΔS, sg.magnetization(sys_) - M0, atol=tol * sys_.nsites)


def test_sun_local_sweeps_with_dipole_dipole(gpu, sg, orc):
    sys_, demag = _two_atom_box(sg, "SUN")
    o, _ = _ewald_oracle(orc, sys_, demag, 0.4)
    N = 3
    Z0 = sys_.coherents_flat()
    S0 = o.expected_spin(Z0)
    _, col = sg.local_colors(sys_)
    order = np.lexsort((np.arange(sys_.nsites), col))
    rng = np.random.default_rng(12)
    rand = np.concatenate([rng.standard_normal((2, sys_.nsites, 2 * N)) / np.sqrt(2), rng.random((2, sys_.nsites, 3))], axis=2)
    prop = sg.mix_proposals(0.3, sg.propose_uniform, 0.3, sg.propose_flip, 0.4, sg.propose_delta(0.5))
    smp = sg.LocalSampler(kT=0.6, nsweeps=2, propose=prop)
    E0 = sg.energy(sys_)
    sg.step(sys_, smp, 1, rand)
    S_ref, Z_ref, dE_ref, dS_ref = o.local_sweeps_sun(S0, Z0, 0.6, 2, 1.0, order, prop.terms, rand)
    Z_gpu = sys_.coherents_flat()
    assert np.max(np.abs(Z_gpu - Z_ref)) < 1e-11
    assert not np.allclose(Z_gpu, Z0)
    assert smp.ΔE == pytest.approx(dE_ref, abs=1e-10 * max(1.0, abs(E0)))
    assert np.allclose(smp.ΔS, dS_ref, atol=1e-10)
    assert smp.ΔE == pytest.approx(sg.energy(sys_) - E0, abs=1e-10 * max(1.0, abs(E0)))


def test_sqw_trajectory_with_dipole_dipole(gpu, sg, orc):
    # S(q,ω) sampling runs the per-stage midpoint path with snapshots when dipole-dipole is
    # on. With a negligible μ0 μB² the trajectory is the plain one: same data as the oracle.
    sys_ = sg.System(sg.diamond_crystal(), [(1, sg.Moment(s=1.5, g=2))], "dipole", dims=(2, 3, 4), seed=101)
    sys_.set_exchange(0.6498, sg.Bond(1, 3, [0, 0, 0]))
    sys_.randomize_spins()
    sys_.enable_dipole_dipole(1e-14)
    sc = sg.SampledCorrelations(sys_, measure=sg.ssf_perp(sys_), energies=np.linspace(0.0, 5.5, 10), dt=0.12)
    o = oracle_of(orc, sys_)
    obs = sc.measure.observables.reshape(-1)
    oc = orc.OracleCorrelations(o, obs, sc.measure.nobs, sc.measure.corr_pairs, sc.n_all_omega, sc.measperiod, sc.dt,
                                sc.integrator.tol)
    S = sys_.dipoles_flat()
    for _ in range(2):
        sg.add_sample(sc, sys_)
        S, _ = oc.add_sample(S, None)
    assert np.max(np.abs(sc.data - oc.data)) < 1e-8 * np.max(np.abs(oc.data))
    assert np.max(np.abs(sys_.dipoles_flat() - S)) < 1e-8


def test_sum_rule_with_dipole_dipole(gpu, sg):
    # test_correlation_sampling.jl:29-50 holds for any trajectory, here one driven by
    # dipole-dipole interactions as well
    cr = sg.fcc_primitive_crystal()
    sys_ = sg.System(cr, [(1, sg.Moment(s=1, g=2))], "dipole", dims=(4, 4, 4), seed=111)
    sys_.set_exchange(1.0, sg.Bond(1, 1, [1, 0, 0]))
    sys_.enable_dipole_dipole(0.3)
    sys_.randomize_spins()
    sc = sg.SampledCorrelations(sys_, measure=sg.ssf_trace(sys_, apply_g=False), energies=np.linspace(0, 10.0, 40), dt=0.08)
    sg.add_sample(sc, sys_)
    d = sc.data
    diag = [c for c, (a, b) in enumerate(sc.measure.corr_pairs) if a == b]
    tot = sum(d[c, 0, 0].sum() for c in diag)
    assert tot.real == pytest.approx(sc.n_all_omega * 64 * 1.0, rel=1e-12)


def test_sun_gradient_with_dipole_dipole(gpu, sg, orc):
    # HZ gains (dE/dS · S) Z with dE/dS the dipole-dipole field at the expected dipoles
    cr = sg.Crystal(sg.lattice_vectors(1.1, 0.9, 1.3, 90, 90, 90), [[0, 0, 0], [0.5, 0.4, 0.3]])
    s = sg.System(cr, [(1, sg.Moment(s=1, g=2))], "SUN", dims=(2, 2, 1), seed=7)
    s.set_exchange(0.3, sg.Bond(1, 2, [0, 0, 0]))
    s.set_onsite_coupling(lambda Sx, Sy, Sz: -0.4 * Sz @ Sz, 1)
    s.set_onsite_coupling(lambda Sx, Sy, Sz: -0.4 * Sz @ Sz, 2)
    s.randomize_spins()
    demag = np.eye(3) / 3
    s.enable_dipole_dipole(0.7, demag)
    o = oracle_of(orc, s)
    Z = s.coherents_flat()
    S = o.expected_spin(Z)
    A = orc.ewald_matrices(s.dims, cr.latvecs, [cr.position(i) for i in (1, 2)], demag, 0.7)
    f = orc.ewald_pairwise_grad(A, s.dims, s.natoms, S, s._g)
    Sx, Sy, Sz = sg.spin_matrices_of_dim(3)
    hz_ref = o.grad(None, Z) + np.einsum("sa,abc,sc->sb", f, np.stack([Sx, Sy, Sz]), Z)
    hz = sg.energy_grad(s)
    assert np.max(np.abs(hz - hz_ref)) < 1e-12 * np.max(np.abs(hz_ref))
    E_ref = o.energy(S, Z) + 0.5 * np.sum(S * f)
    assert sg.energy(s) == pytest.approx(E_ref, abs=1e-12 * abs(E_ref))


def _sun_hz(sg, orc, o, A, sys_, Z):
    # HZ of set_energy_grad_coherents! (Interactions.jl:596-669) with the dipole-dipole field
    # dE/dS at the expected dipoles of Z (normalised or not)
    S = o.expected_spin(Z)
    f = orc.ewald_pairwise_grad(A, sys_.dims, sys_.natoms, S, sys_._g)
    Sx, Sy, Sz = sg.spin_matrices_of_dim(sys_.N)
    return o.grad(None, Z) + np.einsum("sa,abc,sc->sb", f, np.stack([Sx, Sy, Sz]), Z)


def _rhs_sun(Z, xi, HZ, dt, lam):
    # rhs_sun! (Integrators.jl:277-286) with proj (MathBasics.jl:62)
    if lam == 0:
        return -1j * dt * HZ
    v = xi + dt * (1j + lam) * HZ
    c = np.sum(Z.conj() * v, axis=1) / np.sum(np.abs(Z) ** 2, axis=1)
    return -(v - c[:, None] * Z)


def _norm_ket(Z, kap):
    return Z / np.sqrt(np.sum(np.abs(Z) ** 2, axis=1) / kap)[:, None]


def test_sun_langevin_with_dipole_dipole(gpu, sg, orc):
    # Heun for coherent states (Integrators.jl:90-108), one launch per stage on the GPU
    sys_, demag = _two_atom_box(sg, "SUN")
    o, A = _ewald_oracle(orc, sys_, demag, 0.4)
    kap = np.asarray(sys_.kappas, dtype=float).reshape(-1)
    dt, lam, kT = 0.01, 0.2, 0.3
    rng = np.random.default_rng(10)
    noise = (rng.standard_normal((3, sys_.nsites, 3)) + 1j * rng.standard_normal((3, sys_.nsites, 3))) / np.sqrt(2)
    Z = sys_.coherents_flat()
    for k in range(3):
        xi = noise[k] * math.sqrt(2 * dt * lam * kT)
        d1 = _rhs_sun(Z, xi, _sun_hz(sg, orc, o, A, sys_, Z), dt, lam)
        P = _norm_ket(Z + d1, kap)
        d2 = _rhs_sun(P, xi, _sun_hz(sg, orc, o, A, sys_, P), dt, lam)
        Z = _norm_ket(Z + (d1 + d2) / 2, kap)
    sg.step(sys_, sg.Langevin(dt, damping=lam, kT=kT), 3, noise)
    assert np.max(np.abs(sys_.coherents_flat() - Z)) < 1e-12
    assert np.max(np.abs(sys_.dipoles_flat() - o.expected_spin(Z))) < 1e-12


def test_sun_midpoint_with_dipole_dipole(gpu, sg, orc):
    # Schrödinger midpoint (Integrators.jl:422-452) in FP64, then energy conservation
    sys_, demag = _two_atom_box(sg, "SUN")
    o, A = _ewald_oracle(orc, sys_, demag, 0.4)
    kap = np.asarray(sys_.kappas, dtype=float).reshape(-1)
    dt, tol = 0.01, 1e-12
    atol2 = tol * tol * sys_.nsites
    Z = sys_.coherents_flat()
    E0 = sg.energy(sys_)
    for _ in range(3):
        Zp = Z.copy()
        for _ in range(100):
            Zb = (Z + Zp) / 2
            Zpp = Z + _rhs_sun(Zb, 0.0, _sun_hz(sg, orc, o, A, sys_, Zb), dt, 0.0)
            done = np.sum(np.abs(Zp - Zpp) ** 2) <= atol2
            Zp = Zpp
            if done:
                break
        Z = _norm_ket(Zp, kap)
    sg.step(sys_, sg.ImplicitMidpoint(dt, tol=tol), 3)
    assert np.max(np.abs(sys_.coherents_flat() - Z)) < 1e-10
    sg.step(sys_, sg.ImplicitMidpoint(dt, tol=tol), 200)
    assert abs(sg.energy(sys_) - E0) <= 1e-3 * max(1.0, abs(E0))


def test_sun_sqw_trajectory_with_dipole_dipole(gpu, sg):
    # add_sample runs the per-stage SU(N) midpoint path with snapshots: the state after one
    # sample equals plain ImplicitMidpoint stepping over the same number of steps
    a, _ = _two_atom_box(sg, "SUN")
    b, _ = _two_atom_box(sg, "SUN")
    sc = sg.SampledCorrelations(a, measure=sg.ssf_perp(a), energies=np.linspace(0.0, 3.0, 6), dt=0.05)
    sg.add_sample(sc, a)
    nsteps = sc.measperiod * (sc.n_all_omega // 2)
    sg.step(b, sg.ImplicitMidpoint(sc.dt, tol=sc.integrator.tol), nsteps)
    assert np.array_equal(a.coherents_flat(), b.coherents_flat())
    assert np.all(np.isfinite(sc.data)) and np.max(np.abs(sc.data)) > 0
