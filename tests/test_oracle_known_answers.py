"""The FP64 CPU oracle against the reference's RNG-independent known answers.

Each test cites the reference test it restates. These pin the oracle before it is used
as the checker of the GPU kernels.
"""
import numpy as np
import pytest


def _osys(orc, sys_):
    return orc.OracleSystem.from_system(sys_)


@pytest.fixture
def host(sg):
    def make(cryst, s, mode, dims=(1, 1, 1), seed=0):
        return sg.System(cryst, [(1, sg.Moment(s=s, g=2))], mode, dims=dims, seed=seed, device=None)
    return make


def test_rcs_factors_known_values(sg):
    # test_rescaling.jl:154-156: rcs_factors(s)[2]^2 == (1 - 1/2s)^2
    for s in (1, 1.5, 2, 3):
        lam = sg.rcs_factors(s)
        assert lam[2] == pytest.approx(1 - 1 / (2 * s))
    # OnsiteCoupling.jl:46-55 at s=3, all k
    s = 3.0
    lam = sg.rcs_factors(s)
    assert lam[4] == pytest.approx(1 - 3 / s + (11 / 4) / s**2 - (3 / 4) / s**3)
    assert lam[6] == pytest.approx(1 - 7.5 / s + 21.25 / s**2 - 28.125 / s**3 + 17.125 / s**4 - 3.75 / s**5)


def test_stevens_coefficients_easy_axis(sg):
    # -0.1 Sz^2 at s=1 gives c0 = -0.2/3 and c2[q=0] = (-0.1/3) * (1 - 1/2s)
    Sx, Sy, Sz = sg.spin_matrices(1)
    from sunny_gb300.operators import stevens_expansion_for_dipole
    c = stevens_expansion_for_dipole(-0.1 * Sz @ Sz, 1.0)
    assert c[0] == pytest.approx(-0.2 / 3)
    assert c[1 + 2] == pytest.approx(-0.1 / 3 * 0.5)
    assert np.count_nonzero(np.abs(c) > 1e-14) == 2


def test_anisotropy_rescaling(sg, orc, host):
    # test_rescaling.jl:93-109: E(:dipole) = λ_k E(:dipole_uncorrected) for pure-k anisotropy
    cryst = sg.cubic_crystal()
    s = 3
    lam = sg.rcs_factors(s)
    rng = np.random.default_rng(3)
    for k in (2, 4, 6):
        c = rng.standard_normal(2 * k + 1)
        O = sg.stevens_matrices_of_dim(k, 7)
        A = sum(c[k - q] * O[k - q] for q in range(-k, k + 1))
        d = np.array([0.3, -0.5, 0.8])
        Es = []
        for mode, ren in (("dipole", True), ("dipole_uncorrected", False)):
            h = host(cryst, s, mode)
            from sunny_gb300.operators import stevens_expansion_for_dipole
            h._onsite[0] = stevens_expansion_for_dipole(A, s, renormalize=ren)
            S = s * d / np.linalg.norm(d)
            Es.append(_osys(orc, h).energy(S[None, :]))
        assert Es[0] == pytest.approx(lam[k] * Es[1], rel=1e-10)


def test_anisotropy_sun_equivalence(sg, orc, host):
    # test_rescaling.jl:111-137: renormalised dipole anisotropy == SU(N) anisotropy on a dipolar ket
    cryst = sg.cubic_crystal()
    s = 3
    N = 7
    rng = np.random.default_rng(11)
    O2, O4, O6 = (sg.stevens_matrices_of_dim(k, N) for k in (2, 4, 6))
    # index q -> position k - q
    Lam = (rng.standard_normal() * (O2[2] + 3 * O2[0]) + rng.standard_normal() * (O4[4] - 5 * O4[2])
           + rng.standard_normal() * (O4[4] + 5 * O4[0]) + rng.standard_normal() * (O6[6] - 21 * O6[2])
           + rng.standard_normal() * (O6[6] + (105 / 16) * O6[4] + (231 / 16) * O6[0]))
    d = rng.standard_normal(3)
    h0 = host(cryst, s, "dipole")
    from sunny_gb300.operators import stevens_expansion_for_dipole
    h0._onsite[0] = stevens_expansion_for_dipole(Lam, s)
    E0 = _osys(orc, h0).energy((s * d / np.linalg.norm(d))[None, :])
    h1 = host(cryst, s, "SUN")
    h1._onsite[0] = Lam
    z = sg.ket_from_dipole(d, N)
    z = z / np.linalg.norm(z)
    S = sg.expected_spin(z[None, :])
    E1 = _osys(orc, h1).energy(S, z[None, :])
    assert E1 == pytest.approx(E0, rel=1e-9)


def test_biquadratic_renormalization(sg, orc, host):
    # test_rescaling.jl:171-208: dipole-mode biquad (RCS) equals SU(N) biquad on dipolar kets,
    # and :dipole_uncorrected reduces to biquad (S1.S2)^2
    cryst = sg.Crystal(sg.lattice_vectors(1, 1, 1, 90, 90, 90), [[0, 0, 0], [0.3, 0, 0]])
    s1 = 1.5
    bq = 1.2
    rng = np.random.default_rng(5)
    v1, v2 = rng.standard_normal(3), rng.standard_normal(3)
    bond = sg.Bond(1, 2, [0, 0, 0])
    energies = {}
    for mode in ("dipole", "SUN", "dipole_uncorrected"):
        h = host(cryst, s1, mode)
        h.set_exchange(0.0, bond, biquad=bq)
        o = _osys(orc, h)
        if mode == "SUN":
            N = int(2 * s1 + 1)
            zs = []
            for v in (v1, v2):
                z = sg.ket_from_dipole(v, N)
                zs.append(z / np.linalg.norm(z))
            Z = np.array(zs)
            energies[mode] = o.energy(sg.expected_spin(Z), Z)
            S = sg.expected_spin(Z)
        else:
            S = np.array([s1 * v1 / np.linalg.norm(v1), s1 * v2 / np.linalg.norm(v2)])
            energies[mode] = o.energy(S)
            if mode == "dipole_uncorrected":
                assert energies[mode] == pytest.approx(bq * (S[0] @ S[1]) ** 2, rel=1e-10)
    assert energies["dipole"] == pytest.approx(energies["SUN"], rel=1e-9)


def test_gradient_matches_finite_differences(sg, orc, host):
    # the gradient is dE/dS up to components parallel to S; check tangential parts by FD
    cryst = sg.diamond_crystal()
    h = host(cryst, 2, "dipole", dims=(2, 2, 2))
    J = np.array([[0.5, 0.2, -0.4], [0.2, 0.5, -0.4], [0.4, 0.4, 1.5]])
    h.set_exchange(0.5, sg.Bond(1, 3, [0, 0, 0]), biquad=0.3)
    O4 = sg.stevens_matrices_of_dim(4, 5)
    from sunny_gb300.operators import stevens_expansion_for_dipole
    h._onsite[2] = stevens_expansion_for_dipole(0.2 * ((1 / 20) * O4[4] + (1 / 4) * O4[0]), 2.0)
    h._field[:] = [0.0, 0.2, 0.3]
    o = _osys(orc, h)
    rng = np.random.default_rng(1)
    S = rng.standard_normal((h.nsites, 3))
    S = 2.0 * S / np.linalg.norm(S, axis=1)[:, None]
    g = o.grad(S)
    eps = 1e-4   # central differences: truncation ~eps^2, rounding of E ~1e-13 / eps
    for site in (0, 5, 17, 40):
        u = S[site] / np.linalg.norm(S[site])
        for a in range(3):
            # tangential direction: Sunny's anisotropy gradient drops terms parallel to S
            e = np.zeros(3)
            e[a] = 1.0
            ep = e - u * (u @ e)
            dS = np.zeros_like(S)
            dS[site] = eps * ep
            fd = (o.energy(S + dS) - o.energy(S - dS)) / (2 * eps)
            assert fd == pytest.approx(g[site] @ ep, rel=1e-6, abs=1e-8)


def test_kappa_energy_scaling(sg, orc, host):
    # test_rescaling.jl:33-58: linear ~ κ, quadratic ~ κ^2, quartic ~ κ^4 (dipole mode)
    cryst = sg.diamond_crystal()
    rng = np.random.default_rng(2)
    dirs = rng.standard_normal((64, 3))
    dirs /= np.linalg.norm(dirs, axis=1)[:, None]
    for kind, power in (("linear", 1), ("quadratic", 2), ("quartic", 4)):
        Es = []
        for kap in (1.0, 2.0):
            h = host(cryst, 1.5, "dipole", dims=(2, 2, 2))
            h._kappa[:] = kap
            if kind == "linear":
                h._field[:] = [0.0, 0.2, 0.3]
            elif kind == "quadratic":
                h.set_exchange(0.5, sg.Bond(1, 2, [0, 0, 0]))
            else:
                h.set_exchange(0.0, sg.Bond(1, 2, [0, 0, 0]), biquad=0.7)
                # drop the bilinear/scalar shifts, keep the pure quadrupole coupling
                for b in h._pairs:
                    h._pairs[b].scalar = 0.0
                    h._pairs[b].bilin = np.zeros((3, 3))
            Es.append(_osys(orc, h).energy(kap * dirs))
        assert Es[0] == pytest.approx(Es[1] / 2.0**power, rel=1e-10)


def test_midpoint_energy_conservation(sg, orc, host):
    # test_energy_consistency.jl:37-55: (max-min)/sqrt(N) < 1e-3 along an ImplicitMidpoint run
    cryst = sg.diamond_crystal()
    h = host(cryst, 2, "dipole", dims=(2, 2, 2))
    h.set_exchange(0.5, sg.Bond(1, 2, [0, 0, 0]))
    O4 = sg.stevens_matrices_of_dim(4, 5)
    from sunny_gb300.operators import stevens_expansion_for_dipole
    for a in range(8):
        h._onsite[a] = stevens_expansion_for_dipole(0.2 * ((1 / 20) * O4[4] + (1 / 4) * O4[0]), 2.0)
    h._field[:] = [0.0, 0.2, 0.3]
    o = _osys(orc, h)
    rng = np.random.default_rng(4)
    S = rng.standard_normal((h.nsites, 3))
    S = 2.0 * S / np.linalg.norm(S, axis=1)[:, None]
    Es = []
    for _ in range(300):
        st, S, _, _ = o.midpoint(S, None, 0.002, 0.0, 1e-12, 100, 1)
        assert st == 0
        Es.append(o.energy(S))
    assert (max(Es) - min(Es)) / np.sqrt(h.nsites) < 1e-3
    assert np.allclose(np.linalg.norm(S, axis=1), 2.0, rtol=1e-12)


def test_sun_anisotropy_thermal_energy(sg, orc, host):
    # test_samplers.jl:5-9, 64-88: <E> of the SU(3) single-ion model D Sz^2 from Langevin
    D, kT, L = 1.0, 0.5, 20
    a = D / kT
    E_ref = D * (2 - (2 + 2 * a + a**2) * np.exp(-a)) / (a * (1 - (1 + a) * np.exp(-a)))
    h = host(sg.cubic_crystal(), 1, "SUN", dims=(L, 1, 1))
    Sx, Sy, Sz = sg.spin_matrices(1)
    h._onsite[0] = D * Sz @ Sz
    o = _osys(orc, h)
    rng = np.random.default_rng(0)
    Z = rng.standard_normal((L, 3)) + 1j * rng.standard_normal((L, 3))
    Z /= np.linalg.norm(Z, axis=1)[:, None]
    S = sg.expected_spin(Z)
    dt, lam = 0.01, 1.0
    nth, nco = 1000, 10000
    noise = (rng.standard_normal((nth, L, 3)) + 1j * rng.standard_normal((nth, L, 3))) / np.sqrt(2)
    S, Z = o.langevin(S, Z, dt, lam, kT, nth, noise)
    Es = []
    for blk in range(nco // 500):
        noise = (rng.standard_normal((500, L, 3)) + 1j * rng.standard_normal((500, L, 3))) / np.sqrt(2)
        for k in range(0, 500, 10):
            S, Z = o.langevin(S, Z, dt, lam, kT, 10, noise[k:k + 10])
            Es.append(o.energy(S, Z) / L)
    assert np.mean(Es) == pytest.approx(E_ref, rel=0.1)


def test_sum_rule_and_merge_oracle(sg, orc, host):
    # test_correlation_sampling.jl:29-50 (classical sum rule) and :104-154 (merge equals
    # the running accumulation), on the raw accumulator:
    # sum over (α=β, i=j, q, ω) of data = n_all_ω * Ncells * sum_i κ_i^2 for every sample
    cryst = sg.fcc_primitive_crystal()
    h = host(cryst, 1, "dipole", dims=(4, 4, 4))
    h.set_exchange(1.0, sg.Bond(1, 1, [1, 0, 0]))
    o = _osys(orc, h)
    rng = np.random.default_rng(7)
    S = rng.standard_normal((h.nsites, 3))
    S /= np.linalg.norm(S, axis=1)[:, None]
    from sunny_gb300.correlations import adjusted_dt_and_downsampling_factor, CORR_PAIRS
    energies = np.linspace(0, 10.0, 12)
    dt, mp = adjusted_dt_and_downsampling_factor(0.08, len(energies), energies[-1])
    n = 2 * (len(energies) - 1)
    obs = np.tile(np.eye(3)[:, None, :], (1, h.nsites, 1))
    sc = orc.OracleCorrelations(o, obs.reshape(-1), 3, CORR_PAIRS, n, mp, dt, 1e-12)
    S1, _ = sc.add_sample(S, None)
    diag = [c for c, (a, b) in enumerate(CORR_PAIRS) if a == b]
    tot = sum(sc.data[c, 0, 0].sum() for c in diag)
    assert tot.real == pytest.approx(n * 64 * 1.0, rel=1e-12)
    assert abs(tot.imag) < 1e-9
    # merge
    sc0 = orc.OracleCorrelations(o, obs.reshape(-1), 3, CORR_PAIRS, n, mp, dt, 1e-12)
    sc1 = orc.OracleCorrelations(o, obs.reshape(-1), 3, CORR_PAIRS, n, mp, dt, 1e-12)
    sc2 = orc.OracleCorrelations(o, obs.reshape(-1), 3, CORR_PAIRS, n, mp, dt, 1e-12)
    states = [S, S1, rng.standard_normal((h.nsites, 3))]
    states[2] /= np.linalg.norm(states[2], axis=1)[:, None]
    sc0.add_sample(states[0], None); sc1.add_sample(states[0], None)
    for st in states[1:]:
        sc0.add_sample(st, None); sc2.add_sample(st, None)
    mu, nn = orc.merge_means([sc1.data, sc2.data], [1, 2])
    assert nn == 3
    assert np.allclose(mu, sc0.data, rtol=1e-12, atol=1e-12)


def test_replica_exchange_detailed_balance(orc):
    # ParallelTempering.jl:40-73: lnP >= 0 always swaps; otherwise swap iff u < exp(lnP)
    kT = np.array([0.1, 0.2, 0.4, 0.8])
    E = np.array([-4.0, -3.0, -3.5, -1.0])
    ids, acc = orc.replica_exchange(E, kT, [0, 1, 2, 3], 1, np.full(4, 0.999))
    lnP01 = (E[0] - E[1]) * (1 / kT[0] - 1 / kT[1])
    assert acc[0] == (lnP01 >= 0)
    lnP23 = (E[2] - E[3]) * (1 / kT[2] - 1 / kT[3])
    assert acc[2] == (lnP23 >= 0 or 0.999 < np.exp(lnP23))


def test_welford_errors_merge_oracle(sg, orc, host):
    # test_correlation_sampling.jl:104-136 with calculate_errors=true: merging 1 + 2
    # samples gives the data and M of the 3-sample running accumulation
    cryst = sg.fcc_primitive_crystal()
    h = host(cryst, 1, "dipole", dims=(3, 3, 3))
    h.set_exchange(1.0, sg.Bond(1, 1, [1, 0, 0]))
    o = _osys(orc, h)
    rng = np.random.default_rng(17)
    from sunny_gb300.correlations import adjusted_dt_and_downsampling_factor, CORR_PAIRS
    energies = np.linspace(0, 10.0, 8)
    dt, mp = adjusted_dt_and_downsampling_factor(0.08, len(energies), energies[-1])
    n = 2 * (len(energies) - 1)
    obs = np.tile(np.eye(3)[:, None, :], (1, h.nsites, 1)).reshape(-1)
    mk = lambda: orc.OracleCorrelations(o, obs, 3, CORR_PAIRS, n, mp, dt, 1e-12, calculate_errors=True)
    sc0, sc1, sc2 = mk(), mk(), mk()
    states = []
    for _ in range(3):
        S = rng.standard_normal((h.nsites, 3))
        states.append(S / np.linalg.norm(S, axis=1)[:, None])
    for k, S in enumerate(states):
        sc0.add_sample(S, None)
        (sc1 if k == 0 else sc2).add_sample(S, None)
    d, M, nn = orc.merge_with_errors([sc1.data, sc2.data], [sc1.M, sc2.M], [1, 2])
    assert nn == 3
    assert np.allclose(d, sc0.data, rtol=1e-12, atol=1e-13 * np.max(np.abs(sc0.data)))
    assert np.allclose(M, sc0.M, rtol=1e-10, atol=1e-12 * np.max(np.abs(sc0.M)))
    # M is the sum of squared deviations from the final mean
    assert np.max(sc0.M) > 0 and np.min(sc0.M) > -1e-12 * np.max(sc0.M)
