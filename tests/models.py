"""Model builders shared by the tests: small versions of the workloads plus models that
exercise every coupling type of the hot path."""
import math

import numpy as np


def sc_c1(sg, L=16, precision="fp64", seed=1, device=0, s=1.0, J=1.0, D=0.1):
    """Simple cubic AFM Heisenberg with -D Sz^2 (the 16^3, s=1 dipole workload at L=16)."""
    sys_ = sg.System(sg.cubic_crystal(), [(1, sg.Moment(s=s, g=2))], "dipole", dims=(L, L, L), seed=seed,
                     precision=precision, device=device)
    sys_.set_exchange(J, sg.Bond(1, 1, [1, 0, 0]))
    sys_.set_onsite_coupling(lambda Sx, Sy, Sz: -D * Sz @ Sz, 1)
    sys_.randomize_spins()
    return sys_


def pyrochlore_c2(sg, L=16, precision="fp32", seed=1, device=0, J1=1.0, J2=0.05):
    """Pyrochlore Heisenberg AFM with J1 and J2, s=3/2 (the 16^3 x 16 workload at L=16)."""
    cr = sg.pyrochlore_crystal()
    sys_ = sg.System(cr, [(1, sg.Moment(s=1.5, g=2))], "dipole", dims=(L, L, L), seed=seed, precision=precision,
                     device=device)
    b1 = cr.bonds_at_distance(math.sqrt(2) / 4)[0]
    b2 = cr.bonds_at_distance(math.sqrt(6) / 4)[0]
    sys_.set_exchange(J1, b1)
    sys_.set_exchange(J2, b2)
    sys_.randomize_spins()
    return sys_


def triangular_c3(sg, L=(48, 48, 4), precision="fp32", seed=1, device=0):
    """Layered triangular SU(3) model with anisotropic J1 (the 48x48x4 workload)."""
    cr = sg.triangular_crystal(a=4.05, c=6.75)
    sys_ = sg.System(cr, [(1, sg.Moment(s=1, g=2))], "SUN", dims=L, seed=seed, precision=precision, device=device)
    J1 = np.array([[-0.24, 0, 0], [0, -0.24, 0.1], [0, 0.1, -0.24]])
    sys_.set_exchange(J1, sg.Bond(1, 1, [1, 0, 0]))
    sys_.set_exchange(0.05, sg.Bond(1, 1, [1, 2, 0]))   # 2nd neighbour, distance sqrt(3) a
    sys_.set_exchange(0.32, sg.Bond(1, 1, [2, 0, 0]))   # 3rd neighbour, distance 2a
    sys_.set_exchange(-0.05, sg.Bond(1, 1, [0, 0, 1]))  # interlayer
    sys_.set_onsite_coupling(lambda Sx, Sy, Sz: -2.2 * Sz @ Sz, 1)
    sys_.randomize_spins()
    return sys_


def rich_dipole(sg, precision="fp64", device=0, dims=(3, 2, 4), seed=3, biquad_matrix=True):
    """Diamond lattice, s=3, with every dipole-mode coupling: anisotropic exchange, scalar
    and matrix biquadratic, k=2,4,6 anisotropy, field, inhomogeneous kappa."""
    cr = sg.diamond_crystal()
    sys_ = sg.System(cr, [(1, sg.Moment(s=3, g=2))], "dipole", dims=dims, seed=seed, precision=precision, device=device)
    sys_.set_exchange(0.5, sg.Bond(1, 3, [0, 0, 0]), biquad=0.2)
    O2, O4, O6 = (sg.stevens_matrices_of_dim(k, 7) for k in (2, 4, 6))
    A = 0.3 * (O2[2] + 3 * O2[0]) - 0.02 * (O4[4] - 5 * O4[2]) + 0.001 * (O6[6] - 21 * O6[2]) + 0.01 * O2[1]
    for a in range(1, 9):
        sys_.set_onsite_coupling(A, a)
    sys_.set_field([0.05, -0.2, 0.3])
    rng = np.random.default_rng(seed)
    if biquad_matrix:
        B = rng.standard_normal((5, 5)) * 0.01
        b = next(bb for bb in cr.bonds_at_distance(math.sqrt(2) / 2) if bb.i == 1)
        sys_.set_bond_coupling(b, 0.1, rng.standard_normal((3, 3)) * 0.1, B)
    sys_.set_kappas(3.0 * (1 + 0.3 * rng.random(sys_.nsites)))
    sys_.randomize_spins()
    return sys_


def rich_sun(sg, N=3, precision="fp64", device=0, dims=(2, 3, 2), seed=4, biquad=True):
    """SU(N) model on a two-atom cell with field, onsite Λ, anisotropic exchange, scalar
    and matrix biquadratic couplings."""
    cr = sg.Crystal(sg.lattice_vectors(1, 1.1, 1.2, 90, 90, 90), [[0, 0, 0], [0.5, 0.5, 0.3]])
    s = (N - 1) / 2
    sys_ = sg.System(cr, [(1, sg.Moment(s=s, g=2))], "SUN", dims=dims, seed=seed, precision=precision, device=device)
    rng = np.random.default_rng(seed)
    J = rng.standard_normal((3, 3)) * 0.3
    sys_.set_bond_coupling(sg.Bond(1, 2, [0, 0, 0]), 0.05, J, 0.15 if biquad else 0.0)
    sys_.set_bond_coupling(sg.Bond(1, 1, [1, 0, 0]), 0.0, 0.4 * np.eye(3), rng.standard_normal((5, 5)) * 0.05 if biquad else 0.0)
    sys_.set_bond_coupling(sg.Bond(2, 2, [0, 0, 1]), 0.0, -0.2 * np.eye(3), 0.0)
    Sx, Sy, Sz = sg.spin_matrices_of_dim(N)
    H = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
    for a in (1, 2):
        sys_.set_onsite_coupling(-0.7 * Sz @ Sz + 0.05 * (H + H.conj().T), a)
    sys_.set_field([0.1, 0.0, -0.25])
    sys_.randomize_spins()
    return sys_


def oracle_of(orc, sys_):
    return orc.OracleSystem.from_system(sys_)


def energy_consistency_inhomog(sg, precision="fp64", device=0, seed=0, ewald=True):
    """The inhomogeneous dipole system of test_energy_consistency.jl:4-33 (mode :dipole,
    inhomog=true): diamond 2x2x2, s=2, field (0, 0.2, 0.3), anisotropic exchange on
    Bond(1, 2, [0,0,0]), a quartic Stevens term on every atom, a matrix biquadratic
    coupling on Bond(1, 1, [0,0,1]), dipole-dipole 0.5 (if `ewald`), a random field per
    site, random κ, random spins; then to_inhomogeneous with a vacancy at (1,1,1,2),
    exchange 0.5 on (1,1,1,1)-(2,1,1,2) at offset (1,0,0), 0.7 (Si·Sj)^2 on
    (2,2,1,2)-(2,1,1,3) at offset (0,-1,0), and 0.4(Sx^4+Sy^4+Sz^4) at (2,2,1,4).
    Sunny propagates these couplings to every symmetry-equivalent bond and atom, rotated by
    the site symmetries; this host mirror has no symmetry analysis for diamond and sets the
    exchange and the biquadratic term on the one bond and the quartic term unrotated on
    every atom, which changes the model, not the checks."""
    cr = sg.diamond_crystal()
    sys_ = sg.System(cr, [(1, sg.Moment(s=2, g=2))], "dipole", dims=(2, 2, 2), seed=seed, precision=precision,
                     device=device)
    sys_.set_field([0.0, 0.2, 0.3])
    J, K, G, D = 0.5, 1.0, 0.2, 0.4
    sys_.set_bond_coupling(sg.Bond(1, 2, [0, 0, 0]), 0.0, np.array([[J, G, -D], [G, J, -D], [D, D, J + K]]), 0.0)
    O4 = sg.stevens_matrices_of_dim(4, 5)
    for a in range(1, 9):
        sys_.set_onsite_coupling(0.2 * ((1 / 20) * O4[4] + (1 / 4) * O4[0]), a)
    B = np.array([[1.2, 0, 0, 0, 0], [0, 1, 0, 0, 0], [0, 0, 1.1, 0, -1.4], [0, 0, 0, 1, 0], [0, 0, 1.4, 0, 1.3]])
    sys_.set_bond_coupling(sg.Bond(1, 1, [0, 0, 1]), 0.0, np.zeros((3, 3)), 0.1 * B)
    if ewald:
        sys_.enable_dipole_dipole(0.5)
    rng = np.random.default_rng(seed)
    for i in range(sys_.nsites):
        sys_.set_field_at(0.1 * rng.standard_normal(3), i)
    sys_.set_kappas(rng.random(sys_.nsites))
    sys_.randomize_spins()
    s2 = sg.to_inhomogeneous(sys_)
    s2.set_vacancy_at((1, 1, 1, 2))
    s2.set_exchange_at(0.5, (1, 1, 1, 1), (2, 1, 1, 2), offset=(1, 0, 0))
    s2.set_exchange_at(0.0, (2, 2, 1, 2), (2, 1, 1, 3), biquad=0.7, offset=(0, -1, 0))
    s2.set_onsite_coupling_at(lambda Sx, Sy, Sz: 0.4 * (Sx @ Sx @ Sx @ Sx + Sy @ Sy @ Sy @ Sy + Sz @ Sz @ Sz @ Sz),
                              (2, 2, 1, 4))
    return sys_, s2


def diluted_dipole(sg, precision="fp64", device=0, L=6, seed=5, frac=0.2):
    """Bond-diluted, bond-disordered simple cubic s=1 dipole model: to_inhomogeneous of
    J1 = 1 with -0.1 Sz^2, then a fraction `frac` of the bonds removed, every remaining
    bond given J = 1 + 0.3 ξ, a random anisotropic exchange on a few bonds, and a site-
    dependent easy axis on a quarter of the sites."""
    sys_ = sg.System(sg.cubic_crystal(), [(1, sg.Moment(s=1, g=2))], "dipole", dims=(L, L, L), seed=seed,
                     precision=precision, device=device)
    sys_.set_exchange(1.0, sg.Bond(1, 1, [1, 0, 0]))
    sys_.set_onsite_coupling(lambda Sx, Sy, Sz: -0.1 * Sz @ Sz, 1)
    sys_.randomize_spins()
    s2 = sg.to_inhomogeneous(sys_)
    rng = np.random.default_rng(seed)
    for c1 in range(1, L + 1):
        for c2 in range(1, L + 1):
            for c3 in range(1, L + 1):
                for d in range(3):
                    n = [0, 0, 0]
                    n[d] = 1
                    c = [c1, c2, c3]
                    c[d] = (c[d] % L) + 1
                    u = rng.random()
                    if u < frac:
                        Jb = 0.0
                    elif u < frac + 0.05:
                        Jb = np.eye(3) + 0.2 * rng.standard_normal((3, 3))
                    else:
                        Jb = 1.0 + 0.3 * rng.standard_normal()
                    s2.set_exchange_at(Jb, (c1, c2, c3, 1), (*c, 1), offset=n)
    Sx, Sy, Sz = sg.spin_matrices_of_dim(3)
    for i in rng.choice(s2.nsites, size=s2.nsites // 4, replace=False):
        v = rng.standard_normal(3)
        v /= np.linalg.norm(v)
        A = v[0] * Sx + v[1] * Sy + v[2] * Sz
        s2.set_onsite_coupling_at(-0.3 * A @ A, int(i))
    return s2
