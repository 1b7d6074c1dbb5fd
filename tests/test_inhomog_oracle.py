"""Inhomogeneous systems on the CPU: the host mirror of to_inhomogeneous, set_exchange_at,
set_onsite_coupling_at, set_vacancy_at and remove_periodicity, checked through the oracle
against the reference tests' known answers (test_rescaling.jl:210-250,
test_resize.jl:150-200, test_energy_consistency.jl:58-76)."""
import numpy as np
import pytest

from models import energy_consistency_inhomog, diluted_dipole, rich_dipole, rich_sun, oracle_of


def test_to_inhomogeneous_keeps_energy_and_gradient(sg, orc):
    for hom in (rich_dipole(sg, device=None), rich_sun(sg, device=None)):
        inh = sg.to_inhomogeneous(hom)
        assert not inh.is_homogeneous() and hom.is_homogeneous()
        oh, oi = oracle_of(orc, hom), oracle_of(orc, inh)
        if hom.N:
            Z = hom.coherents_flat()
            S = hom.dipoles_flat()
            assert oi.energy(S, Z) == pytest.approx(oh.energy(S, Z), rel=1e-13)
            assert np.allclose(oi.grad(Z=Z), oh.grad(Z=Z), rtol=0, atol=1e-12)
        else:
            S = hom.dipoles_flat()
            assert oi.energy(S) == pytest.approx(oh.energy(S), rel=1e-13)
            assert np.allclose(oi.grad(S), oh.grad(S), rtol=0, atol=1e-12)
    with pytest.raises(ValueError, match="already inhomogeneous"):
        sg.to_inhomogeneous(inh)


def test_inhomogeneous_spin_s_known_answer(sg, orc):
    # test_rescaling.jl:210-233: energy unchanged by to_inhomogeneous, and the same energy
    # from couplings set site by site. The reference's crystal has space group 1, so the
    # exchange sits on the one bond only (set_bond_coupling: no propagation).
    cr = sg.Crystal(sg.lattice_vectors(1, 1, 2, 90, 90, 90), [[0, 0, 0], [0, 0, 0.5]])
    mom = [(1, sg.Moment(s=1, g=2)), (2, sg.Moment(s=1.5, g=2))]
    sys_ = sg.System(cr, mom, "dipole", device=None, seed=1)
    sys_.randomize_spins()
    sys_.set_onsite_coupling(lambda Sx, Sy, Sz: Sz @ Sz, 1)
    sys_.set_onsite_coupling(lambda Sx, Sy, Sz: Sz @ Sz, 2)
    sys_.set_bond_coupling(sg.Bond(1, 2, [0, 0, 0]), 0.0, 1.0, 0.0)
    S = sys_.dipoles_flat()
    E = oracle_of(orc, sys_).energy(S)
    assert oracle_of(orc, sg.to_inhomogeneous(sys_)).energy(S) == pytest.approx(E, rel=1e-14)
    s3 = sg.to_inhomogeneous(sg.System(cr, mom, "dipole", device=None))
    s3.set_onsite_coupling_at(lambda Sx, Sy, Sz: Sz @ Sz, (1, 1, 1, 1))
    s3.set_onsite_coupling_at(lambda Sx, Sy, Sz: Sz @ Sz, (1, 1, 1, 2))
    s3.set_exchange_at(1.0, (1, 1, 1, 1), (1, 1, 1, 2), offset=(0, 0, 0))
    assert oracle_of(orc, s3).energy(S) == pytest.approx(E, rel=1e-14)
    with pytest.raises(ValueError, match="to_inhomogeneous"):
        sys_.set_exchange_at(1.0, (1, 1, 1, 1), (1, 1, 1, 2))


def test_overwrite_every_bond_doubles_energy(sg, orc):
    # test_resize.jl:150-180 (without the reshape): triangular FM, E0 = J N 6/2; setting 2J
    # on every bond site by site doubles it
    cr = sg.Crystal(sg.lattice_vectors(1, 1, 10, 90, 90, 120), [[0, 0, 0]])
    dims = (6, 6, 2)
    sys_ = sg.System(cr, [(1, sg.Moment(s=1, g=2))], "dipole", dims=dims, device=None)
    sys_.polarize_spins((0, 0, 1))
    J = 1.5
    sys_.set_exchange(J, sg.Bond(1, 1, [1, 0, 0]))
    S = sys_.dipoles_flat()
    E0 = J * np.prod(dims) * (6 / 2)
    assert oracle_of(orc, sys_).energy(S) == pytest.approx(E0, rel=1e-14)
    s2 = sg.to_inhomogeneous(sys_)
    assert oracle_of(orc, s2).energy(S) == pytest.approx(E0, rel=1e-14)
    for b in list(sys_._pairs):
        for i in range(s2.nsites):
            s2.set_exchange_at(2 * J, i, s2.bonded_site(i, b), offset=b.n)
    assert oracle_of(orc, s2).energy(S) == pytest.approx(2 * E0, rel=1e-14)


def test_remove_periodicity_known_answer(sg, orc):
    # test_resize.jl:184-200
    sys_ = sg.System(sg.cubic_crystal(), [(1, sg.Moment(s=1, g=2))], "dipole", dims=(3, 3, 3), device=None, seed=0)
    sys_.set_exchange(1.0, sg.Bond(1, 1, [1, 0, 0]))
    S = sys_.dipoles_flat()
    assert oracle_of(orc, sys_).energy(S) == pytest.approx(81)
    s2 = sg.to_inhomogeneous(sys_)
    s2.remove_periodicity((True, False, False))
    assert oracle_of(orc, s2).energy(S) == pytest.approx(72)
    s2.remove_periodicity((True, False, True))
    assert oracle_of(orc, s2).energy(S) == pytest.approx(63)


def test_vacancy_removes_the_site_from_its_neighbours(sg, orc):
    _, s2 = energy_consistency_inhomog(sg, device=None, ewald=False)
    v = s2.site_index(1, 1, 1, 2)
    assert s2.kappas[v] == 0 and np.all(s2.dipoles_flat()[v] == 0)
    for i, lst in enumerate(s2._site_pairs):
        if i != v:
            assert all(s2.bonded_site(i, b) != v for b, _, _ in lst)
    assert len(s2._site_pairs[v]) > 0            # its own list is kept, as in the reference


@pytest.mark.parametrize("mode", ["dipole", "SUN"])
def test_local_energy_change_equals_energy_difference(sg, orc, mode):
    # test_energy_consistency.jl:58-76 (its SU(N) case is the inhomogeneous one)
    if mode == "dipole":
        _, sys_ = energy_consistency_inhomog(sg, device=None, ewald=False)
    else:
        sys_ = sg.to_inhomogeneous(rich_sun(sg, device=None))
        sys_.set_exchange_at(0.3, (1, 1, 1, 1), (2, 1, 1, 2), biquad=0.2, offset=(1, 0, 0))
        sys_.set_onsite_coupling_at(lambda Sx, Sy, Sz: 0.3 * Sx @ Sx, (1, 2, 1, 2))
        sys_.set_vacancy_at((2, 3, 2, 1))
    o = oracle_of(orc, sys_)
    rng = np.random.default_rng(3)
    S = sys_.dipoles_flat()
    Z = sys_.coherents_flat() if sys_.N else None
    kap = sys_.kappas
    for _ in range(5):
        i = int(rng.integers(0, sys_.nsites))
        if sys_.N:
            zn = rng.standard_normal(sys_.N) + 1j * rng.standard_normal(sys_.N)
            zn *= np.sqrt(kap[i]) / np.linalg.norm(zn)
            dE = o.local_energy_change(S, i, zn, Z=Z)
            Z1 = Z.copy()
            Z1[i] = zn
            S1 = o.expected_spin(Z1)
            ref = o.energy(S1, Z1) - o.energy(S, Z)
        else:
            v = rng.standard_normal(3)
            Sn = kap[i] * v / np.linalg.norm(v)
            dE = o.local_energy_change(S, i, Sn)
            S1 = S.copy()
            S1[i] = Sn
            ref = o.energy(S1) - o.energy(S)
        assert dE == pytest.approx(ref, abs=1e-12)


def test_inhomogeneous_gradient_matches_finite_differences(sg, orc):
    sys_ = diluted_dipole(sg, device=None, L=3)
    o = oracle_of(orc, sys_)
    S = sys_.dipoles_flat()
    g = o.grad(S)
    rng = np.random.default_rng(1)
    h = 1e-6
    for _ in range(6):
        # along a direction tangent to the sphere: the classical Stevens gradient omits the
        # |S|^2 dependence (OnsiteCoupling.jl:316-425), which is constant on the sphere
        i = int(rng.integers(0, sys_.nsites))
        t = np.cross(S[i], rng.standard_normal(3))
        t /= np.linalg.norm(t)
        Sp, Sm = S.copy(), S.copy()
        Sp[i] += h * t
        Sm[i] -= h * t
        fd = (o.energy(Sp) - o.energy(Sm)) / (2 * h)
        assert g[i] @ t == pytest.approx(fd, abs=1e-6)
