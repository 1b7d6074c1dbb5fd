"""Inhomogeneous systems (to_inhomogeneous, set_exchange_at, set_onsite_coupling_at,
set_vacancy_at, remove_periodicity) on the GPU, through the C ABI's per-site couplings
(sgb_set_bonds_at, sgb_set_onsite_at), against the FP64 oracle's restatement of the
reference's per-site loops (Interactions.jl:433-440, 535-540, 311-373)."""
import numpy as np
import pytest

from models import energy_consistency_inhomog, diluted_dipole, rich_sun, oracle_of

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("builder", ["consistency", "diluted"])
def test_gradient_and_energy_parity(gpu, sg, orc, builder):
    sys_ = energy_consistency_inhomog(sg, ewald=False)[1] if builder == "consistency" else diluted_dipole(sg)
    o = oracle_of(orc, sys_)
    S = sys_.dipoles_flat()
    g = sg.energy_grad(sys_)
    assert np.max(np.abs(g - o.grad(S))) <= 1e-12 * max(1.0, np.max(np.abs(g)))
    assert sg.energy(sys_) == pytest.approx(o.energy(S), rel=1e-12, abs=1e-12)


def test_homogeneous_and_inhomogeneous_agree_on_the_gpu(gpu, sg):
    hom, _ = energy_consistency_inhomog(sg, ewald=True)
    inh = sg.to_inhomogeneous(hom)
    assert sg.energy(inh) == pytest.approx(sg.energy(hom), rel=1e-12)
    assert rel(sg.energy_grad(inh), sg.energy_grad(hom)) < 1e-12


def test_langevin_and_midpoint_parity(gpu, sg, orc):
    sys_ = diluted_dipole(sg, L=5)
    o = oracle_of(orc, sys_)
    S0 = sys_.dipoles_flat()
    rng = np.random.default_rng(7)
    noise = rng.standard_normal((50, sys_.nsites, 3))
    sg.step(sys_, sg.Langevin(0.02, damping=0.1, kT=0.4), nsteps=50, noise=noise)
    S_ref, _ = o.langevin(S0, None, 0.02, 0.1, 0.4, 50, noise)
    assert rel(sys_.dipoles_flat(), S_ref) < 1e-11
    S1 = sys_.dipoles_flat()
    sg.step(sys_, sg.ImplicitMidpoint(0.02), nsteps=20)
    st, S_ref, _, _ = o.midpoint(S1, None, 0.02, 0.0, 1e-12, 100, 20)
    assert st == 0
    assert rel(sys_.dipoles_flat(), S_ref) < 1e-9


def test_midpoint_energy_conservation_inhomogeneous(gpu, sg):
    # test_energy_consistency.jl:37-55 with make_system(mode=:dipole, inhomog=true), dipole-
    # dipole interactions included: (max - min)/sqrt(N) of E along 1500 steps < 1e-3
    _, sys_ = energy_consistency_inhomog(sg, ewald=True)
    integ = sg.ImplicitMidpoint(0.002)
    Es = []
    for _ in range(1500):
        sg.step(sys_, integ)
        Es.append(sg.energy(sys_))
    assert (max(Es) - min(Es)) / np.sqrt(sys_.nsites) < 1e-3
    S = sys_.dipoles_flat()
    assert np.allclose(np.linalg.norm(S, axis=1), sys_.kappas, rtol=1e-10, atol=1e-14)


def test_fp32_inhomogeneous_steps(gpu, sg):
    s64 = diluted_dipole(sg, L=5, precision="fp64")
    s32 = diluted_dipole(sg, L=5, precision="fp32")
    s32.set_state_flat(dipoles=s64.dipoles_flat())
    assert rel(sg.energy_grad(s32), sg.energy_grad(s64)) < 1e-5
    rng = np.random.default_rng(2)
    noise = rng.standard_normal((1, s64.nsites, 3))
    for s in (s32, s64):
        sg.step(s, sg.Langevin(0.02, damping=0.1, kT=0.4), noise=noise)
    assert rel(s32.dipoles_flat(), s64.dipoles_flat()) < 1e-5
    for _ in range(20):
        sg.step(s32, sg.ImplicitMidpoint(0.02, tol=1e-6))
        sg.step(s64, sg.ImplicitMidpoint(0.02))
        assert abs(sg.energy(s32) - sg.energy(s64)) / abs(sg.energy(s64)) < 1e-5


@pytest.mark.parametrize("mode", ["dipole", "SUN"])
def test_local_energy_change_and_sweeps(gpu, sg, orc, mode):
    if mode == "dipole":
        sys_ = diluted_dipole(sg, L=4)
    else:
        sys_ = sg.to_inhomogeneous(rich_sun(sg))
        sys_.set_exchange_at(0.3, (1, 1, 1, 1), (2, 1, 1, 2), biquad=0.2, offset=(1, 0, 0))
        sys_.set_onsite_coupling_at(lambda Sx, Sy, Sz: 0.3 * Sx @ Sx, (1, 2, 1, 2))
        sys_.set_vacancy_at((2, 3, 2, 1))
    o = oracle_of(orc, sys_)
    rng = np.random.default_rng(4)
    S = sys_.dipoles_flat()
    Z = sys_.coherents_flat() if sys_.N else None
    kap = sys_.kappas
    for _ in range(5):
        i = int(rng.integers(0, sys_.nsites))
        if sys_.N:
            zn = rng.standard_normal(sys_.N) + 1j * rng.standard_normal(sys_.N)
            zn *= np.sqrt(kap[i]) / np.linalg.norm(zn)
            ref = o.local_energy_change(S, i, zn, Z=Z)
            got = sg.local_energy_change(sys_, i, zn)
        else:
            v = rng.standard_normal(3)
            Sn = kap[i] * v / np.linalg.norm(v)
            ref = o.local_energy_change(S, i, Sn)
            got = sg.local_energy_change(sys_, i, Sn)
        assert got == pytest.approx(ref, abs=1e-12 * max(1.0, abs(sg.energy(sys_))))
    if mode == "dipole":
        # sweeps with caller randoms: the GPU's colour-class order replayed on the oracle
        ncol, col = sg.local_colors(sys_)
        order = np.lexsort((np.arange(sys_.nsites), col))
        rnd = np.concatenate([rng.standard_normal((2, sys_.nsites, 3)), rng.random((2, sys_.nsites, 3))], axis=2)
        prop = sg.propose_delta(0.4)
        smp = sg.LocalSampler(kT=0.5, nsweeps=2, propose=prop)
        sg.step(sys_, smp, 1, rnd)
        S_ref, dE_ref, _ = o.local_sweeps(S, 0.5, 2, 1.0, order, prop.terms, rnd)
        assert np.max(np.abs(sys_.dipoles_flat() - S_ref)) < 1e-12 * np.max(np.abs(S_ref))
        assert smp.ΔE == pytest.approx(dE_ref, abs=1e-10)
