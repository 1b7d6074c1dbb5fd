"""SU(N) coherent-state parity of the CUDA path against the FP64 CPU oracle."""
import numpy as np
import pytest

from models import rich_sun, triangular_c3, oracle_of

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.max(np.abs(a - b)) / max(1e-300, np.max(np.abs(b)))


@pytest.mark.parametrize("N", [3, 4, 5])
@pytest.mark.parametrize("biquad", [True, False])
def test_hz_and_energy_fp64(gpu, sg, orc, N, biquad):
    sys_ = rich_sun(sg, N=N, biquad=biquad)
    o = oracle_of(orc, sys_)
    Z = sys_.coherents_flat()
    S = sys_.dipoles_flat()
    assert np.allclose(S, sg.expected_spin(Z), atol=1e-13)
    hz = sg.energy_grad(sys_)
    assert rel(hz, o.grad(Z=Z)) < 1e-12
    assert sg.energy(sys_) == pytest.approx(o.energy(S, Z), rel=1e-12, abs=1e-12)


@pytest.mark.parametrize("N", [3, 5])
def test_heun_injected_noise_fp64(gpu, sg, orc, N):
    sys_ = rich_sun(sg, N=N)
    o = oracle_of(orc, sys_)
    Z0, S0 = sys_.coherents_flat(), sys_.dipoles_flat()
    rng = np.random.default_rng(N)
    noise = (rng.standard_normal((25, sys_.nsites, N)) + 1j * rng.standard_normal((25, sys_.nsites, N))) / np.sqrt(2)
    sg.step(sys_, sg.Langevin(0.01, damping=0.1, kT=0.3), nsteps=25, noise=noise)
    S_ref, Z_ref = o.langevin(S0, Z0, 0.01, 0.1, 0.3, 25, noise)
    assert rel(sys_.coherents_flat(), Z_ref) < 1e-11
    assert rel(sys_.dipoles_flat(), S_ref) < 1e-11


@pytest.mark.parametrize("N", [3, 4])
def test_midpoint_fp64(gpu, sg, orc, N):
    sys_ = rich_sun(sg, N=N)
    o = oracle_of(orc, sys_)
    Z0, S0 = sys_.coherents_flat(), sys_.dipoles_flat()
    sg.step(sys_, sg.ImplicitMidpoint(0.01), nsteps=30)
    st, S_ref, Z_ref, _ = o.midpoint(S0, Z0, 0.01, 0.0, 1e-12, 100, 30)
    assert st == 0
    assert rel(sys_.coherents_flat(), Z_ref) < 1e-9
    assert rel(sys_.dipoles_flat(), S_ref) < 1e-9
    # κ invariance |Z|^2 = κ (test_rescaling.jl:10-29)
    assert np.allclose(np.sum(np.abs(sys_.coherents_flat()) ** 2, axis=1), sys_.kappas, rtol=1e-12)


def test_sun_thermal_energy_device_noise(gpu, sg):
    # test_samplers.jl:5-9, 64-88: SU(3) single-ion D Sz^2, Langevin with device noise
    D, kT = 1.0, 0.5
    a = D / kT
    E_ref = D * (2 - (2 + 2 * a + a**2) * np.exp(-a)) / (a * (1 - (1 + a) * np.exp(-a)))
    sys_ = sg.System(sg.cubic_crystal(), [(1, sg.Moment(s=1, g=2))], "SUN", dims=(20, 1, 1), seed=0)
    sys_.set_onsite_coupling(lambda Sx, Sy, Sz: D * Sz @ Sz, 1)
    sys_.randomize_spins()
    integ = sg.Langevin(0.01, damping=1.0, kT=kT)
    sg.step(sys_, integ, nsteps=1000)
    Es = []
    for _ in range(1000):
        sg.step(sys_, integ, nsteps=10)
        Es.append(sg.energy_per_site(sys_))
    assert np.mean(Es) == pytest.approx(E_ref, rel=0.1)


def test_triangular_fp32_vs_fp64(gpu, sg, orc):
    s64 = triangular_c3(sg, L=(6, 6, 2), precision="fp64", seed=3)
    s32 = triangular_c3(sg, L=(6, 6, 2), precision="fp32", seed=3)
    s32.set_state_flat(coherents=s64.coherents_flat())
    o = oracle_of(orc, s64)
    Z0, S0 = s64.coherents_flat(), s64.dipoles_flat()
    rng = np.random.default_rng(0)
    noise = (rng.standard_normal((1, s64.nsites, 3)) + 1j * rng.standard_normal((1, s64.nsites, 3))) / np.sqrt(2)
    sg.step(s32, sg.Langevin(0.02, damping=0.1, kT=0.3), noise=noise)
    S_ref, Z_ref = o.langevin(S0, Z0, 0.02, 0.1, 0.3, 1, noise)
    assert rel(s32.coherents_flat(), Z_ref) < 1e-5
    assert sg.energy(s32) == pytest.approx(o.energy(s32.dipoles_flat(), s32.coherents_flat()), rel=1e-5)


@pytest.mark.parametrize("N", [3, 4])
def test_heun_cluster_kernel_matches_grid_and_oracle(gpu, sg, orc, N):
    # SU(N) Langevin with the lattice held by one thread-block cluster: same trajectory as
    # the persistent grid kernel and the FP64 oracle, biquadratic couplings included
    a, b = rich_sun(sg, N=N, biquad=N == 3), rich_sun(sg, N=N, biquad=N == 3)
    o = oracle_of(orc, a)
    Z0 = a.coherents_flat()
    rng = np.random.default_rng(31)
    noise = (rng.standard_normal((10, a.nsites, N)) + 1j * rng.standard_normal((10, a.nsites, N))) / np.sqrt(2)
    a.set_langevin_cluster(0)
    b.set_langevin_cluster(1)
    integ = sg.Langevin(0.01, damping=0.1, kT=0.3)
    sg.step(a, integ, 10, noise)
    sg.step(b, integ, 10, noise)
    _, Zref = o.langevin(o.expected_spin(Z0), Z0, 0.01, 0.1, 0.3, 10, noise)
    assert rel(b.coherents_flat(), a.coherents_flat()) < 1e-12
    assert rel(b.coherents_flat(), Zref) < 1e-11
    assert rel(b.dipoles_flat(), o.expected_spin(Zref)) < 1e-11


def test_heun_cluster_kernel_fp32_triangular(gpu, sg):
    a, b = triangular_c3(sg, L=(12, 12, 4)), triangular_c3(sg, L=(12, 12, 4))
    a.set_langevin_cluster(0)
    b.set_langevin_cluster(1)
    integ = sg.Langevin(0.02, damping=0.1, kT=0.3)
    sg.step(a, integ, 30)
    sg.step(b, integ, 30)
    assert rel(b.coherents_flat(), a.coherents_flat()) < 1e-4
