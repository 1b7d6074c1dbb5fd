"""Dipole-mode parity of the CUDA path (through the C ABI) against the FP64 CPU oracle.

Tolerances: FP64 kernels agree with the oracle to rounding (1e-12 relative for one step /
one gradient); after 1000 Langevin steps the trajectory agrees to 1e-5 relative, the bar
of the reference's own oracle for chaotic trajectories. FP32 kernels are judged per step
(1e-5) and on FP64-reduced energies (1e-5 relative).
"""
import numpy as np
import pytest

from models import sc_c1, rich_dipole, pyrochlore_c2, oracle_of

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.max(np.abs(a - b)) / max(1e-300, np.max(np.abs(b)))


@pytest.mark.parametrize("builder", ["rich", "rich_nomatrix", "sc", "wrap"])
def test_gradient_and_energy_fp64(gpu, sg, orc, builder):
    if builder == "rich":
        sys_ = rich_dipole(sg)
    elif builder == "rich_nomatrix":
        sys_ = rich_dipole(sg, dims=(1, 1, 2), biquad_matrix=False)
    elif builder == "sc":
        sys_ = sc_c1(sg, L=5)
    else:
        # L=1 and L=2 axes: bonds wrap onto the site itself or onto the same neighbour twice
        sys_ = sg.System(sg.cubic_crystal(), [(1, sg.Moment(s=2, g=2))], "dipole", dims=(1, 2, 3), seed=5)
        sys_.set_exchange(0.8, sg.Bond(1, 1, [1, 0, 0]))
        sys_.set_bond_coupling(sg.Bond(1, 1, [1, 1, 0]), 0.2, np.array([[0.1, 0.2, 0.3], [0.0, -0.4, 0.5], [0.6, 0.0, 0.7]]), 0.3)
        sys_.set_bond_coupling(sg.Bond(1, 1, [0, 2, 1]), 0.0, 0.5, 0.0)
        sys_.randomize_spins()
    o = oracle_of(orc, sys_)
    S = sys_.dipoles_flat()
    g_gpu = sg.energy_grad(sys_)
    g_ref = o.grad(S)
    assert rel(g_gpu, g_ref) < 1e-12
    E_gpu, E_ref = sg.energy(sys_), o.energy(S)
    assert E_gpu == pytest.approx(E_ref, rel=1e-12, abs=1e-12)
    M = sg.magnetization(sys_)
    assert np.allclose(M, S.sum(axis=0), rtol=1e-12, atol=1e-12)


def test_langevin_injected_noise_fp64(gpu, sg, orc):
    sys_ = rich_dipole(sg)
    o = oracle_of(orc, sys_)
    rng = np.random.default_rng(0)
    S0 = sys_.dipoles_flat()
    noise = rng.standard_normal((1, sys_.nsites, 3))
    sg.step(sys_, sg.Langevin(0.01, damping=0.1, kT=0.3), noise=noise)
    S1, _ = o.langevin(S0, None, 0.01, 0.1, 0.3, 1, noise)
    assert rel(sys_.dipoles_flat(), S1) < 1e-12
    noise = rng.standard_normal((40, sys_.nsites, 3))
    sg.step(sys_, sg.Langevin(0.01, damping=0.1, kT=0.3), nsteps=40, noise=noise)
    S2, _ = o.langevin(S1, None, 0.01, 0.1, 0.3, 40, noise)
    assert rel(sys_.dipoles_flat(), S2) < 1e-11


def test_langevin_1000_steps_fp64_c1_model(gpu, sg, orc):
    # 8^3 version of the simple-cubic workload, 1000 steps with identical noise: 1e-5 relative
    sys_ = sc_c1(sg, L=8)
    o = oracle_of(orc, sys_)
    S0 = sys_.dipoles_flat()
    rng = np.random.default_rng(1)
    noise = rng.standard_normal((1000, sys_.nsites, 3))
    sg.step(sys_, sg.Langevin(0.02, damping=0.1, kT=0.5), nsteps=1000, noise=noise)
    S_ref, _ = o.langevin(S0, None, 0.02, 0.1, 0.5, 1000, noise)
    assert rel(sys_.dipoles_flat(), S_ref) < 1e-5
    assert sg.energy(sys_) == pytest.approx(o.energy(S_ref), rel=1e-5)


def test_device_noise_replays_on_oracle(gpu, sg, orc):
    sys_ = sc_c1(sg, L=6, seed=7)
    o = oracle_of(orc, sys_)
    S0 = sys_.dipoles_flat()
    step0 = sys_.noise_step
    sg.step(sys_, sg.Langevin(0.02, damping=0.1, kT=0.5), nsteps=30)
    noise = np.stack([sg.langevin_noise(sys_, step0 + k) for k in range(30)])
    S_ref, _ = o.langevin(S0, None, 0.02, 0.1, 0.5, 30, noise)
    assert rel(sys_.dipoles_flat(), S_ref) < 1e-11


def test_device_noise_statistics(gpu, sg):
    sys_ = sc_c1(sg, L=32)
    x = np.concatenate([sg.langevin_noise(sys_, k).ravel() for k in range(4)])
    assert abs(x.mean()) < 0.01
    assert x.std() == pytest.approx(1.0, abs=0.01)
    # distinct steps give independent draws
    a, b = sg.langevin_noise(sys_, 0).ravel(), sg.langevin_noise(sys_, 1).ravel()
    assert abs(np.corrcoef(a, b)[0, 1]) < 0.02


def test_midpoint_fp64(gpu, sg, orc):
    sys_ = rich_dipole(sg)
    o = oracle_of(orc, sys_)
    S0 = sys_.dipoles_flat()
    it = sg.step(sys_, sg.ImplicitMidpoint(0.01), nsteps=50)
    st, S_ref, _, it_ref = o.midpoint(S0, None, 0.01, 0.0, 1e-12, 100, 50)
    assert st == 0
    assert rel(sys_.dipoles_flat(), S_ref) < 1e-9
    # same fixed-point iteration counts, up to rounding at the convergence threshold
    assert abs(it - it_ref) <= 2
    # damped midpoint (damping > 0 with kT = 0)
    S1 = sys_.dipoles_flat()
    sg.step(sys_, sg.ImplicitMidpoint(0.01, damping=0.2), nsteps=20)
    st, S_ref, _, _ = o.midpoint(S1, None, 0.01, 0.2, 1e-12, 100, 20)
    assert rel(sys_.dipoles_flat(), S_ref) < 1e-9


def test_midpoint_energy_conservation_gpu(gpu, sg):
    # test_energy_consistency.jl:37-55 on the GPU path, FP64: s=2 diamond with exchange,
    # quartic anisotropy and a field
    sys_ = sg.System(sg.diamond_crystal(), [(1, sg.Moment(s=2, g=2))], "dipole", dims=(2, 2, 2), seed=0)
    sys_.set_exchange(0.5, sg.Bond(1, 2, [0, 0, 0]))
    O4 = sg.stevens_matrices_of_dim(4, 5)
    for a in range(1, 9):
        sys_.set_onsite_coupling(0.2 * ((1 / 20) * O4[4] + (1 / 4) * O4[0]), a)
    sys_.set_field([0.0, 0.2, 0.3])
    sys_.randomize_spins()
    Es = []
    integ = sg.ImplicitMidpoint(0.002)
    for _ in range(150):
        sg.step(sys_, integ, nsteps=10)
        Es.append(sg.energy(sys_))
    assert (max(Es) - min(Es)) / np.sqrt(sys_.nsites) < 1e-3


def test_midpoint_nonconvergence_reports_error(gpu, sg):
    sys_ = sc_c1(sg, L=4)
    S0 = sys_.dipoles_flat()
    with pytest.raises(sg.SunnyGPUError, match="failed to converge") as ei:
        sg.step(sys_, sg.ImplicitMidpoint(0.05, tol=0.0), max_iters=3)
    assert ei.value.code == -3
    # the failed step leaves the state unchanged, and the handle stays usable
    assert np.array_equal(sys_.dipoles_flat(), S0)
    sg.step(sys_, sg.ImplicitMidpoint(0.05), nsteps=2)


def test_bounded_wait_times_out_and_handle_survives(gpu, sg):
    # a barrier that expects one more CTA than it launches can only end at the wait limit
    import time
    sys_ = sc_c1(sg, L=4)
    sys_._sync_to_device()
    sys_.set_wait_limit(1e-3)
    t0 = time.perf_counter()
    rc = sys_._lib.sgb_wait_probe(sys_.handle)
    took = time.perf_counter() - t0
    assert rc == sg._abi.SGB_ERR_TIMEOUT
    assert b"timed out" in sys_._lib.sgb_last_error(sys_.handle)
    assert took < 1.0            # the 1 ms limit, not the 4 s default
    # the next calls on the handle run normally, under the limit and after restoring it
    S0 = sys_.dipoles_flat()
    sg.step(sys_, sg.ImplicitMidpoint(0.02), nsteps=3)
    assert not np.array_equal(sys_.dipoles_flat(), S0)
    sys_.set_wait_limit(0)
    sg.step(sys_, sg.Langevin(0.02, damping=0.1, kT=0.5), nsteps=3)
    assert np.isfinite(sg.energy(sys_))


def test_kappa_and_vacancy_invariants(gpu, sg):
    # test_rescaling.jl:10-29: |S| = κ preserved; κ = 0 sites stay empty
    sys_ = rich_dipole(sg)
    kap = sys_.kappas.copy()
    kap[5] = 0.0
    sys_.set_kappas(kap)
    sg.step(sys_, sg.Langevin(0.005, damping=0.1, kT=0.1), nsteps=100)
    sg.step(sys_, sg.ImplicitMidpoint(0.005, damping=0.1), nsteps=20)
    S = sys_.dipoles_flat()
    assert np.allclose(np.linalg.norm(S, axis=1), kap, rtol=1e-12, atol=1e-14)
    assert np.all(S[5] == 0)


def test_fp32_path_per_step_and_energy(gpu, sg, orc):
    sys64 = pyrochlore_c2(sg, L=3, precision="fp64", seed=2)
    sys32 = pyrochlore_c2(sg, L=3, precision="fp32", seed=2)
    S0 = sys64.dipoles_flat()
    sys32.set_state_flat(dipoles=S0)
    o = oracle_of(orc, sys64)
    rng = np.random.default_rng(3)
    noise = rng.standard_normal((1, sys64.nsites, 3))
    sg.step(sys32, sg.Langevin(0.025, damping=0.1, kT=0.2), noise=noise)
    S1, _ = o.langevin(S0, None, 0.025, 0.1, 0.2, 1, noise)
    assert rel(sys32.dipoles_flat(), S1) < 1e-5
    # energy of the FP32 state, reduced in FP64, against the FP64 oracle on the same state
    S = sys32.dipoles_flat()
    assert sg.energy(sys32) == pytest.approx(o.energy(S), rel=1e-5)
    # midpoint with a precision-aware tolerance, from a thermalised state: step by step,
    # the FP32 energy stays within 1e-5 relative of the FP64 path's from the same state (the
    # method's own O(dt^2) energy oscillation is common to both)
    sg.step(sys64, sg.Langevin(0.025, damping=0.1, kT=0.2), nsteps=500)
    sys32.set_state_flat(dipoles=sys64.dipoles_flat())
    for _ in range(20):
        sg.step(sys32, sg.ImplicitMidpoint(0.025, tol=1e-6))
        sg.step(sys64, sg.ImplicitMidpoint(0.025))
        assert abs(sg.energy(sys32) - sg.energy(sys64)) / abs(sg.energy(sys64)) < 1e-5


def test_pyrochlore_fp64_langevin_parity(gpu, sg, orc):
    sys_ = pyrochlore_c2(sg, L=2, precision="fp64", seed=9)
    o = oracle_of(orc, sys_)
    S0 = sys_.dipoles_flat()
    rng = np.random.default_rng(4)
    noise = rng.standard_normal((20, sys_.nsites, 3))
    sg.step(sys_, sg.Langevin(0.025, damping=0.1, kT=0.2), nsteps=20, noise=noise)
    S_ref, _ = o.langevin(S0, None, 0.025, 0.1, 0.2, 20, noise)
    assert rel(sys_.dipoles_flat(), S_ref) < 1e-11


@pytest.mark.parametrize("builder", ["rich", "sc"])
def test_langevin_cluster_kernel_matches_grid_and_oracle(gpu, sg, orc, builder):
    # the cluster-resident Heun kernel (small lattices in distributed shared memory) and
    # the persistent grid kernel give the same FP64 trajectory as the oracle
    def make():
        return rich_dipole(sg) if builder == "rich" else sc_c1(sg, L=8)
    a, b = make(), make()
    o = oracle_of(orc, a)
    S0 = a.dipoles_flat()
    noise = np.random.default_rng(21).standard_normal((20, a.nsites, 3))
    a.set_langevin_cluster(0)
    b.set_langevin_cluster(1)
    integ = sg.Langevin(0.02, damping=0.1, kT=0.5)
    sg.step(a, integ, 20, noise)
    sg.step(b, integ, 20, noise)
    ref, _ = o.langevin(S0, None, 0.02, 0.1, 0.5, 20, noise)
    assert rel(b.dipoles_flat(), a.dipoles_flat()) < 1e-12
    assert rel(b.dipoles_flat(), ref) < 1e-12


def test_langevin_cluster_kernel_fp32_device_noise(gpu, sg):
    a, b = sc_c1(sg, L=16, precision="fp32"), sc_c1(sg, L=16, precision="fp32")
    a.set_langevin_cluster(0)
    b.set_langevin_cluster(1)
    integ = sg.Langevin(0.02, damping=0.1, kT=0.5)
    sg.step(a, integ, 50)
    sg.step(b, integ, 50)
    assert rel(b.dipoles_flat(), a.dipoles_flat()) < 1e-5
    assert a.langevin_kernel() == 0 and b.langevin_kernel() == 16   # 4,096 sites: 16 CTAs of 256
    # the timed choice runs every candidate on a copy of the state and leaves it unchanged
    c, c2 = sc_c1(sg, L=16, precision="fp32"), sc_c1(sg, L=16, precision="fp32")
    assert c.langevin_kernel() == -1
    c2.set_langevin_cluster(0)
    sg.step(c, integ, 30)
    sg.step(c2, integ, 30)
    assert c.langevin_kernel() in (0, 4, 8, 16)
    assert rel(c.dipoles_flat(), c2.dipoles_flat()) < 1e-5
