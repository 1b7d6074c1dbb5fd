"""SU(N) general pair couplings (Σ_k A_k ⊗ B_k, Types.jl:23-30) on the GPU against the
oracle: HZ and energy (Interactions.jl:486-505, 660-666), the Langevin and Schrödinger-
midpoint steps, and local_energy_change (Interactions.jl:364-370)."""
import numpy as np
import pytest

from models import rich_sun, oracle_of

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def general_model(sg, N=3, precision="fp64", seed=4, dims=(2, 3, 2)):
    """rich_sun plus two non-separable couplings: a random Hermitian operator on the
    product space of Bond(1, 2, [0,0,0]) and (Si·Sj)^3 on Bond(1, 1, [1,0,0])."""
    s = rich_sun(sg, N=N, precision=precision, seed=seed, dims=dims)
    rng = np.random.default_rng(seed + 100)
    H = rng.standard_normal((N * N, N * N)) + 1j * rng.standard_normal((N * N, N * N))
    s.set_pair_coupling_op(0.05 * (H + H.conj().T), sg.Bond(1, 2, [0, 0, 0]))
    s.set_pair_coupling_op(lambda Si, Sj: 0.01 * np.linalg.matrix_power(sum(a @ b for a, b in zip(Si, Sj)), 3),
                           sg.Bond(1, 1, [1, 0, 0]))
    s.randomize_spins()
    return s


@pytest.mark.parametrize("N", [3, 4])
def test_hz_and_energy_parity(gpu, sg, orc, N):
    s = general_model(sg, N=N)
    o = oracle_of(orc, s)
    Z, S = s.coherents_flat(), s.dipoles_flat()
    hz = sg.energy_grad(s)
    hz = hz[..., 0] + 1j * hz[..., 1] if hz.ndim == 3 else hz
    ref = o.grad(Z=Z)
    assert np.max(np.abs(hz - ref)) <= 1e-12 * max(1.0, np.max(np.abs(ref)))
    assert sg.energy(s) == pytest.approx(o.energy(S, Z), rel=1e-12, abs=1e-12)


def test_dynamics_parity(gpu, sg, orc):
    s = general_model(sg, N=3)
    o = oracle_of(orc, s)
    Z0 = s.coherents_flat()
    rng = np.random.default_rng(1)
    noise = (rng.standard_normal((10, s.nsites, 3)) + 1j * rng.standard_normal((10, s.nsites, 3))) / np.sqrt(2)
    sg.step(s, sg.Langevin(0.01, damping=0.1, kT=0.3), nsteps=10, noise=noise)
    _, Z_ref = o.langevin(o.expected_spin(Z0), Z0, 0.01, 0.1, 0.3, 10, noise)
    assert rel(s.coherents_flat(), Z_ref) < 1e-11
    Z1 = s.coherents_flat()
    sg.step(s, sg.ImplicitMidpoint(0.01), nsteps=10)
    st, _, Z_ref, _ = o.midpoint(o.expected_spin(Z1), Z1, 0.01, 0.0, 1e-12, 100, 10)
    assert st == 0
    assert rel(s.coherents_flat(), Z_ref) < 1e-9


def test_local_energy_change(gpu, sg, orc):
    s = general_model(sg, N=3, dims=(3, 3, 2))
    o = oracle_of(orc, s)
    Z, S = s.coherents_flat(), s.dipoles_flat()
    rng = np.random.default_rng(2)
    for _ in range(5):
        i = int(rng.integers(0, s.nsites))
        zn = rng.standard_normal(3) + 1j * rng.standard_normal(3)
        zn /= np.linalg.norm(zn)
        assert sg.local_energy_change(s, i, zn) == pytest.approx(o.local_energy_change(S, i, zn, Z=Z), abs=1e-12)


def test_fp32_general(gpu, sg):
    s64 = general_model(sg, N=3)
    s32 = general_model(sg, N=3, precision="fp32")
    s32.set_state_flat(coherents=s64.coherents_flat())
    assert rel(sg.energy_grad(s32), sg.energy_grad(s64)) < 1e-5
    assert sg.energy(s32) == pytest.approx(sg.energy(s64), rel=1e-5)
