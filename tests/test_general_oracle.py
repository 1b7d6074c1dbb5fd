"""SU(N) general pair couplings (Σ_k A_k ⊗ B_k, Types.jl:23-30) in the oracle and the host
mirror: the decomposition, the energy (Interactions.jl:495-503), HZ (Interactions.jl:660-666)
and local_energy_change (Interactions.jl:364-370)."""
import numpy as np
import pytest

from models import oracle_of


def two_site(sg, N=3, op=None, seed=0, dims=(1, 1, 1)):
    cr = sg.Crystal(sg.lattice_vectors(1, 1.1, 1.2, 90, 90, 90), [[0, 0, 0], [0.5, 0.5, 0.3]])
    s = sg.System(cr, [(1, sg.Moment(s=(N - 1) / 2, g=2))], "SUN", dims=dims, seed=seed, device=None)
    if op is not None:
        s.set_pair_coupling_op(op, sg.Bond(1, 2, [0, 0, 0]))
    s.randomize_spins()
    return s


def random_hermitian(rng, n):
    H = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    return (H + H.conj().T) / 2


@pytest.mark.parametrize("N", [2, 3, 4])
def test_decomposition_rebuilds_the_operator(sg, N):
    rng = np.random.default_rng(N)
    op = random_hermitian(rng, N * N)
    terms = sg.tensor_decomposition(op, N, N)
    assert np.allclose(sum(np.kron(a, b) for a, b in terms), op, atol=1e-12)
    for a, b in terms:
        assert np.allclose(a, a.conj().T) and np.allclose(b, b.conj().T)


@pytest.mark.parametrize("N", [3, 4])
def test_energy_is_the_product_state_expectation(sg, orc, N):
    rng = np.random.default_rng(10 + N)
    op = random_hermitian(rng, N * N)
    s = two_site(sg, N, op, seed=N)
    Z = s.coherents_flat()
    o = oracle_of(orc, s)
    psi = np.kron(Z[0], Z[1])
    assert o.energy(s.dipoles_flat(), Z) == pytest.approx(np.vdot(psi, op @ psi).real, rel=1e-12, abs=1e-12)


def test_bilinear_as_general_equals_bilinear(sg, orc):
    # J Si·Sj entered as a general operator gives the energy and HZ of the bilinear coupling
    N = 3
    J = np.array([[0.3, 0.1, 0.0], [0.1, -0.2, 0.05], [0.0, 0.05, 0.4]])
    a = two_site(sg, N, seed=2)
    a.set_bond_coupling(sg.Bond(1, 2, [0, 0, 0]), 0.0, J, 0.0)
    b = two_site(sg, N, lambda Si, Sj: sum(J[p, q] * Si[p] @ Sj[q] for p in range(3) for q in range(3)), seed=2)
    b.set_state_flat(coherents=a.coherents_flat())
    oa, ob = oracle_of(orc, a), oracle_of(orc, b)
    Z, S = a.coherents_flat(), a.dipoles_flat()
    assert ob.energy(S, Z) == pytest.approx(oa.energy(S, Z), rel=1e-12)
    assert np.allclose(ob.grad(Z=Z), oa.grad(Z=Z), atol=1e-12)


def test_hz_is_the_energy_derivative(sg, orc):
    N = 4
    rng = np.random.default_rng(3)
    s = two_site(sg, N, random_hermitian(rng, N * N), seed=3, dims=(2, 1, 1))
    s.set_pair_coupling_op(random_hermitian(rng, N * N), sg.Bond(1, 1, [1, 0, 0]))
    o = oracle_of(orc, s)
    Z = s.coherents_flat()
    HZ = o.grad(Z=Z)
    h = 1e-6
    for _ in range(4):
        d = rng.standard_normal(Z.shape) + 1j * rng.standard_normal(Z.shape)
        Zp, Zm = Z + h * d, Z - h * d
        fd = (o.energy(o.expected_spin(Zp), Zp) - o.energy(o.expected_spin(Zm), Zm)) / (2 * h)
        assert fd == pytest.approx(2 * np.vdot(HZ, d).real, rel=1e-6, abs=1e-8)


def test_local_energy_change_with_general_terms(sg, orc):
    N = 3
    rng = np.random.default_rng(5)
    s = two_site(sg, N, random_hermitian(rng, N * N), seed=5, dims=(3, 2, 2))
    s.set_pair_coupling_op(random_hermitian(rng, N * N), sg.Bond(1, 1, [1, 0, 0]))
    o = oracle_of(orc, s)
    Z, S = s.coherents_flat(), s.dipoles_flat()
    for _ in range(5):
        i = int(rng.integers(0, s.nsites))
        zn = rng.standard_normal(N) + 1j * rng.standard_normal(N)
        zn /= np.linalg.norm(zn)
        Z1 = Z.copy()
        Z1[i] = zn
        ref = o.energy(o.expected_spin(Z1), Z1) - o.energy(S, Z)
        assert o.local_energy_change(S, i, zn, Z=Z) == pytest.approx(ref, abs=1e-12)
