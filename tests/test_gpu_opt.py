"""minimize_energy on the GPU (dipole modes, FP64) against the reference's known answers
(test_optimization.jl:1-28, 57-73) and the oracle's gradient at the result."""
import numpy as np
import pytest

from models import oracle_of, rich_dipole

pytestmark = pytest.mark.gpu


def _fm_square(sg, dims=(3, 3, 1), seed=0, mode="dipole"):
    # H = -Σ Si·Sj - Σ (Siᶻ)² on the square lattice, s = 3/2 (z-polarized ground state)
    cr = sg.Crystal(sg.lattice_vectors(1, 1, 2, 90, 90, 90), [[0, 0, 0]])
    s = sg.System(cr, [(1, sg.Moment(s=1.5, g=2))], mode, dims=dims, seed=seed)
    s.set_exchange(-1.0, sg.Bond(1, 1, [1, 0, 0]))
    s.set_onsite_coupling(lambda Sx, Sy, Sz: -Sz @ Sz, 1)
    return s


def _projected_grad_max(o, S, kap):
    g = o.grad(S) * kap[:, None]
    u = S / np.where(kap == 0, 1, kap)[:, None]
    g -= u * np.sum(u * g, axis=1)[:, None]
    return np.max(np.abs(g))


@pytest.mark.parametrize("mode", ["dipole", "SUN"])
def test_fm_optimization(gpu, sg, mode):
    sys_ = _fm_square(sg, mode=mode)
    # from the x-polarized state without jitter the symmetry cannot break
    sys_.polarize_spins([1, 0, 0])
    r = sg.minimize_energy(sys_, jitter=0)
    assert r.converged
    x = 1.5 if mode == "dipole" else 1.487610951765511   # test_optimization.jl:16
    assert np.allclose(sys_.dipoles_flat(), [x, 0, 0], atol=1e-8)
    # from a random state it reaches ±z
    sys_.randomize_spins()
    r = sg.minimize_energy(sys_)
    assert r.converged
    assert np.allclose(np.abs(sys_.dipoles_flat()), [0, 0, 1.5], atol=1e-8)
    assert sg.energy_per_site(sys_) == pytest.approx(-6.75, rel=1e-12)
    assert r.energy == pytest.approx(sg.energy(sys_), rel=1e-14)


def test_vacancies(gpu, sg):
    cr = sg.Crystal(sg.lattice_vectors(1, 1, 10, 90, 90, 90), [[0, 0, 0]])
    sys_ = sg.System(cr, [(1, sg.Moment(s=1, g=2))], "dipole", dims=(3, 3, 1), seed=1)
    sys_.set_exchange(1.0, sg.Bond(1, 1, [1, 0, 0]))
    kap = np.ones(9)
    kap[0] = 0.01
    best = []
    for trial in range(4):
        sys_.set_kappas(kap)
        sys_.randomize_spins()
        sg.minimize_energy(sys_)
        best.append(sg.energy_per_site(sys_))
    assert min(best) == pytest.approx(-0.8889, abs=1e-4)
    kap[0] = 0.0   # set_vacancy_at!
    best = []
    for trial in range(4):
        sys_.set_kappas(kap)
        sys_.randomize_spins()
        sg.minimize_energy(sys_)
        best.append(sg.energy_per_site(sys_))
    assert min(best) == pytest.approx(-8 / 9, rel=1e-10)


def test_stationary_point_by_oracle(gpu, sg, orc):
    sys_ = rich_dipole(sg)
    r = sg.minimize_energy(sys_, maxiters=3000)
    S = sys_.dipoles_flat()
    o = oracle_of(orc, sys_)
    kap = np.asarray(sys_.kappas, dtype=float).reshape(-1)
    assert r.energy == pytest.approx(o.energy(S), rel=1e-12)
    scale = np.sqrt(np.sum((o.grad(S) * kap[:, None]) ** 2) / sys_.nsites)
    assert _projected_grad_max(o, S, kap) <= 1e-8 * scale
    assert r.converged


def test_rejects_fp32(gpu, sg):
    s = _fm_square(sg)
    f = sg.System(s.crystal, [(1, sg.Moment(s=1.5, g=2))], "dipole", dims=(2, 2, 1), seed=1, precision="fp32")
    f.set_exchange(-1.0, sg.Bond(1, 1, [1, 0, 0]))
    f.randomize_spins()
    with pytest.raises(sg.SunnyGPUError, match="FP64"):
        sg.minimize_energy(f)
