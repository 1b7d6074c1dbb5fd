"""Host side of the adjoint: the unit coupling sets of the parameters combine linearly
into the System's couplings (the premise of the adjoint's E(θ) = E_rest + Σ θ_k E_k),
checked with the FP64 oracle's energy and gradient."""
import numpy as np

from adjoint_models import sc_params


def test_unit_coupling_sets_are_linear(sg, orc):
    from sunny_gb300.adjoint import unit_coupling_sets
    theta = np.array([1.0, 0.1, 0.05])
    sys_ = sg.System(sg.cubic_crystal(), [(1, sg.Moment(s=1, g=2))], "dipole", dims=(4, 4, 4), seed=3, device=None)
    params = sc_params(sg)
    for f, v in zip(params, theta):
        f(sys_, v)
    sys_.randomize_spins()
    S = sys_.dipoles_flat()
    full = orc.OracleSystem.from_system(sys_)
    bonds, counts, onsite = unit_coupling_sets(sys_, params)
    assert counts == [3, 6, 0]
    assert np.count_nonzero(onsite[2]) > 0 and not np.any(onsite[:2])
    # energy and gradient of Σ θ_k E_k from the unit sets, through the oracle
    E, g = 0.0, np.zeros_like(S)
    k0 = 0
    for k in range(3):
        twin = sg.System(sg.cubic_crystal(), [(1, sg.Moment(s=1, g=2))], "dipole", dims=(4, 4, 4), device=None)
        params[k](twin, 1.0)
        o = orc.OracleSystem.from_system(twin)
        E += theta[k] * o.energy(S)
        g += theta[k] * o.grad(S)
        k0 += counts[k]
    assert E == np.float64(full.energy(S)) or abs(E - full.energy(S)) < 1e-12 * abs(E)
    assert np.max(np.abs(g - full.grad(S))) < 1e-12
