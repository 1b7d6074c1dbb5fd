"""The differentiation workload: simple cubic dipole lattice, s=1, parameters J1 (nearest
neighbour), J2 (second neighbour) and D (onsite -D Sz^2), shared by the adjoint tests and
the benchmark."""
import numpy as np


def sc_params(sg):
    return [
        lambda s, v: s.set_exchange(v, sg.Bond(1, 1, [1, 0, 0])),
        lambda s, v: s.set_exchange(v, sg.Bond(1, 1, [1, 1, 0])),
        lambda s, v: s.set_onsite_coupling(lambda Sx, Sy, Sz: -v * Sz @ Sz, 1),
    ]


def sc_system(sg, L, theta, seed=3, device=0):
    sys_ = sg.System(sg.cubic_crystal(), [(1, sg.Moment(s=1, g=2))], "dipole", dims=(L, L, L), seed=seed,
                     device=device)
    for f, v in zip(sc_params(sg), theta):
        f(sys_, float(v))
    sys_.randomize_spins()
    return sys_


def tangent(S, rng):
    """A random direction tangent to every spin."""
    d = rng.standard_normal(S.shape)
    n = S / np.linalg.norm(S, axis=1)[:, None]
    return d - n * np.sum(d * n, axis=1)[:, None]
