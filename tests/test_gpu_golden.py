"""The CUDA path (FP64) against the committed golden fixtures written by the oracle
(tests/golden/make_golden.py), through the C-ABI, with the parity tolerances of the
other GPU tests."""
from pathlib import Path

import numpy as np
import pytest

from models import rich_dipole, rich_sun

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden" / "oracle_small.npz"


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


def test_dipole_golden(gpu, sg, golden):
    d = rich_dipole(sg)
    S0 = golden["dip_S0"]
    d.set_state_flat(dipoles=S0)
    assert rel(sg.energy_grad(d), golden["dip_grad"]) < 1e-12
    assert sg.energy(d) == pytest.approx(float(golden["dip_E"]), rel=1e-12)
    sg.step(d, sg.Langevin(0.01, damping=0.1, kT=0.3), nsteps=3, noise=golden["dip_noise"])
    assert rel(d.dipoles_flat(), golden["dip_heun3"]) < 1e-11
    d.set_state_flat(dipoles=S0)
    sg.step(d, sg.ImplicitMidpoint(0.02), nsteps=3)
    assert rel(d.dipoles_flat(), golden["dip_mid3"]) < 1e-9


def test_sun_golden(gpu, sg, golden):
    s = rich_sun(sg, N=3)
    Z0 = golden["sun_Z0"]
    s.set_state_flat(coherents=Z0)
    assert rel(sg.energy_grad(s), golden["sun_grad"]) < 1e-12
    assert sg.energy(s) == pytest.approx(float(golden["sun_E"]), rel=1e-12)
    sg.step(s, sg.Langevin(0.01, damping=0.1, kT=0.3), nsteps=2, noise=golden["sun_noise"])
    assert rel(s.coherents_flat(), golden["sun_heun2"]) < 1e-11
    s.set_state_flat(coherents=Z0)
    sg.step(s, sg.ImplicitMidpoint(0.02), nsteps=2)
    assert rel(s.coherents_flat(), golden["sun_mid2"]) < 1e-9


def test_sqw_golden(gpu, sg, golden):
    q = sg.System(sg.diamond_crystal(), [(1, sg.Moment(s=1.5, g=2))], "dipole", dims=(2, 3, 4), seed=101)
    q.set_exchange(0.6498, sg.Bond(1, 3, [0, 0, 0]))
    q.set_state_flat(dipoles=golden["sqw_S0"])
    sc = sg.SampledCorrelations(q, measure=sg.ssf_perp(q), energies=np.linspace(0.0, 5.5, 10), dt=0.12)
    sg.add_sample(sc, q)
    d = sc.data
    assert rel(q.dipoles_flat(), golden["sqw_S1"]) < 1e-9
    for got, key in ((d.sum(axis=(1, 2)), "sqw_sum_ij"), (d[:, 0, 0], "sqw_block_00"), (d[:, 3, 7], "sqw_block_37")):
        ref = golden[key]
        assert np.max(np.abs(got - ref)) < 1e-10 * np.max(np.abs(ref)), key
    sc.close()
