"""Replica groups: ReplicaBatch over SU(N) (or otherwise non-batchable) prototypes. The
replicas are device clones of the prototype (clone_system, as Sunny's ParallelTempering
makes them, ParallelTempering.jl:20-37) whose persistent launches run concurrently on
their own streams. Each replica must follow exactly the trajectory that the same clone
follows alone, and a batched add_sample must accumulate the same data as one
add_sample per replica (CorrelationSampling.jl:156-176, merged as
SampledCorrelations.jl:128-142)."""
import numpy as np
import pytest

from models import rich_sun, triangular_c3

pytestmark = pytest.mark.gpu


def test_sun_group_langevin_matches_single_systems(gpu, sg):
    proto = rich_sun(sg, N=3, device=None, dims=(3, 2, 2))
    b = sg.ReplicaBatch(proto, [proto.dims] * 3, kT=[0.1, 0.3, 0.6], seed=21)
    b.randomize_spins()
    starts = [b.get_state(r) for r in range(3)]
    b.langevin(0.01, 0.2, 30)
    for r in range(3):
        s = sg.clone_system(proto, seed=21 + r, device=0)
        s.set_state_flat(coherents=starts[r])
        sg.step(s, sg.Langevin(0.01, damping=0.2, kT=[0.1, 0.3, 0.6][r]), 30)
        assert np.max(np.abs(b.get_state(r) - s.coherents_flat())) < 1e-12
        assert b.energies()[r] == pytest.approx(sg.energy(s), abs=1e-12 * max(1.0, abs(sg.energy(s))))
        s.close()
    n0 = b.noise(1, 5)
    assert n0.shape == (proto.nsites, 3) and np.iscomplexobj(n0)
    b.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_sun_group_sample_equals_per_replica_samples(gpu, sg, precision):
    proto = rich_sun(sg, N=3, device=None, dims=(3, 2, 2), precision=precision)
    R = 4
    b = sg.ReplicaBatch(proto, [proto.dims] * R, kT=[0.3] * R, seed=5, precision=precision)
    b.randomize_spins()
    b.langevin(0.02, 0.1, 100)
    starts = [b.get_state(r) for r in range(R)]
    kw = dict(energies=np.linspace(0, 4.0, 8), dt=0.05, tol=1e-12 if precision == "fp64" else 1e-6)
    sc = sg.SampledCorrelations(b, measure=sg.ssf_perp(proto), **kw)
    sg.add_sample(sc, b)
    ends = [b.get_state(r) for r in range(R)]
    single = sg.clone_system(proto, device=0, precision=precision)
    sc1 = sg.SampledCorrelations(single, measure=sg.ssf_perp(single), **kw)
    for r in range(R):
        single.set_state_flat(coherents=starts[r])
        sg.add_sample(sc1, single)
        tol = 1e-12 if precision == "fp64" else 1e-5
        assert np.max(np.abs(single.coherents_flat() - ends[r])) < tol
    scale = np.max(np.abs(sc1.data))
    tol = 1e-11 if precision == "fp64" else 1e-4
    assert np.max(np.abs(sc.data - sc1.data)) < tol * scale
    assert sc.nsamples == sc1.nsamples == R
    sc.close()
    sc1.close()
    single.close()
    b.close()


def test_triangular_su3_group_runs_concurrently(gpu, sg):
    # the SU(3) triangular workload (48 x 48 x 4): eight replicas per batched add_sample
    proto = triangular_c3(sg, precision="fp32", device=None)
    b = sg.ReplicaBatch(proto, [proto.dims] * 8, kT=[0.3] * 8, seed=2, precision="fp32")
    b.randomize_spins()
    b.langevin(0.02, 0.1, 50)
    sc = sg.SampledCorrelations(b, measure=sg.ssf_perp(proto), energies=np.linspace(0, 3.0, 10), dt=0.05, tol=1e-6)
    sg.add_sample(sc, b)
    assert sc.nsamples == 8 and np.all(np.isfinite(sc.data))
    E = b.energies()
    assert np.all(np.isfinite(E))
    sc.close()
    b.close()


def test_group_with_dipole_dipole(gpu, sg):
    # dipole mode with dipole-dipole interactions becomes a group too
    cr = sg.Crystal(sg.lattice_vectors(2, 2, 2, 90, 90, 90), [[0, 0, 0]])
    proto = sg.System(cr, [(1, sg.Moment(s=1, g=2))], "dipole", dims=(3, 3, 2), seed=4, device=None)
    proto.set_exchange(1.0, sg.Bond(1, 1, [1, 0, 0]))
    proto.enable_dipole_dipole(0.5)
    b = sg.ReplicaBatch(proto, [proto.dims] * 2, kT=[0.2, 0.4], seed=9)
    b.randomize_spins()
    starts = [b.get_state(r) for r in range(2)]
    kw = dict(energies=np.linspace(0, 4.0, 6), dt=0.05)
    sc = sg.SampledCorrelations(b, measure=sg.ssf_trace(proto), **kw)
    sg.add_sample(sc, b)
    single = sg.clone_system(proto, device=0)
    sc1 = sg.SampledCorrelations(single, measure=sg.ssf_trace(single), **kw)
    for r in range(2):
        single.set_state_flat(dipoles=starts[r])
        sg.add_sample(sc1, single)
        assert np.max(np.abs(single.dipoles_flat() - b.get_state(r))) < 1e-12
    assert np.max(np.abs(sc.data - sc1.data)) < 1e-11 * np.max(np.abs(sc1.data))
    with pytest.raises(sg.SunnyGPUError, match="ParallelTempering"):
        sg.ParallelTempering(b, 0.01, 0.1).replica_exchange(1)
    sc.close()
    sc1.close()
    single.close()
    b.close()
