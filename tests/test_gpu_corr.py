"""SampledCorrelations parity: the GPU accumulator (sum of conj(A)A products, window
applied at read-out) against the oracle's per-sample windowed running mean
(CorrelationSampling.jl:48-139), plus the reference's RNG-independent identities."""
import numpy as np
import pytest

from models import oracle_of, rich_sun

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


def diamond_reference_model(sg, precision="fp64"):
    # the configuration of test_correlation_sampling.jl:156-169 (diamond 2x3x4, s=3/2, J=0.6498)
    sys_ = sg.System(sg.diamond_crystal(), [(1, sg.Moment(s=1.5, g=2))], "dipole", dims=(2, 3, 4), seed=101,
                     precision=precision)
    sys_.set_exchange(0.6498, sg.Bond(1, 3, [0, 0, 0]))
    sys_.randomize_spins()
    return sys_


def oracle_corr(orc, sys_, sc):
    o = oracle_of(orc, sys_)
    obs = sc.measure.observables
    if sys_.N:
        flat = np.stack([np.swapaxes(obs, -1, -2).real, np.swapaxes(obs, -1, -2).imag], -1).reshape(-1)
    else:
        flat = obs.reshape(-1)
    return o, orc.OracleCorrelations(o, flat, sc.measure.nobs, sc.measure.corr_pairs, sc.n_all_omega, sc.measperiod,
                                     sc.dt, sc.integrator.tol)


@pytest.mark.parametrize("window", ["cosine", "rectangular"])
def test_sqw_parity_fp64(gpu, sg, orc, window):
    sys_ = diamond_reference_model(sg)
    sc = sg.SampledCorrelations(sys_, measure=sg.ssf_perp(sys_), energies=np.linspace(0.0, 5.5, 10), dt=0.12)
    o, oc = oracle_corr(orc, sys_, sc)
    S = sys_.dipoles_flat()
    for _ in range(3):
        sg.add_sample(sc, sys_, window=window)
        S, _ = oc.add_sample(S, None, window=window)
        # Langevin decorrelation between samples, identical noise on both sides
    assert sc.nsamples == 3
    d = sc.data
    assert d.shape == oc.data.shape == (6, 8, 8, 2, 3, 4, 18)
    assert np.max(np.abs(d - oc.data)) < 1e-10 * np.max(np.abs(oc.data))
    assert np.max(np.abs(sys_.dipoles_flat() - S)) < 1e-9


def test_sum_rule_gpu(gpu, sg):
    # test_correlation_sampling.jl:29-50 on the raw accumulator: sum over (α=α, i=i, q, ω)
    # of data = n_all_ω * Ncells * sum_i κ_i^2, for any spin state
    cr = sg.fcc_primitive_crystal()
    sys_ = sg.System(cr, [(1, sg.Moment(s=1, g=2))], "dipole", dims=(4, 4, 4), seed=111)
    sys_.set_exchange(1.0, sg.Bond(1, 1, [1, 0, 0]))
    sys_.randomize_spins()
    sg.step(sys_, sg.Langevin(0.05, damping=0.1, kT=0.1), nsteps=200)
    sc = sg.SampledCorrelations(sys_, measure=sg.ssf_trace(sys_, apply_g=False), energies=np.linspace(0, 10.0, 100), dt=0.08)
    sg.add_sample(sc, sys_)
    d = sc.data
    diag = [c for c, (a, b) in enumerate(sc.measure.corr_pairs) if a == b]
    tot = sum(d[c, 0, 0].sum() for c in diag)
    assert tot.real == pytest.approx(sc.n_all_omega * 64 * 1.0, rel=1e-12)
    assert abs(tot.imag) < 1e-9 * tot.real
    # imaginary part of the diagonal correlations vanishes (test_correlation_sampling.jl:59-67)
    assert np.max(np.abs(np.imag(d[diag]))) < 1e-12 * np.max(np.abs(d))


def test_merge_equals_running_accumulation(gpu, sg):
    # test_correlation_sampling.jl:104-136
    sys_ = diamond_reference_model(sg)
    kw = dict(measure=sg.ssf_trace(sys_), energies=np.linspace(0, 5.5, 25), dt=0.12)
    sc0, sc1, sc2 = (sg.SampledCorrelations(sys_, **kw) for _ in range(3))
    lang = sg.Langevin(0.07, damping=0.1, kT=0.1723)
    sg.step(sys_, lang, nsteps=400)
    S = sys_.dipoles_flat()
    sg.add_sample(sc0, sys_)
    sys_.set_state_flat(dipoles=S)
    sg.add_sample(sc1, sys_)
    for _ in range(2):
        sys_.set_state_flat(dipoles=S)
        sg.step(sys_, lang, nsteps=400)
        S = sys_.dipoles_flat()
        sg.add_sample(sc0, sys_)
        sys_.set_state_flat(dipoles=S)
        sg.add_sample(sc2, sys_)
    merged = sg.merge_correlations([sc1, sc2])
    assert merged.nsamples == 3
    assert np.allclose(merged.data, sc0.data, rtol=1e-12, atol=1e-14 * np.max(np.abs(sc0.data)))


def test_static_correlations(gpu, sg, orc):
    # SampledCorrelationsStatic (energies=nothing): sum over q of the trace = Ncells * κ^2
    sys_ = sg.System(sg.fcc_primitive_crystal(), [(1, sg.Moment(s=1, g=2))], "dipole", dims=(4, 4, 4), seed=3)
    sys_.set_exchange(1.0, sg.Bond(1, 1, [1, 0, 0]))
    sys_.randomize_spins()
    sc = sg.SampledCorrelations(sys_, measure=sg.ssf_trace(sys_, apply_g=False), energies=None, dt=float("nan"))
    S = sys_.dipoles_flat()
    sg.add_sample(sc, sys_)
    assert np.array_equal(sys_.dipoles_flat(), S)   # no time integration
    d = sc.data
    diag = [c for c, (a, b) in enumerate(sc.measure.corr_pairs) if a == b]
    tot = sum(d[c, 0, 0].sum() for c in diag)
    assert tot.real == pytest.approx(64.0, rel=1e-12)


@pytest.mark.parametrize("tol,order", [(1e-7, 4), (1e-6, 4), (1e-6, 0)])
def test_sqw_fp32_per_bin_error(gpu, sg, orc, tol, order):
    # 1e-6 is the FP32 midpoint tolerance the benchmark runs with; order 4 is the default
    # extrapolated first iterate, 0 the reference's S' = S
    sys64 = diamond_reference_model(sg, "fp64")
    sys32 = diamond_reference_model(sg, "fp32")
    sys32.set_midpoint_predictor(order)
    sys32.set_state_flat(dipoles=sys64.dipoles_flat())
    kw = dict(energies=np.linspace(0.0, 5.5, 10), dt=0.12)
    sc = sg.SampledCorrelations(sys32, measure=sg.ssf_perp(sys32), tol=tol, **kw)
    o, oc = oracle_corr(orc, sys64, sc)
    oc.tol = 1e-12
    sg.add_sample(sc, sys32)
    oc.add_sample(sys64.dipoles_flat(), None)
    ref = oc.data
    err = np.abs(sc.data - ref)
    # per-bin error bound of 1% of the bin, with a floor of 1e-4 of the largest bin for
    # bins that are zero up to rounding
    assert np.all(err <= 0.01 * np.abs(ref) + 1e-4 * np.max(np.abs(ref)))


def test_sqw_sun_parity(gpu, sg, orc):
    sys_ = rich_sun(sg, N=3, dims=(2, 2, 2))
    sc = sg.SampledCorrelations(sys_, measure=sg.ssf_trace(sys_), energies=np.linspace(0, 4.0, 6), dt=0.05)
    o, oc = oracle_corr(orc, sys_, sc)
    S, Z = sys_.dipoles_flat(), sys_.coherents_flat()
    sg.add_sample(sc, sys_)
    oc.add_sample(S, Z)
    assert np.max(np.abs(sc.data - oc.data)) < 1e-10 * np.max(np.abs(oc.data))


def test_accumulator_outlives_its_system(gpu, sg):
    # destroying the System first detaches its accumulators: data can still be read,
    # adding samples raises instead of touching freed memory
    sys_ = diamond_reference_model(sg)
    sc = sg.SampledCorrelations(sys_, measure=sg.ssf_perp(sys_), energies=np.linspace(0.0, 5.5, 10), dt=0.12)
    sg.add_sample(sc, sys_)
    before = sc.data
    sys_.close()
    assert sc.nsamples == 1
    assert np.array_equal(sc.data, before)
    with pytest.raises(sg.SunnyGPUError, match="destroyed"):
        sc._check(sc._lib.sgb_corr_add_sample(sc._h, 0))
    sc.close()


@pytest.mark.parametrize("order", [0, 2, 4])
def test_batched_fp32_sqw_per_bin_error(gpu, sg, orc, order):
    # the headline path: FP32 replicas sampled in one batched add_sample (tol 1e-6)
    # against the FP64 oracle's running mean over the same initial states, with the
    # reference's first iterate (order 0) and with the extrapolated one (order 2, default)
    proto = diamond_reference_model(sg, "fp64")
    kw = dict(energies=np.linspace(0.0, 5.5, 10), dt=0.12)
    b = sg.ReplicaBatch(proto, [proto.dims] * 3, kT=[0.2] * 3, precision="fp32", seed=4)
    b.set_midpoint_predictor(order)
    b.randomize_spins()
    states = [b.get_state(r) for r in range(3)]
    sc = sg.SampledCorrelations(b, measure=sg.ssf_perp(proto), tol=1e-6, **kw)
    sg.add_sample(sc, b)
    o, oc = oracle_corr(orc, proto, sc)
    oc.tol = 1e-12
    for r in range(3):
        oc.add_sample(states[r], None)
    ref = oc.data
    err = np.abs(sc.data - ref)
    assert np.all(err <= 0.01 * np.abs(ref) + 1e-4 * np.max(np.abs(ref)))
    sc.close()
    b.close()


def test_calculate_errors_parity_and_merge(gpu, sg, orc):
    # calculate_errors=true: running mean and Welford M against the oracle
    # (CorrelationSampling.jl:117-134), and merge with M (SampledCorrelations.jl:128-142)
    sys_ = diamond_reference_model(sg)
    kw = dict(measure=sg.ssf_perp(sys_), energies=np.linspace(0.0, 5.5, 10), dt=0.12, calculate_errors=True)
    sc0, sc1, sc2 = (sg.SampledCorrelations(sys_, **kw) for _ in range(3))
    o, oc = oracle_corr(orc, sys_, sc0)
    oc.M = np.zeros(oc.data.shape)
    rng = np.random.default_rng(23)
    states = []
    for _ in range(3):
        S = rng.standard_normal((sys_.nsites, 3))
        states.append(1.5 * S / np.linalg.norm(S, axis=1)[:, None])
    for k, S in enumerate(states):
        sys_.set_state_flat(dipoles=S)
        sg.add_sample(sc0, sys_)
        sys_.set_state_flat(dipoles=S)
        sg.add_sample(sc1 if k == 0 else sc2, sys_)
        oc.add_sample(S, None)
    scale = np.max(np.abs(oc.data))
    assert np.max(np.abs(sc0.data - oc.data)) < 1e-10 * scale
    assert np.max(np.abs(sc0.M - oc.M)) < 1e-10 * np.max(np.abs(oc.M))
    merged = sg.merge_correlations([sc1, sc2])
    assert merged.nsamples == 3
    assert np.max(np.abs(merged.data - sc0.data)) < 1e-12 * scale
    assert np.max(np.abs(merged.M - sc0.M)) < 1e-10 * np.max(np.abs(sc0.M))
    # accumulators with and without errors do not merge
    plain = sg.SampledCorrelations(sys_, measure=sg.ssf_perp(sys_), energies=np.linspace(0.0, 5.5, 10), dt=0.12)
    with pytest.raises(sg.SunnyGPUError, match="calculate_errors"):
        sg.merge_correlations([sc0, plain])


def test_batched_calculate_errors_equals_single(gpu, sg):
    # one batched add_sample over 3 replicas == 3 single add_samples, mean and M
    cr = sg.diamond_crystal()
    proto = sg.System(cr, [(1, sg.Moment(s=1.5, g=2))], "dipole", dims=(2, 3, 2), seed=101, device=None)
    proto.set_exchange(0.6498, sg.Bond(1, 3, [0, 0, 0]))
    b = sg.ReplicaBatch(proto, [(2, 3, 2)] * 3, kT=[0.2] * 3, seed=2)
    b.randomize_spins()
    states = [b.get_state(r) for r in range(3)]
    kw = dict(energies=np.linspace(0, 5.5, 10), dt=0.12, calculate_errors=True)
    scb = sg.SampledCorrelations(b, measure=sg.ssf_perp(proto), **kw)
    sg.add_sample(scb, b)
    single = sg.System(cr, [(1, sg.Moment(s=1.5, g=2))], "dipole", dims=(2, 3, 2), seed=101)
    single.set_exchange(0.6498, sg.Bond(1, 3, [0, 0, 0]))
    scs = sg.SampledCorrelations(single, measure=sg.ssf_perp(single), **kw)
    for r in range(3):
        single.set_state_flat(dipoles=states[r])
        sg.add_sample(scs, single)
    assert np.max(np.abs(scb.data - scs.data)) < 1e-11 * np.max(np.abs(scs.data))
    assert np.max(np.abs(scb.M - scs.M)) < 1e-10 * np.max(np.abs(scs.M))
    scb.close()
    b.close()


def test_batched_predictor_reaches_the_same_fixed_point(gpu, sg):
    # FP64 batch with the order-4 first iterate against the single-system path (which
    # starts from S' = S as the reference does): equal within the midpoint tolerance
    cr = sg.diamond_crystal()
    proto = sg.System(cr, [(1, sg.Moment(s=1.5, g=2))], "dipole", dims=(2, 3, 2), seed=101, device=None)
    proto.set_exchange(0.6498, sg.Bond(1, 3, [0, 0, 0]))
    b = sg.ReplicaBatch(proto, [(2, 3, 2)] * 2, kT=[0.2] * 2, seed=2)
    b.set_midpoint_predictor(4)
    b.randomize_spins()
    states = [b.get_state(r) for r in range(2)]
    kw = dict(energies=np.linspace(0, 5.5, 10), dt=0.12)
    scb = sg.SampledCorrelations(b, measure=sg.ssf_perp(proto), **kw)
    sg.add_sample(scb, b)
    single = sg.System(cr, [(1, sg.Moment(s=1.5, g=2))], "dipole", dims=(2, 3, 2), seed=101)
    single.set_exchange(0.6498, sg.Bond(1, 3, [0, 0, 0]))
    scs = sg.SampledCorrelations(single, measure=sg.ssf_perp(single), **kw)
    for r in range(2):
        single.set_state_flat(dipoles=states[r])
        sg.add_sample(scs, single)
        assert rel(b.get_state(r), single.dipoles_flat()) < 1e-9
    assert rel(scb.data, scs.data) < 1e-9
    scb.close()
    b.close()


def test_intensities_parity(gpu, sg, orc):
    # intensities(sc, qpts; energies, kT) (DataRetrieval.jl:77-171) against the oracle's
    # restatement on its own data: on-grid, off-grid (rounded), negative and zero q,
    # nonnegative / all / listed energies, with and without the classical-to-quantum factor
    sys_ = diamond_reference_model(sg)
    kw = dict(energies=np.linspace(0.0, 5.5, 10), dt=0.12)
    sc = sg.SampledCorrelations(sys_, measure=sg.ssf_perp(sys_), **kw)
    o, oc = oracle_corr(orc, sys_, sc)
    S = sys_.dipoles_flat()
    sg.add_sample(sc, sys_)
    oc.add_sample(S, None)
    cr = sys_.crystal
    pos = np.array([cr._pos[a] for a in range(sys_.natoms)])
    qs = np.array([[0.0, 0.0, 0.0], [-0.2, 0.4, -0.1], [0.5, 1 / 3, 0.25], [1.26, -0.74, 0.49], [-0.5, 0.0, 0.75]])
    comb = sc.measure.combiner
    for energies, kT in (("available", None), ("available_with_negative", 0.4), ([-1.0, 0.0, 0.61, 2.0], None)):
        res = sg.intensities(sc, qs, energies=energies, kT=kT)
        ws, widx = sg.correlations._energy_indices(sc, energies)
        ref = orc.intensities(oc.data, cr.recipvecs, pos, sys_.dims, qs, widx, comb, sc.n_all_omega, sc.dw, kT, ws)
        assert res.data.shape == ref.shape
        assert np.max(np.abs(res.data - ref)) < 1e-9 * np.max(np.abs(ref))
    # the reference golden vector's q = 0 column: the cosine window's spectrum of the
    # conserved total moment, I(0, Δω) = I(0, 0) / 2 and ~0 above (test_correlation_sampling.jl:167)
    col = sg.intensities(sc, qs[:1], energies="available", kT=None).data[:, 0]
    assert col[1] == pytest.approx(0.5 * col[0], rel=1e-10)
    assert np.max(np.abs(col[2:])) < 1e-10 * col[0]
    # the device trace combiner and the host path for a custom combiner agree
    sct = sg.SampledCorrelations(sys_, measure=sg.ssf_trace(sys_), **kw)
    scc = sg.SampledCorrelations(sys_, measure=sg.ssf_custom(lambda q, m: np.trace(m.real), sys_), **kw)
    for x in (sct, scc):
        sys_.set_state_flat(dipoles=S)
        sg.add_sample(x, sys_)
    a = sg.intensities(sct, qs, energies="available").data
    b = sg.intensities(scc, qs, energies="available").data
    assert np.max(np.abs(a - b)) < 1e-12 * np.max(np.abs(a))
    st = sg.intensities_static(sct, qs)
    assert np.allclose(st.data, sg.intensities(sct, qs, energies="available_with_negative").data.sum(axis=0) * sct.dw,
                       rtol=1e-12)


def test_intensities_with_errors_mode_equal_deferred(gpu, sg):
    # the Welford accumulator holds the transformed mean: same intensities as the deferred sum
    sys_ = diamond_reference_model(sg)
    kw = dict(measure=sg.ssf_perp(sys_), energies=np.linspace(0.0, 5.5, 10), dt=0.12)
    a = sg.SampledCorrelations(sys_, **kw)
    b = sg.SampledCorrelations(sys_, calculate_errors=True, **kw)
    rng = np.random.default_rng(5)
    for _ in range(2):
        S = rng.standard_normal((sys_.nsites, 3))
        S = 1.5 * S / np.linalg.norm(S, axis=1)[:, None]
        for x in (a, b):
            sys_.set_state_flat(dipoles=S)
            sg.add_sample(x, sys_)
    qs = np.array([[0.0, 0.0, 0.0], [0.5, 1 / 3, 0.25], [-0.5, 0.0, 0.75]])
    ia = sg.intensities(a, qs, energies="available_with_negative", kT=0.3).data
    ib = sg.intensities(b, qs, energies="available_with_negative", kT=0.3).data
    assert np.max(np.abs(ia - ib)) < 1e-10 * np.max(np.abs(ia))


@pytest.mark.parametrize("nw", [200, 300])
def test_own_time_transform_matches_cufft(gpu, sg, nw):
    # the hand-written Bluestein time transform of FP32 accumulators against cuFFT's, from
    # the same start: equal up to FP32 rounding of the two transforms
    import ctypes as C
    proto = sg.System(sg.diamond_crystal(), [(1, sg.Moment(s=1.5, g=2))], "dipole", dims=(2, 3, 4), seed=31,
                      precision="fp32", device=None)
    proto.set_exchange(0.6498, sg.Bond(1, 3, [0, 0, 0]))
    b = sg.ReplicaBatch(proto, [proto.dims] * 3, kT=[0.3] * 3, precision="fp32", seed=2)
    b.randomize_spins()
    b.langevin(0.05, 0.1, 100)
    start = [b.get_state(r) for r in range(3)]
    kw = dict(energies=np.linspace(0, 5.5, nw), dt=0.05, tol=1e-6)
    datas = []
    for kind in (0, 1):
        for r in range(3):
            b.set_state(r, start[r])
        sc = sg.SampledCorrelations(b, measure=sg.ssf_trace(proto), **kw)
        assert sc._lib.sgb_corr_set_time_transform(sc._h, kind) == 0
        assert sc._lib.sgb_corr_time_transform(sc._h) == kind
        sg.add_sample(sc, b)
        datas.append(sc.data)
        sc.close()
    scale = np.max(np.abs(datas[1]))
    assert np.max(np.abs(datas[0] - datas[1])) < 2e-5 * scale
    b.close()


def test_time_transform_falls_back_beyond_its_length(gpu, sg):
    # the own kernel's 1024-point convolution covers 512 < n_all_ω + n_all_ω/2 <= 1024:
    # nω = 400 and nω = 40 use cuFFT, nω = 300 the own kernel
    s = sg.System(sg.cubic_crystal(), [(1, sg.Moment(s=1, g=2))], "dipole", dims=(2, 2, 2), seed=3, precision="fp32")
    s.set_exchange(1.0, sg.Bond(1, 1, [1, 0, 0]))
    s.randomize_spins()
    sc = sg.SampledCorrelations(s, measure=sg.ssf_trace(s), energies=np.linspace(0, 4.0, 400), dt=0.05, tol=1e-6)
    assert sc._lib.sgb_corr_time_transform(sc._h) == 1
    sc2 = sg.SampledCorrelations(s, measure=sg.ssf_trace(s), energies=np.linspace(0, 4.0, 300), dt=0.05, tol=1e-6)
    assert sc2._lib.sgb_corr_time_transform(sc2._h) == 0
    sc3 = sg.SampledCorrelations(s, measure=sg.ssf_trace(s), energies=np.linspace(0, 4.0, 40), dt=0.05, tol=1e-6)
    assert sc3._lib.sgb_corr_time_transform(sc3._h) == 1
    sc.close()
    sc2.close()
    sc3.close()


def test_own_time_transform_with_series_straddling_replicas(gpu, sg):
    # 3 observables x 1 sublattice x 27 cells = 81 series per replica: CTAs of 8 series
    # straddle replicas and take the per-series path
    proto = sg.System(sg.cubic_crystal(), [(1, sg.Moment(s=1, g=2))], "dipole", dims=(3, 3, 3), seed=8,
                      precision="fp32", device=None)
    proto.set_exchange(1.0, sg.Bond(1, 1, [1, 0, 0]))
    b = sg.ReplicaBatch(proto, [proto.dims] * 3, kT=[0.5] * 3, precision="fp32", seed=9)
    b.randomize_spins()
    b.langevin(0.05, 0.1, 50)
    start = [b.get_state(r) for r in range(3)]
    kw = dict(energies=np.linspace(0, 5.0, 200), dt=0.05, tol=1e-6)
    datas = []
    for kind in (0, 1):
        for r in range(3):
            b.set_state(r, start[r])
        sc = sg.SampledCorrelations(b, measure=sg.ssf_trace(proto), **kw)
        assert sc._lib.sgb_corr_set_time_transform(sc._h, kind) == 0
        assert sc._lib.sgb_corr_time_transform(sc._h) == kind
        sg.add_sample(sc, b)
        datas.append(sc.data)
        sc.close()
    assert np.max(np.abs(datas[0] - datas[1])) < 2e-5 * np.max(np.abs(datas[1]))
    b.close()
