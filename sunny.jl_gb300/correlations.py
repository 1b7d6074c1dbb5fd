"""SampledCorrelations mirror: measurement specs, the GPU-resident S(q,ω) accumulator,
add_sample and merge_correlations.

Follows src/SampledCorrelations/*.jl and src/Measurements/MeasureSpec.jl of Sunny.jl
v0.9.2. The accumulator lives on the device and is tied to one `System`.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _abi
from .operators import spin_matrices_of_dim
from .system import ImplicitMidpoint, System

CORR_PAIRS = [(3, 3), (2, 3), (1, 3), (2, 2), (1, 2), (1, 1)]  # MeasureSpec.jl:117


class MeasureSpec:
    """Observables (nobs per site) and 1-based correlation pairs (MeasureSpec.jl:5-27)."""

    def __init__(self, observables: np.ndarray, corr_pairs, combiner=None, kind: str = "custom", formfactors=None):
        self.observables = observables      # dipole: (nobs, ns, 3); SU(N): (nobs, ns, N, N) complex
        self.corr_pairs = list(corr_pairs)
        self.combiner = combiner
        self.kind = kind                    # "trace" / "perp" run the combiner on the device
        self.formfactors = formfactors      # per atom: callable of |q|^2, or None for 1

    @property
    def nobs(self):
        return self.observables.shape[0]


def all_dipole_observables(sys: System, apply_g: bool = True) -> np.ndarray:
    """MeasureSpec.jl:53-76, in site order."""
    ns = sys.nsites
    G = sys._g if apply_g else np.broadcast_to(np.eye(3), (ns, 3, 3))
    if sys.N == 0:
        # component α is the row α of g: op . S = g[α, :] . S
        return np.ascontiguousarray(np.transpose(G, (1, 0, 2)))       # (3, ns, 3)
    S = spin_matrices_of_dim(sys.N)
    obs = np.einsum("iab,bmn->aimn", G.astype(complex), np.stack(S))  # (3, ns, N, N)
    return obs


def ssf_custom(f, sys: System, apply_g: bool = True) -> MeasureSpec:
    """ssf_custom (MeasureSpec.jl:115-130)."""
    def combiner(q, corr):
        m = np.array([[corr[5], corr[4], corr[2]],
                      [np.conj(corr[4]), corr[3], corr[1]],
                      [np.conj(corr[2]), np.conj(corr[1]), corr[0]]])
        return f(q, m)
    return MeasureSpec(all_dipole_observables(sys, apply_g), CORR_PAIRS, combiner)


def ssf_trace(sys: System, apply_g: bool = True, formfactors=None) -> MeasureSpec:
    m = ssf_custom(lambda q, ssf: np.trace(ssf.real), sys, apply_g)
    m.kind, m.formfactors = "trace", formfactors
    return m


def ssf_perp(sys: System, apply_g: bool = True, formfactors=None) -> MeasureSpec:
    def f(q, ssf):
        q2 = float(np.dot(q, q))
        ssf = ssf.real
        return (2 / 3) * np.trace(ssf) if q2 == 0 else np.trace(ssf) - q @ ssf @ q / q2
    m = ssf_custom(f, sys, apply_g)
    m.kind, m.formfactors = "perp", formfactors
    return m


def adjusted_dt_and_downsampling_factor(dt: float, nw: int, wmax: float):
    """SampledCorrelations.jl:152-173."""
    assert math.pi / dt > wmax, "Desired `ωmax` not possible with specified `dt`. Choose smaller `dt` value."
    n_all_w = 2 * (int(nw) - 1)
    dw = wmax / (nw - 1)
    measperiod = math.ceil(math.pi / (dt * wmax))
    dt_new = 2 * math.pi / (dw * measperiod * n_all_w)
    return dt_new, measperiod


class SampledCorrelations:
    """SampledCorrelations(sys; measure, energies, dt, integrator) (SampledCorrelations.jl:199-269).

    `sys` may also be a ReplicaBatch of equal-size replicas: each add_sample then
    integrates every replica and accumulates one sample per replica (the parallel
    sampling pattern of Sunny's docs/src/parallelism.md, merged on the device)."""

    def __init__(self, sys, *, measure: MeasureSpec, energies, dt, calculate_errors=False,
                 integrator: ImplicitMidpoint | None = None, tol: float | None = None):
        if energies is None:
            n_all_w, measperiod, dw = 1, 1, math.nan
            if not math.isnan(dt):
                raise ValueError("Must use dt=NaN when energies=nothing")
        else:
            energies = np.asarray(energies, dtype=float)
            nw = len(energies)
            n_all_w = 2 * (nw - 1)
            wmax = energies[-1]
            if not (energies[0] == 0 and wmax > 0):
                raise ValueError("`energies` must be a range from 0 to a positive value")
            dE = np.diff(energies)
            if not np.allclose(dE, dE[0]):
                raise ValueError("`energies` must be equally spaced.")
            dt, measperiod = adjusted_dt_and_downsampling_factor(dt, nw, wmax)
            dw = wmax / (nw - 1)
        integrator = integrator or ImplicitMidpoint(1.0)  # dt is set below
        if tol is not None:
            integrator.tol = tol
        self.sys = sys
        self.measure = measure
        self.dw = dw
        self.dt = dt
        self.measperiod = measperiod
        self.n_all_omega = n_all_w
        self.integrator = integrator
        self.calculate_errors = calculate_errors
        obs = measure.observables
        if sys.N:
            o = np.ascontiguousarray(np.stack([np.swapaxes(obs, -1, -2).real, np.swapaxes(obs, -1, -2).imag], -1).reshape(-1))
        else:
            o = np.ascontiguousarray(obs, dtype=float).reshape(-1)
        pairs = np.ascontiguousarray(np.array(measure.corr_pairs, dtype=np.int32) - 1).reshape(-1)
        self._obs_keep, self._pairs_keep = o, pairs
        d = _abi.CorrDesc()
        d.nobs = measure.nobs
        d.obs = _abi.dptr(o)
        d.ncorr = len(measure.corr_pairs)
        d.pairs = pairs.ctypes.data_as(C.POINTER(C.c_int32))
        d.n_all_omega = n_all_w
        d.measperiod = measperiod
        d.dt = 0.0 if math.isnan(dt) else dt
        d.damping = integrator.damping
        d.tol = integrator.tol
        d.max_iters = 100
        d.calculate_errors = 1 if calculate_errors else 0
        h = C.c_void_p()
        self._batch = None
        from .tempering import ReplicaBatch
        if isinstance(sys, ReplicaBatch):
            if len(set(sys.dims_list)) != 1 or sys.dims_list[0] != sys.proto.dims:
                raise ValueError("batched sampling needs replicas with the prototype's dims")
            self._batch = sys
            sys._check(sys._lib.sgb_batch_corr_create(sys.handle, C.byref(d), C.byref(h)))
            self._lib = sys._lib
        else:
            sys._sync_to_device()
            _abi.check(sys._lib.sgb_corr_create(sys.handle, C.byref(d), C.byref(h)), sys._lib, sys.handle)
            self._lib = sys._lib
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._lib.sgb_corr_destroy(self._h)
            self._h = None

    def _check(self, rc):
        if rc != _abi.SGB_OK:
            if self._batch is not None and self._batch.handle is not None:
                self._batch._check(rc)
            # errors of an accumulator whose owner was closed are in the process-wide message
            owner = None if self._batch is not None else self.sys.handle
            _abi.check(rc, self._lib, owner)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def nsamples(self) -> int:
        n = C.c_int64()
        self._check(self._lib.sgb_corr_data(self._h, None, None, C.byref(n)))
        return n.value

    @property
    def shape(self):
        ncorr = len(self.measure.corr_pairs)
        proto = self._batch.proto if self._batch is not None else self.sys
        na = proto.natoms
        return (ncorr, na, na, *proto.dims, self.n_all_omega)

    @property
    def M(self):
        """sc.M: Welford sums of squared deviations [c, i, j, q1, q2, q3, ω] (calculate_errors=true), else None."""
        if not self.calculate_errors:
            return None
        shp = self.shape
        flat = np.zeros(int(np.prod(shp)))
        self._check(self._lib.sgb_corr_data(self._h, None, _abi.dptr(flat), None))
        return flat.reshape(shp[::-1]).transpose(tuple(range(len(shp) - 1, -1, -1)))

    @property
    def data(self) -> np.ndarray:
        """sc.data: complex array indexed [c, i, j, q1, q2, q3, ω] (0-based)."""
        shp = self.shape
        flat = np.zeros(2 * int(np.prod(shp)))
        self._check(self._lib.sgb_corr_data(self._h, _abi.dptr(flat), None, None))
        z = flat[0::2] + 1j * flat[1::2]
        return z.reshape(shp[::-1]).transpose(tuple(range(len(shp) - 1, -1, -1)))


def add_sample(sc: SampledCorrelations, sys, window: str = "cosine"):
    """add_sample!(sc, sys; window) (CorrelationSampling.jl:156-176). Mutates sys (or
    every replica of a ReplicaBatch, adding one sample per replica)."""
    if sys is not sc.sys:
        raise ValueError("a GPU SampledCorrelations is bound to the System it was created with")
    w = {"cosine": 0, "rectangular": 1}[window]
    if sc._batch is not None:
        sc._batch._sync_members()
        sc._check(sc._lib.sgb_corr_add_sample(sc._h, w))
        sc._batch._touch()
        return
    sys._sync_to_device()
    rc = sys._lib.sgb_corr_add_sample(sc._h, w)
    sys._dev_newer = True
    _abi.check(rc, sys._lib, sys.handle)


def merge_correlations(scs):
    """merge_correlations (SampledCorrelations.jl:128-142): returns a new accumulator on the
    system of the first one holding the combined samples."""
    first = scs[0]
    out = SampledCorrelations.__new__(SampledCorrelations)
    out.__dict__.update({k: v for k, v in first.__dict__.items() if k != "_h"})
    d = _abi.CorrDesc()
    d.nobs = first.measure.nobs
    d.obs = _abi.dptr(first._obs_keep)
    d.ncorr = len(first.measure.corr_pairs)
    d.pairs = first._pairs_keep.ctypes.data_as(C.POINTER(C.c_int32))
    d.n_all_omega = first.n_all_omega
    d.measperiod = first.measperiod
    d.dt = 0.0 if math.isnan(first.dt) else first.dt
    d.damping = first.integrator.damping
    d.tol = first.integrator.tol
    d.max_iters = 100
    d.calculate_errors = 1 if first.calculate_errors else 0
    lib = first._lib
    h = C.c_void_p()
    if first._batch is not None:
        first._batch._check(lib.sgb_batch_corr_create(first._batch.handle, C.byref(d), C.byref(h)))
    else:
        _abi.check(lib.sgb_corr_create(first.sys.handle, C.byref(d), C.byref(h)), lib, first.sys.handle)
    out._h = h
    for sc in scs:
        out._check(lib.sgb_corr_merge(out._h, sc._h))
    return out


def compare_correlations(sc_a: SampledCorrelations, sc_b: SampledCorrelations) -> dict:
    """Per-bin agreement of two calculate_errors accumulators of one layout (no counterpart
    in the reference): whether sc_a's means agree with sc_b's within their error bars.

    Per bin, Δ = mean_a − mean_b and s = M_a/(n_a(n_a−1)) + M_b/(n_b(n_b−1)) (the variance
    of Δ if both estimate one S(q,ω), from Welford's M as in CorrelationSampling.jl:117-134).
    Returns
      chi2_ratio     Σ|Δ|² / Σs: about 1 when independent samples differ by noise alone,
                     below 1 when the two accumulators hold samples from the same starts;
      frac_z_gt_3    fraction of bins with |Δ| > 3√s (e^-9 = 1.2e-4 for complex Gaussian noise
                     of independent samples);
      noise_rel      √(Σs / Σ|mean_b|²): the relative size of the statistical error bars;
      rel_rms_diff   √(Σ|Δ|² / Σ|mean_b|²): the RMS per-bin difference relative to the RMS bin.
                     E|Δ|² is the squared systematic difference plus noise, so this bounds the
                     systematic per-bin difference from above;
      bias_rel       √(max(0, Σ|Δ|² − Σs) / Σ|mean_b|²): the difference beyond the error bars
                     (meaningful for independent samples);
      rms_ratio      √(Σ|mean_a|² / Σ|mean_b|²).
    """
    out = np.zeros(9)
    sc_a._check(sc_a._lib.sgb_corr_compare(sc_a._h, sc_b._h, _abi.dptr(out)))
    d2, s, s2, mb2, ma2, nz3, npos, nbins, varB = out
    return {"chi2_ratio": d2 / s if s > 0 else math.nan,
            "frac_z_gt_3": nz3 / max(npos, 1.0),
            "noise_rel": math.sqrt(s / mb2) if mb2 > 0 else math.nan,
            "rel_rms_diff": math.sqrt(d2 / mb2) if mb2 > 0 else math.nan,
            "bias_rel": math.sqrt(max(0.0, d2 - s) / mb2) if mb2 > 0 else math.nan,
            "rms_ratio": math.sqrt(ma2 / mb2) if mb2 > 0 else math.nan,
            "bins": int(nbins), "samples": (sc_a.nsamples, sc_b.nsamples)}


def systematic_difference(a1: SampledCorrelations, b1: SampledCorrelations, a2: SampledCorrelations,
                          b2: SampledCorrelations) -> dict:
    """Systematic per-bin difference between two sampling paths a and b (no counterpart in
    the reference), from paired samples split into two halves of disjoint starts: a1/b1
    hold the first half on each path, a2/b2 the second (calculate_errors on all four).
    With D_h = mean_a_h − mean_b_h per bin, E[Re Σ D1·conj(D2)] is the squared systematic
    difference summed over bins, since the halves' noise is independent. Returns
      bias_rel        √(max(0, Σ Re D1·conj(D2)) / Σ|mean_b|²), the RMS systematic
                      difference relative to the RMS bin;
      bias_rel_upper  √((max(0, Σ Re D1·conj(D2)) + 2 sd) / Σ|mean_b|²), a bound that two
                      standard deviations of the cross sum (estimated from partial sums over
                      interleaved bin sets) keep above the estimate even when noise makes
                      the cross sum negative;
      cross_rel2      the cross sum over Σ|mean_b|² (may be negative by noise)."""
    out = np.zeros(3)
    a1._check(a1._lib.sgb_corr_cross(a1._h, b1._h, a2._h, b2._h, _abi.dptr(out)))
    t0, t1, var = out
    sd = math.sqrt(max(var, 0.0))
    return {"bias_rel": math.sqrt(max(0.0, t0) / t1) if t1 > 0 else math.nan,
            "bias_rel_upper": math.sqrt((max(0.0, t0) + 2 * sd) / t1) if t1 > 0 else math.nan,
            "cross_rel2": t0 / t1 if t1 > 0 else math.nan,
            "cross_rel2_sd": sd / t1 if t1 > 0 else math.nan}


def merge_host(datas, counts, Ms=None):
    """merge_correlations' arithmetic on host arrays (SampledCorrelations.jl:128-142): the
    count-weighted mean of the data and, with Ms, the combined Welford M. Used to merge
    accumulators read back from several processes (one GPU each)."""
    d = np.array(datas[0], dtype=complex)
    n = int(counts[0])
    M = None if Ms is None else np.array(Ms[0], dtype=float)
    for k in range(1, len(datas)):
        m = int(counts[k])
        if n + m == 0:
            continue
        mu = (n / (n + m)) * d + (m / (n + m)) * datas[k]
        if M is not None:
            M = (M + n * np.abs(mu - d) ** 2) + (Ms[k] + m * np.abs(mu - datas[k]) ** 2)
        d, n = mu, n + m
    return d, n, M


def allreduce_correlations(data, count, M=None, group=None):
    """Merge one accumulator per process (replicas on several GPUs) with torch.distributed:
    every rank returns the merged (data, count, M), identical to merge_host over the
    ranks' accumulators. The reductions are two sums over ranks, so any backend works
    (gloo on CPU, NCCL on GPU tensors)."""
    import torch
    import torch.distributed as dist
    c = torch.tensor([float(count)], dtype=torch.float64)
    dist.all_reduce(c, group=group)
    total = c.item()
    d = np.asarray(data, dtype=complex)
    w = torch.from_numpy(np.ascontiguousarray(np.stack([d.real, d.imag]) * float(count)))
    dist.all_reduce(w, group=group)
    mu = (w[0].numpy() + 1j * w[1].numpy()) / total if total > 0 else np.zeros_like(d)
    Mt = None
    if M is not None:
        # M = Σ_r [M_r + n_r |d_r - μ|²]: the per-rank Welford sums about the common mean
        part = torch.from_numpy(np.ascontiguousarray(np.asarray(M, dtype=float) + count * np.abs(d - mu) ** 2))
        dist.all_reduce(part, group=group)
        Mt = part.numpy()
    return mu, int(round(total)), Mt


def available_energies(sc: SampledCorrelations, negative_energies: bool = False):
    """CorrelationUtils.jl:29-37."""
    if math.isnan(sc.dw):
        return math.nan
    n = sc.n_all_omega
    nonneg = n // 2 + 1
    w = np.fft.fftfreq(n, 1.0 / (n * sc.dw))
    w[nonneg - 1] *= -1
    return w if negative_energies else w[:nonneg]


def available_wave_vectors(sc: SampledCorrelations):
    """CorrelationUtils.jl:9-19 (no reshaping): q in RLU for every data index."""
    Ls = sc.sys.dims
    offs = [1 if L % 2 else 0 for L in Ls]
    hi = [L - L // 2 - o for L, o in zip(Ls, offs)]
    lo = [1 - L // 2 - o for L, o in zip(Ls, offs)]
    grids = [np.arange(l, h + 1) / L for l, h, L in zip(lo, hi, Ls)]
    return np.stack(np.meshgrid(*grids, indexing="ij"), -1)


# ---- intensities (DataRetrieval.jl:1-181, PhaseAveraging.jl) ---------------------------------

class Intensities:
    """Intensities(crystal, qpts, energies, data): data[ω, q] (static: data[q])."""

    def __init__(self, crystal, qpts, energies, data):
        self.crystal, self.qpts, self.energies, self.data = crystal, qpts, energies, data


def _energy_indices(sc: SampledCorrelations, energies):
    """Energy axis indices (DataRetrieval.jl:64-71, 85-95)."""
    n = sc.n_all_omega
    if math.isnan(sc.dw):
        return np.array([math.nan]), np.array([0], dtype=np.int32)
    if isinstance(energies, str) and energies == "available":
        w = available_energies(sc)
        return w, np.arange(len(w), dtype=np.int32)
    if isinstance(energies, str) and energies == "available_with_negative":
        w = available_energies(sc, negative_energies=True)
        return w, np.arange(n, dtype=np.int32)
    ref = available_energies(sc, negative_energies=True)
    energies = np.asarray(energies, dtype=float)
    if np.any(np.diff(energies) < 0):
        raise ValueError("Specified energies must be an ordered list.")
    if energies.min() < ref.min() or energies.max() > ref.max():
        raise ValueError("Specified energies includes values for which there is no available data.")
    idx = []
    for val in energies:
        # find_idx_of_nearest_fft_energy (DataRetrieval.jl:37-58)
        found = None
        for i in range(len(ref) - 1):
            x1, x2 = ref[i], ref[i + 1]
            if x1 <= val <= x2:
                found = i if abs(x1 - val) < abs(x2 - val) else i + 1
                break
        if found is None and ref[-1] <= val <= 0.0:
            found = len(ref) - 1 if abs(ref[-1] - val) <= abs(val) else 0
        if found is None:
            raise ValueError("Value does not lie in bounds of reference list.")
        idx.append(found)
    idx = np.array(idx, dtype=np.int32)
    return ref[idx], idx


def intensities(sc: SampledCorrelations, qpts, *, energies="available", kT=None):
    """intensities(sc, qpts; energies, kT) (DataRetrieval.jl:77-143): wave vectors in RLU
    are rounded to the accumulator's grid (pruned_wave_vector_info), phase-averaged with
    form factors and combined on the device; returns data[ω, q]."""
    if kT is not None and kT <= 0:
        raise ValueError("Positive `kT` required for classical-to-quantum corrections, or set `kT=nothing` to disable.")
    proto = sc._batch.proto if sc._batch is not None else sc.sys
    cr = proto.crystal
    Ls = np.array(proto.dims)
    qs = np.atleast_2d(np.asarray(qpts, dtype=float))
    ms = np.rint(qs * Ls[None, :]).astype(np.int64)           # round to nearest (ties to even)
    wrapped = np.mod(ms, Ls[None, :])
    qidx = np.ascontiguousarray(wrapped[:, 0] + Ls[0] * (wrapped[:, 1] + Ls[1] * wrapped[:, 2]), dtype=np.int32)
    qrlu = ms / Ls[None, :]
    qabs = qrlu @ cr.recipvecs.T                                # recipvecs * (m ./ dims)
    pos = np.array([cr._pos[a] for a in range(proto.natoms)])
    ffs = sc.measure.formfactors
    q2 = np.sum(qabs * qabs, axis=1)
    ff = np.ones((len(qs), proto.natoms))
    if ffs is not None:
        for a, f in enumerate(ffs):
            if f is not None:
                ff[:, a] = [f(x) for x in q2]
    pref = ff * np.exp(-2j * np.pi * (qrlu @ pos.T))           # prefactors_for_phase_averaging
    pbuf = np.ascontiguousarray(np.stack([pref.real, pref.imag], -1).reshape(-1))
    ws, widx = _energy_indices(sc, energies)
    widx = np.ascontiguousarray(widx, dtype=np.int32)
    kind = sc.measure.kind
    comb = {"trace": 0, "perp": 1}.get(kind, 2)
    if comb < 2 and [tuple(p) for p in sc.measure.corr_pairs] != CORR_PAIRS:
        comb = 2
    nq, nw = len(qs), len(widx)
    ncorr = len(sc.measure.corr_pairs)
    out = np.zeros(nq * nw * (2 * ncorr if comb == 2 else 1))
    qc = np.ascontiguousarray(qabs, dtype=float).reshape(-1)
    sc._check(sc._lib.sgb_corr_intensities(sc._h, nq, qidx.ctypes.data_as(C.POINTER(C.c_int32)), _abi.dptr(pbuf),
                                           _abi.dptr(qc), nw, widx.ctypes.data_as(C.POINTER(C.c_int32)), comb,
                                           _abi.dptr(out)))
    if comb == 2:
        el = out.reshape(nq, nw, ncorr, 2)
        el = el[..., 0] + 1j * el[..., 1]
        vals = np.array([[sc.measure.combiner(qabs[k], el[k, t]) for t in range(nw)] for k in range(nq)], dtype=float)
    else:
        vals = out.reshape(nq, nw)
    data = vals.T.copy()                                       # [ω, q]
    if not math.isnan(sc.dw):
        data /= sc.n_all_omega * sc.dw
        if kT is not None:
            c2q = np.array([1.0 if w == 0 else abs((w / kT) / (1 - math.exp(-w / kT))) for w in ws])
            data *= c2q[:, None]
        return Intensities(cr, qs, ws, data)
    return Intensities(cr, qs, None, data[0])


def intensities_static(sc: SampledCorrelations, qpts, *, bounds=(-math.inf, math.inf), kT=None):
    """intensities_static (DataRetrieval.jl:159-177): energy-integrated intensities."""
    if math.isnan(sc.dw):
        return intensities(sc, qpts, energies="available", kT=None)
    ws = available_energies(sc, negative_energies=True)
    sel = [w for w in ws if bounds[0] <= w < bounds[1]]
    if not sel:
        raise ValueError("No information available within specified energy `bounds`. Try a larger interval.")
    res = intensities(sc, qpts, kT=kT, energies=sorted(sel))
    return Intensities(res.crystal, res.qpts, None, res.data.sum(axis=0) * sc.dw)
