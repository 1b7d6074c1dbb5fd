#!/usr/bin/env python
"""Benchmark: S(q,ω) samples/s (and site-steps/s) on one GB300.

Workload: dipole-mode pyrochlore Heisenberg antiferromagnet, 16x16x16 conventional cells
x 16 sites (65,536 spins), s=3/2, J1=1.0 meV, J2=0.05 meV; thermalised by Langevin at
kT=0.2 meV (damping 0.1); then SampledCorrelations with ImplicitMidpoint (dt=0.025 ->
0.024933, measurement period 21), energies 0..6 meV in 200 bins (n_all_ω = 398), 3x3 spin
correlations (ssf_trace: 6 pairs x 16 x 16 sublattices). One step = one add_sample!: a
4,179-step implicit-midpoint trajectory with 200 snapshots, space and time FFTs and the
FP64 accumulation of 2.5e9 complex bins (40 GB).

Arms: the FP32 path (FP32 state and arithmetic, FP64 convergence sums, energies and
accumulator) is the headline; the plain FP64 path is timed beside it. `--impl reference`
times the CPU restatement of Sunny's algorithm (the FP64 oracle) on the host cores.

Data are synthetic (seeded random initial spins); no dataset is involved.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "site-steps/s & S(q,ω) samples/s: FP32/batched vs plain FP64 GPU at stated error"
L = 16
NOMEGA = 200
WMAX = 6.0
DT = 0.025


# DRAM bytes (dram__bytes read + write) per full-size launch of the dominant kernel: the
# snapshot stream plus L2 write-backs, both per step, so scaled by steps from the capture.
# ncu, k_batch_midpoint at L = 16 with 8 replicas, nω = 20 (399 steps, 805 iterations), the
# shared-index tile shape: DRAM read + write per launch, scaled to the headline's 4,179
# steps; and L2 sectors × 32 B per site-iteration per tile shape (by neighbour-index
# source), with the L2 peak that ncu's lts__throughput implies (12.0 TB/s at 35.8 %). The
# global-index figure was measured before steps were accepted lazily and is lowered by the
# 39.5 B per site-iteration that change removed from the shared-index shape (the
# acceptance traffic does not depend on where the neighbour indices come from).
DRAM_BYTES_PER_LAUNCH = {"k_batch_midpoint": (0.099e9 + 6.158e9) * 4179 / 399}
L2_BYTES_PER_SITE_ITER = {2: 402.5, 0: 463.5}
L2_PEAK_GBS_NCU = 33400.0


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, dev: int):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                       "-lms", "200", "-i", str(dev)], stdout=subprocess.PIPE,
                                      stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        out, _ = self.p.communicate(timeout=10)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def build_system(sg, precision, device, seed=1):
    """The pyrochlore model at the module-level size L."""
    cr = sg.pyrochlore_crystal()
    sys_ = sg.System(cr, [(1, sg.Moment(s=1.5, g=2))], "dipole", dims=(L, L, L), seed=seed, precision=precision,
                     device=device)
    sys_.set_exchange(1.0, cr.bonds_at_distance(math.sqrt(2) / 4)[0])
    sys_.set_exchange(0.05, cr.bonds_at_distance(math.sqrt(6) / 4)[0])
    sys_.randomize_spins()
    return sys_


def run_arm(sg, precision, device, warmup, steps, tol, thermal_steps=2000, e2e_steps=0):
    lib = sg.load_library()
    sys_ = build_system(sg, precision, device)
    sg.step(sys_, sg.Langevin(DT, damping=0.1, kT=0.2), nsteps=thermal_steps)
    sc = sg.SampledCorrelations(sys_, measure=sg.ssf_trace(sys_), energies=np.linspace(0, WMAX, NOMEGA), dt=DT,
                                tol=tol)
    for _ in range(warmup):
        sg.add_sample(sc, sys_)
    lib.sgb_synchronize(sys_.handle)
    lib.sgb_corr_profile(sc._h, 1)
    launches0 = lib.sgb_kernel_launches(sys_.handle)
    clocks = Clocks(device)
    lib.sgb_event_record(sys_.handle, 0)
    for _ in range(steps):
        sg.add_sample(sc, sys_)
    lib.sgb_event_record(sys_.handle, 1)
    import ctypes as C
    ms = C.c_float()
    lib.sgb_event_elapsed(sys_.handle, 0, 1, C.byref(ms))
    clk = clocks.stop()
    launches = lib.sgb_kernel_launches(sys_.handle) - launches0
    ph = np.zeros(4)
    n = C.c_int64()
    its = C.c_int64()
    lib.sgb_corr_phase_times(sc._h, ph.ctypes.data_as(C.POINTER(C.c_double)), C.byref(n), C.byref(its))
    lib.sgb_corr_profile(sc._h, 0)
    res = {"ms": ms.value, "phase_ms": (ph / max(1, n.value)).tolist(), "launches": launches, "clocks": clk,
           "nsamples": sc.nsamples, "nsteps_per_sample": sc.measperiod * (sc.n_all_omega // 2), "ns": sys_.nsites,
           "measperiod": sc.measperiod, "n_all_omega": sc.n_all_omega, "dt": sc.dt,
           "iters_per_step": its.value / max(1, n.value) / (sc.measperiod * (sc.n_all_omega // 2))}
    if e2e_steps:
        # end to end through the public API: pinned-host state in, add_sample, state out
        S = sys_.dipoles_flat()
        lib.sgb_synchronize(sys_.handle)
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            sys_.set_state_flat(dipoles=S)
            sg.add_sample(sc, sys_)
            S = sys_.dipoles_flat()
        t1 = time.perf_counter()
        res["e2e_s"] = t1 - t0
        res["e2e_steps"] = e2e_steps
        bytes_state = sys_.nsites * 3 * (4 if precision == "fp32" else 8)
        res["h2d"] = bytes_state
        res["d2h"] = bytes_state
    sc.close()
    sys_.close()
    return res


def stated_error(sg, device, L_=16, nomega=200, nrep=8, nsamples=32, decorr=1000, thermal_steps=2000, seed=11, tol32=1e-6,
                 first_accept=False, predictor=None):
    """Error of the FP32 batched S(q,w) path against the plain FP64 path on the pyrochlore
    model with L_^3 conventional cells (L_=16, nomega=200 is the benchmark workload).

    Each FP32 batched add_sample integrates nrep 4,179-step (at nomega=200) implicit-
    midpoint trajectories at tol 1e-6 with the degree-4 first iterate; the plain FP64 path
    (tol 1e-12, first iterate S' = S) integrates the same trajectories from the same
    starting states, one add_sample each (calculate_errors=true on both). A decorrelating
    Langevin run (kT 0.2, damping 0.1, `decorr` steps) precedes every batched pass after
    the first. The accumulators hold the benchmark's diagonal correlations S^xx, S^yy,
    S^zz (whose sum the benchmark's trace measure reports).
    Energy: the exact dynamics conserve it; the spherical midpoint method keeps it up to a
    bounded O(dt^2) oscillation, so the relative change over each trajectory is reported
    for both paths, with the FP32 - FP64 difference at the end of the first trajectory.
    S(q,w): two trajectories from one start separate by chaos whatever the arithmetic, so a
    per-sample difference is mostly noise. The samples are split into two halves of
    disjoint starts, each half accumulated on both paths. Per half, compare_correlations
    checks the difference bin by bin against the Welford error bars. Across halves, the
    paired differences D1 and D2 have independent noise, so Re sum D1 conj(D2) estimates the
    squared systematic difference alone (sgb_corr_cross); relative to the RMS bin it gives
    the systematic per-bin difference of the FP32 path, with an upper bound from the
    estimate plus two standard deviations."""
    cr = sg.pyrochlore_crystal()

    def model(precision, dev):
        s_ = sg.System(cr, [(1, sg.Moment(s=1.5, g=2))], "dipole", dims=(L_, L_, L_), seed=seed, precision=precision,
                       device=dev)
        s_.set_exchange(1.0, cr.bonds_at_distance(math.sqrt(2) / 4)[0])
        s_.set_exchange(0.05, cr.bonds_at_distance(math.sqrt(6) / 4)[0])
        s_.randomize_spins()
        return s_

    energies = np.linspace(0, WMAX, nomega)
    proto = model("fp32", None)
    b = sg.ReplicaBatch(proto, [proto.dims] * nrep, kT=[0.2] * nrep, precision="fp32", device=device, seed=seed)
    if predictor is not None:
        b.set_midpoint_predictor(predictor)
    if first_accept:
        b.set_midpoint_first_accept(True)
    b.randomize_spins()
    b.langevin(DT, 0.1, thermal_steps)
    s64 = model("fp64", device)
    diag = sg.MeasureSpec(sg.ssf_trace(proto).observables, [(1, 1), (2, 2), (3, 3)])
    kw = dict(measure=diag, energies=energies, dt=DT, calculate_errors=True)
    sc32 = [sg.SampledCorrelations(b, tol=tol32, **kw) for _ in range(2)]
    sc64 = [sg.SampledCorrelations(s64, tol=1e-12, **kw) for _ in range(2)]
    nsteps = sc32[0].measperiod * (sc32[0].n_all_omega // 2)
    npass = max(2, nsamples // nrep)
    e32, e64 = [], []
    end_diff = None
    t0 = time.perf_counter()
    for p in range(npass):
        half = 0 if p < npass // 2 else 1
        if p:
            b.langevin(DT, 0.1, decorr)
        starts = [b.get_state(r) for r in range(nrep)]
        Ea = b.energies()
        sg.add_sample(sc32[half], b)
        Eb = b.energies()
        e32.extend(np.abs(Eb - Ea) / np.abs(Ea))
        for r in range(nrep):
            s64.set_state_flat(dipoles=starts[r])
            E0 = sg.energy(s64)
            sg.add_sample(sc64[half], s64)
            E1 = sg.energy(s64)
            e64.append(abs(E1 - E0) / abs(E0))
            if end_diff is None:
                end_diff = abs(Eb[r] - E1) / abs(E1)
    halves = [sg.compare_correlations(sc32[h], sc64[h]) for h in range(2)]
    sysd = sg.systematic_difference(sc32[0], sc64[0], sc32[1], sc64[1])
    wall = time.perf_counter() - t0
    for c in sc32 + sc64:
        c.close()
    b.close()
    s64.close()
    e32 = np.array(e32)
    return {"workload": f"pyrochlore {L_}^3 x 16 ({16 * L_**3} spins), nw={nomega}, {nsteps} midpoint steps per sample, "
                        f"{npass * nrep} samples per path from the same starts ({nrep} replicas x {npass} passes "
                        f"on FP32, two halves of {npass // 2 * nrep}), {decorr} Langevin steps between passes, "
                        "S^xx, S^yy, S^zz",
            "energy_rel_err_per_sample_max": float(e32.max()),
            "energy_rel_err_per_sample_median": float(np.median(e32)),
            "energy_rel_err_per_step": float(e32.max()) / nsteps,
            "fp64_energy_rel_err_per_sample_max": float(max(e64)),
            "fp64_energy_rel_err_per_sample_median": float(np.median(e64)),
            "energy_rel_diff_fp32_fp64_same_start": float(end_diff),
            "sqw_vs_fp64_halves": halves,
            "sqw_systematic": sysd,
            "sqw_systematic_rel_rms": sysd["bias_rel"],
            "sqw_systematic_rel_rms_upper": sysd["bias_rel_upper"],
            "steps_per_sample": nsteps, "wall_s": wall, "fp32_tol": tol32, "first_accept": first_accept,
            "predictor": predictor,
            "limits": {"energy_rel_err": 1e-5, "sqw_per_bin_rel": 1e-2}}


def run_batched(sg, device, nrep, warmup, steps, tol, thermal_steps=2000, predictor=None, mid_shape=None,
                first_accept=False):
    """Batched FP32 sampling: `nrep` replicas of the pyrochlore model advance in one
    persistent launch; each add_sample adds nrep samples with a rank-nrep accumulator pass.
    `mid_shape` (a row of sgb_batch_midpoint_shapes) replaces the autotuner's choice after
    the first warm-up sample, e.g. to profile one shape."""
    import ctypes as C
    lib = sg.load_library()
    proto = build_system(sg, "fp32", None)
    b = sg.ReplicaBatch(proto, [proto.dims] * nrep, kT=[0.2] * nrep, precision="fp32", device=device, seed=7)
    if predictor is not None:
        b.set_midpoint_predictor(predictor)
    if first_accept:
        b.set_midpoint_first_accept(True)
    b.randomize_spins()
    b.langevin(DT, 0.1, thermal_steps)
    sc = sg.SampledCorrelations(b, measure=sg.ssf_trace(proto), energies=np.linspace(0, WMAX, NOMEGA), dt=DT, tol=tol)
    for w in range(warmup):
        sg.add_sample(sc, b)
        if w == 0 and mid_shape is not None:
            if lib.sgb_batch_select_midpoint_shape(b.handle, int(mid_shape)) != 0:
                raise ValueError(f"no midpoint shape row {mid_shape}")
    lib.sgb_corr_profile(sc._h, 1)
    launches0 = lib.sgb_batch_kernel_launches(b.handle)
    clocks = Clocks(device)
    lib.sgb_batch_event_record(b.handle, 0)
    for _ in range(steps):
        sg.add_sample(sc, b)
    lib.sgb_batch_event_record(b.handle, 1)
    ms = C.c_float()
    lib.sgb_batch_event_elapsed(b.handle, 0, 1, C.byref(ms))
    clk = clocks.stop()
    ph = np.zeros(4)
    n = C.c_int64()
    its = C.c_int64()
    lib.sgb_corr_phase_times(sc._h, ph.ctypes.data_as(C.POINTER(C.c_double)), C.byref(n), C.byref(its))
    nsteps_sample = sc.measperiod * (sc.n_all_omega // 2)
    res = {"ms": ms.value, "phase_ms": (ph / max(1, n.value)).tolist(), "launches": lib.sgb_batch_kernel_launches(b.handle) - launches0,
           "clocks": clk, "nrep": nrep, "ns": proto.nsites, "nsteps_per_sample": nsteps_sample,
           "iters_per_step": its.value / max(1, n.value) / nsteps_sample, "n_all_omega": sc.n_all_omega}
    shapes = (C.c_int32 * (7 * 16))()
    tms = (C.c_float * 16)()
    chosen = C.c_int32(-1)
    nsh = lib.sgb_batch_midpoint_shapes(b.handle, 16, shapes, tms, C.byref(chosen))

    def shape(k):
        r = shapes[7 * k:7 * k + 7]
        d = {"kernel": "cell blocks" if r[5] else "sublattice tiles", "bonds_gathered": r[1], "ctas_per_sm": r[2],
             "grid": r[3], "smem": r[4], "tune_ms_3_steps": round(tms[k], 4)}
        if r[5]:
            d["block_cells"] = [r[6] & 0xff, (r[6] >> 8) & 0xff, (r[6] >> 16) & 0xff]
            d["threads"] = 32 * ((r[6] >> 24) & 0xff)
        else:
            d["nbr_index_bytes_smem"] = r[0]
        return d
    res["midpoint_shapes"] = {"chosen": chosen.value, "shapes": [shape(k) for k in range(max(0, min(nsh, 16)))]}
    # end to end: every replica's state in from host memory, add_sample, every state out
    states = [b.get_state(r) for r in range(nrep)]
    t0 = time.perf_counter()
    e2e_steps = max(2, steps // 2)
    for _ in range(e2e_steps):
        for r in range(nrep):
            b.set_state(r, states[r])
        sg.add_sample(sc, b)
        states = [b.get_state(r) for r in range(nrep)]
    res["e2e_s"] = time.perf_counter() - t0
    res["e2e_steps"] = e2e_steps
    res["h2d"] = res["d2h"] = nrep * proto.nsites * 3 * 4
    sc.close()
    b.close()
    return res


def run_tempering(sg, device, nsteps=20000, exch_interval=100, seed=2024):
    """256 simple-cubic replicas, L drawn uniformly from {8,12,16,24,32}, kT on a geometric
    0.1-2.0 ladder, J=1, -0.1 Sz^2, Langevin damping 0.2, exchanges every 100 steps within
    groups of equal L; FP32 state, FP64 energies; one CUDA graph per exchange round."""
    import ctypes as C
    lib = sg.load_library()
    rng = np.random.default_rng(seed)
    Ls = rng.choice([8, 12, 16, 24, 32], size=256)
    kT = np.geomspace(0.1, 2.0, 256)
    proto = sg.System(sg.cubic_crystal(), [(1, sg.Moment(s=1, g=2))], "dipole", dims=(8, 8, 8), seed=1, device=None)
    proto.set_exchange(1.0, sg.Bond(1, 1, [1, 0, 0]))
    proto.set_onsite_coupling(lambda Sx, Sy, Sz: -0.1 * Sz @ Sz, 1)
    b = sg.ReplicaBatch(proto, [(int(L),) * 3 for L in Ls], kT=kT, precision="fp32", device=device, seed=seed)
    b.randomize_spins()
    pt = sg.ParallelTempering(b, 0.02, 0.2)
    pt.step_ensemble(2 * exch_interval, exch_interval)          # warm-up (graph capture)
    lib.sgb_batch_event_record(b.handle, 0)
    pt.step_ensemble(nsteps, exch_interval)
    lib.sgb_batch_event_record(b.handle, 1)
    ms = C.c_float()
    lib.sgb_batch_event_elapsed(b.handle, 0, 1, C.byref(ms))
    nsites = int(sum(int(L) ** 3 for L in Ls))
    acc = pt.n_accept.sum()
    hms = (C.c_float * 3)()
    hb = C.c_int32(0)
    lib.sgb_batch_langevin_shapes(b.handle, hms, C.byref(hb))
    out = {"site_steps_per_s": nsites * nsteps / (ms.value / 1000.0), "ms": ms.value, "steps": nsteps,
           "replicas": 256, "total_sites": nsites, "graph": pt.graph_active, "accepted_swaps": int(acc),
           "us_per_step": 1000.0 * ms.value / nsteps,
           "langevin_autotune": {"ctas_per_sm": hb.value,
                                 "tune_ms_10_steps": {str(k): (None if hms[i] >= 1e29 else round(hms[i], 4))
                                                      for i, k in enumerate((4, 3, 2))}}}
    b.close()
    return out


def dynamics_rate(sg, kind, precision, device, nsteps):
    """Site-steps/s of plain Langevin dynamics for the other two single-system workloads:
    'sc'  -- simple cubic 16^3, s=1, J=1, -0.1 Sz^2, dt=0.02, damping 0.1, kT=0.5 (dipole)
    'tri' -- layered triangular 48x48x4 SU(3), anisotropic J1, J2, J3, Jc, -2.2 Sz^2,
             dt=0.02 (assumed), damping 0.1, kT=0.3."""
    import ctypes as C
    lib = sg.load_library()
    if kind == "sc":
        sys_ = sg.System(sg.cubic_crystal(), [(1, sg.Moment(s=1, g=2))], "dipole", dims=(16, 16, 16), seed=1,
                         precision=precision, device=device)
        sys_.set_exchange(1.0, sg.Bond(1, 1, [1, 0, 0]))
        sys_.set_onsite_coupling(lambda Sx, Sy, Sz: -0.1 * Sz @ Sz, 1)
        integ = sg.Langevin(0.02, damping=0.1, kT=0.5)
    else:
        cr = sg.triangular_crystal(a=4.05, c=6.75)
        sys_ = sg.System(cr, [(1, sg.Moment(s=1, g=2))], "SUN", dims=(48, 48, 4), seed=1, precision=precision,
                         device=device)
        J1 = np.array([[-0.24, 0, 0], [0, -0.24, 0.1], [0, 0.1, -0.24]])
        sys_.set_exchange(J1, sg.Bond(1, 1, [1, 0, 0]))
        sys_.set_exchange(0.05, sg.Bond(1, 1, [1, 2, 0]))
        sys_.set_exchange(0.32, sg.Bond(1, 1, [2, 0, 0]))
        sys_.set_exchange(-0.05, sg.Bond(1, 1, [0, 0, 1]))
        sys_.set_onsite_coupling(lambda Sx, Sy, Sz: -2.2 * Sz @ Sz, 1)
        integ = sg.Langevin(0.02, damping=0.1, kT=0.3)
    sys_.randomize_spins()
    sg.step(sys_, integ, nsteps=200)
    lib.sgb_synchronize(sys_.handle)
    lib.sgb_event_record(sys_.handle, 0)
    sg.step(sys_, integ, nsteps=nsteps)
    lib.sgb_event_record(sys_.handle, 1)
    ms = C.c_float()
    lib.sgb_event_elapsed(sys_.handle, 0, 1, C.byref(ms))
    E = sg.energy_per_site(sys_)
    ns = sys_.nsites
    M = sg.magnetization(sys_) / ns
    kern = sys_.langevin_kernel()
    sys_.close()
    return {"site_steps_per_s": ns * nsteps / (ms.value / 1000.0), "us_per_step": 1000.0 * ms.value / nsteps,
            "kernel": f"cluster of {kern} CTAs" if kern > 0 else "grid",
            "nsites": ns, "steps": nsteps, "energy_per_site": E, "magnetization_per_site": M.tolist(),
            "abs_magnetization_per_site": float(np.linalg.norm(M))}


def batched_langevin_rate(sg, device, nrep=64, nsteps=2000):
    """Site-steps/s of FP32 Langevin on `nrep` copies of the simple cubic 16^3 model
    (s=1, J=1, -0.1 Sz^2, dt=0.02, damping 0.1, kT=0.5) advanced together in one persistent
    launch (the replica batch), with per-replica energy and magnetisation afterwards."""
    import ctypes as C
    lib = sg.load_library()
    proto = sg.System(sg.cubic_crystal(), [(1, sg.Moment(s=1, g=2))], "dipole", dims=(16, 16, 16), seed=1, device=None)
    proto.set_exchange(1.0, sg.Bond(1, 1, [1, 0, 0]))
    proto.set_onsite_coupling(lambda Sx, Sy, Sz: -0.1 * Sz @ Sz, 1)
    b = sg.ReplicaBatch(proto, [(16, 16, 16)] * nrep, kT=[0.5] * nrep, precision="fp32", device=device, seed=3)
    b.randomize_spins()
    b.langevin(0.02, 0.1, 200)
    lib.sgb_batch_event_record(b.handle, 0)
    b.langevin(0.02, 0.1, nsteps)
    lib.sgb_batch_event_record(b.handle, 1)
    ms = C.c_float()
    lib.sgb_batch_event_elapsed(b.handle, 0, 1, C.byref(ms))
    ns = 16 ** 3
    E = b.energies() / ns
    Ms = np.array([np.mean(b.get_state(r), axis=0) for r in range(nrep)])
    b.close()
    return {"site_steps_per_s": nrep * ns * nsteps / (ms.value / 1000.0), "us_per_step": 1000.0 * ms.value / nsteps,
            "replicas": nrep, "nsites_per_replica": ns, "steps": nsteps, "energy_per_site_mean": float(E.mean()),
            "abs_magnetization_per_site_mean": float(np.mean(np.linalg.norm(Ms, axis=1)))}


def local_sampler_rate(sg, precision, device, nsweeps=200):
    """Single-spin Metropolis proposals/s of the LocalSampler on the simple cubic 16^3
    model (s=1, J=1, -0.1 Sz^2) at kT=0.5 with propose_delta(0.3): colour-class parallel
    sweeps in one persistent launch."""
    import ctypes as C
    lib = sg.load_library()
    sys_ = sg.System(sg.cubic_crystal(), [(1, sg.Moment(s=1, g=2))], "dipole", dims=(16, 16, 16), seed=1,
                     precision=precision, device=device)
    sys_.set_exchange(1.0, sg.Bond(1, 1, [1, 0, 0]))
    sys_.set_onsite_coupling(lambda Sx, Sy, Sz: -0.1 * Sz @ Sz, 1)
    sys_.randomize_spins()
    smp = sg.LocalSampler(kT=0.5, propose=sg.propose_delta(0.3))
    sg.step(sys_, smp, 20)
    lib.sgb_synchronize(sys_.handle)
    lib.sgb_event_record(sys_.handle, 0)
    sg.step(sys_, smp, nsweeps)
    lib.sgb_event_record(sys_.handle, 1)
    ms = C.c_float()
    lib.sgb_event_elapsed(sys_.handle, 0, 1, C.byref(ms))
    ns = sys_.nsites
    ncol, _ = sg.local_colors(sys_)
    E = sg.energy_per_site(sys_)
    sys_.close()
    return {"proposals_per_s": ns * nsweeps / (ms.value / 1000.0), "us_per_sweep": 1000.0 * ms.value / nsweeps,
            "nsites": ns, "sweeps": nsweeps, "colour_classes": ncol, "energy_per_site": E}


def run_adjoint(sg, device, L_=24, nw=64, checkpoint=64):
    """Differentiation workload: simple cubic 24^3 dipole lattice (13,824 spins, s=1) from a
    state thermalised by Langevin at kT=0.3; parameters J1 (1.0), J2 (0.1), D (0.05, onsite
    -D Sz^2); loss = mean squared difference of one sample's S(q,w) (nw=64 up to 16 meV:
    dt 0.025 -> 0.02454, measurement period 8, 504 midpoint steps) against the sample at
    J1=1.1, J2=0.08, D=0.07 from the same state; adjoint with a checkpoint every 64 steps,
    checked by central differences (h=1e-4) of the same loss."""
    params = [lambda s_, v: s_.set_exchange(v, sg.Bond(1, 1, [1, 0, 0])),
              lambda s_, v: s_.set_exchange(v, sg.Bond(1, 1, [1, 1, 0])),
              lambda s_, v: s_.set_onsite_coupling(lambda Sx, Sy, Sz: -v * Sz @ Sz, 1)]
    theta0, theta_t = np.array([1.0, 0.1, 0.05]), np.array([1.1, 0.08, 0.07])
    s = sg.System(sg.cubic_crystal(), [(1, sg.Moment(s=1, g=2))], "dipole", dims=(L_, L_, L_), seed=5, device=device)
    for f, v in zip(params, theta0):
        f(s, float(v))
    s.randomize_spins()
    sg.step(s, sg.Langevin(0.02, damping=0.1, kT=0.3), nsteps=1000)
    S0 = s.dipoles_flat()
    adj = sg.SampledCorrelationsAdjoint(s, params, measure=sg.ssf_trace(s), energies=np.linspace(0.0, 16.0, nw),
                                        dt=0.025)
    adj.set_params(theta_t)
    _, target = adj.loss(S0, return_data=True)
    adj.set_target(target)
    adj.set_params(theta0)
    adj.loss_and_grad(S0, checkpoint=checkpoint)          # warm-up (plans, buffers)
    t0 = time.perf_counter()
    loss, g = adj.loss_and_grad(S0, checkpoint=checkpoint)
    t_adj = time.perf_counter() - t0
    t0 = time.perf_counter()
    adj.loss(S0)
    t_fwd = time.perf_counter() - t0
    fd = np.zeros(3)
    for k in range(3):
        e = np.zeros(3)
        e[k] = 1e-4
        adj.set_params(theta0 + e)
        lp = adj.loss(S0)
        adj.set_params(theta0 - e)
        lm = adj.loss(S0)
        fd[k] = (lp - lm) / 2e-4
    adj.close()
    s.close()
    return {"workload": f"simple cubic {L_}^3 (13,824 spins) dipole, J1/J2/D, nw={nw}, {adj.nsteps} midpoint steps, "
                        f"checkpoint every {checkpoint}", "loss": loss, "grad": g.tolist(), "fd_grad": fd.tolist(),
            "fd_rel_err": float(np.linalg.norm(g - fd) / np.linalg.norm(fd)), "ms_loss_and_grad": 1000 * t_adj,
            "ms_forward_only": 1000 * t_fwd, "dtype": "f64"}


def run_c3_sqw(sg, device, precision, nsamples):
    """S(q,w) samples/s of the SU(3) workload: layered triangular 48x48x4 (9,216 sites), spin-1
    coherent states, anisotropic J1, J2, J3, Jc, -2.2 Sz^2; Langevin at kT=0.3 (damping 0.1),
    then SampledCorrelations with nw=150 up to 7.5 meV (dt 0.025 -> measurement period 17,
    2,533 midpoint steps per sample), ssf_perp."""
    import ctypes as C
    lib = sg.load_library()
    cr = sg.triangular_crystal(a=4.05, c=6.75)
    s = sg.System(cr, [(1, sg.Moment(s=1, g=2))], "SUN", dims=(48, 48, 4), seed=1, precision=precision, device=device)
    J1 = np.array([[-0.24, 0, 0], [0, -0.24, 0.1], [0, 0.1, -0.24]])
    s.set_exchange(J1, sg.Bond(1, 1, [1, 0, 0]))
    s.set_exchange(0.05, sg.Bond(1, 1, [1, 2, 0]))
    s.set_exchange(0.32, sg.Bond(1, 1, [2, 0, 0]))
    s.set_exchange(-0.05, sg.Bond(1, 1, [0, 0, 1]))
    s.set_onsite_coupling(lambda Sx, Sy, Sz: -2.2 * Sz @ Sz, 1)
    s.randomize_spins()
    sg.step(s, sg.Langevin(0.025, damping=0.1, kT=0.3), nsteps=1000)
    sc = sg.SampledCorrelations(s, measure=sg.ssf_perp(s), energies=np.linspace(0, 7.5, 150), dt=0.025,
                                tol=1e-6 if precision == "fp32" else 1e-12)
    sg.add_sample(sc, s)                                   # warm-up (plans)
    lib.sgb_synchronize(s.handle)
    lib.sgb_event_record(s.handle, 0)
    for _ in range(nsamples):
        sg.add_sample(sc, s)
    lib.sgb_event_record(s.handle, 1)
    ms = C.c_float()
    lib.sgb_event_elapsed(s.handle, 0, 1, C.byref(ms))
    out = {"samples_per_s": nsamples / (ms.value / 1000.0), "ms_per_sample": ms.value / nsamples,
           "steps_per_sample": sc.measperiod * (sc.n_all_omega // 2), "nsites": s.nsites}
    sc.close()
    s.close()
    return out


def run_c3_group(sg, device, nrep=8, passes=2):
    """The SU(3) workload of run_c3_sqw sampled as a replica group: `nrep` FP32 clones whose
    midpoint trajectories run concurrently (each on its own stream, an equal share of the
    SMs), one rank-nrep accumulation per batched add_sample."""
    import ctypes as C
    lib = sg.load_library()
    cr = sg.triangular_crystal(a=4.05, c=6.75)
    p = sg.System(cr, [(1, sg.Moment(s=1, g=2))], "SUN", dims=(48, 48, 4), seed=1, precision="fp32", device=None)
    J1 = np.array([[-0.24, 0, 0], [0, -0.24, 0.1], [0, 0.1, -0.24]])
    p.set_exchange(J1, sg.Bond(1, 1, [1, 0, 0]))
    p.set_exchange(0.05, sg.Bond(1, 1, [1, 2, 0]))
    p.set_exchange(0.32, sg.Bond(1, 1, [2, 0, 0]))
    p.set_exchange(-0.05, sg.Bond(1, 1, [0, 0, 1]))
    p.set_onsite_coupling(lambda Sx, Sy, Sz: -2.2 * Sz @ Sz, 1)
    b = sg.ReplicaBatch(p, [p.dims] * nrep, kT=[0.3] * nrep, precision="fp32", device=device, seed=1)
    b.randomize_spins()
    b.langevin(0.025, 0.1, 1000)
    sc = sg.SampledCorrelations(b, measure=sg.ssf_perp(p), energies=np.linspace(0, 7.5, 150), dt=0.025, tol=1e-6)
    sg.add_sample(sc, b)                                   # warm-up (plans, kernel choice)
    lib.sgb_batch_event_record(b.handle, 0)
    for _ in range(passes):
        sg.add_sample(sc, b)
    lib.sgb_batch_event_record(b.handle, 1)
    ms = C.c_float()
    lib.sgb_batch_event_elapsed(b.handle, 0, 1, C.byref(ms))
    out = {"samples_per_s": nrep * passes / (ms.value / 1000.0), "ms_per_pass": ms.value / passes, "replicas": nrep,
           "steps_per_sample": sc.measperiod * (sc.n_all_omega // 2), "nsites": p.nsites}
    sc.close()
    b.close()
    return out


# ---- CPU restatement (oracle) timing ----------------------------------------------------------

def _cpu_sample_worker(args):
    """Time a bounded part of one sample on one core: `nmid` midpoint steps and `nblk`
    (c, i, j) correlation blocks of the accumulation. Returns the extrapolated seconds
    for one full sample."""
    nmid, nblk, seed = args
    sys.path.insert(0, str(ROOT))
    import __graft_entry__ as ge
    sg = ge.package()
    orc = ge.oracle()
    sys_ = build_system(sg, "fp64", None, seed=seed)
    o = orc.OracleSystem.from_system(sys_)
    S = sys_.dipoles_flat()
    dt, mp = sg.adjusted_dt_and_downsampling_factor(DT, NOMEGA, WMAX)
    nsteps_sample = mp * (NOMEGA - 1)
    t0 = time.perf_counter()
    st, S, _, _ = o.midpoint(S, None, dt, 0.0, 1e-12, 100, nmid)
    t_step = (time.perf_counter() - t0) / nmid
    # accumulation: the sample FFTs (timed on one of the 3 x 16 observable rows and
    # scaled by 48) plus nblk of the 1536 pair blocks
    n = 2 * (NOMEGA - 1)
    rng = np.random.default_rng(seed)
    buf = np.zeros((1, L, L, L, 1, n), dtype=complex)
    buf[..., : n // 2 + 1] = rng.standard_normal((1, L, L, L, 1, n // 2 + 1))
    t0 = time.perf_counter()
    A = np.conj(np.fft.fftn(np.conj(buf), axes=(1, 2, 3))) / math.sqrt(L**3)
    A = np.fft.fft(A, axis=5)
    t_fft = (time.perf_counter() - t0) * 48
    T = n // 2 + 1
    offs = np.fft.fftfreq(n, 1.0 / n)
    ncontrib = (T - np.abs(offs)).astype(float)
    win = np.cos(np.linspace(0, np.pi, n + 1)[:-1]) ** 2
    data = np.zeros((L, L, L, n), dtype=complex)
    t0 = time.perf_counter()
    for b in range(nblk):
        corr = np.conj(A[0, :, :, :, 0, :]) * A[0, :, :, :, 0, :]
        corr = np.fft.fft(np.fft.ifft(corr, axis=3) / ncontrib * win, axis=3)
        data += (corr - data) * 0.5
    t_blk = (time.perf_counter() - t0) / nblk
    return t_step * nsteps_sample + t_fft + t_blk * 6 * 16 * 16, t_step


def cpu_baseline(threads: int, nmid: int, nblk: int):
    if threads <= 1:
        t_sample, t_step = _cpu_sample_worker((nmid, nblk, 1))
        return 1.0 / t_sample, 1, t_step
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    with ctx.Pool(threads) as pool:
        out = pool.map(_cpu_sample_worker, [(nmid, nblk, 1 + k) for k in range(threads)])
    return sum(1.0 / t for t, _ in out), threads, statistics.median(s for _, s in out)


def _cpu_c1_worker(args):
    """FP64 Langevin (the oracle's stochastic Heun) on the simple cubic 16^3 model (s=1,
    J=1, -0.1 Sz^2, dt 0.02, damping 0.1, kT 0.5) from a random state, on one core: returns
    (site-steps/s, energy per site, magnetisation per site) after `nsteps` steps."""
    nsteps, seed = args
    sys.path.insert(0, str(ROOT))
    import __graft_entry__ as ge
    sg = ge.package()
    orc = ge.oracle()
    s_ = sg.System(sg.cubic_crystal(), [(1, sg.Moment(s=1, g=2))], "dipole", dims=(16, 16, 16), seed=seed, device=None)
    s_.set_exchange(1.0, sg.Bond(1, 1, [1, 0, 0]))
    s_.set_onsite_coupling(lambda Sx, Sy, Sz: -0.1 * Sz @ Sz, 1)
    s_.randomize_spins()
    o = orc.OracleSystem.from_system(s_)
    S = s_.dipoles_flat()
    noise = np.random.default_rng(seed).standard_normal((nsteps, s_.nsites, 3))
    t0 = time.perf_counter()
    S, _ = o.langevin(S, None, 0.02, 0.1, 0.5, nsteps, noise)
    t = time.perf_counter() - t0
    return s_.nsites * nsteps / t, o.energy(S) / s_.nsites, (S.sum(0) / s_.nsites).tolist()


def cpu_c1(threads: int, nsteps: int):
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    with ctx.Pool(threads) as pool:
        out = pool.map(_cpu_c1_worker, [(nsteps, 1 + k) for k in range(threads)])
    M = np.array([m for _, _, m in out])
    return {"site_steps_per_s": sum(r for r, _, _ in out), "cores": threads, "steps_per_core": nsteps,
            "workload": "simple cubic 16^3 (4,096 spins) FP64 Langevin, one system per core",
            "energy_per_site_mean": float(np.mean([e for _, e, _ in out])),
            "abs_magnetization_per_site_mean": float(np.mean(np.linalg.norm(M, axis=1)))}


def reference_arm(args, rank, world):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    vals = []
    for _ in range(args.warmup):
        cpu_baseline(threads, 4, 4)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        v, cores, t_step = cpu_baseline(threads, 20, 12)
        vals.append(v)
    wall = time.perf_counter() - t0
    value = statistics.median(vals)
    sample = ("per core: 20 FP64 implicit-midpoint steps of the 65,536-spin pyrochlore and 12 of the 1,536 "
              "(c,i,j) correlation blocks plus the sample FFTs, extrapolated to one full add_sample; "
              f"{cores} independent systems in parallel (one per core)")
    line = {"metric": METRIC, "value": value, "unit": "samples/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * wall / max(1, args.steps), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": "pyrochlore 16x16x16x16 (65,536 spins) S(q,w) sampling, nw=200, 6 meV, "
                                   "ImplicitMidpoint dt=0.024933 x 21 per snapshot", "global_batch": 1, "seq_len": 1,
                       "parallelism": "replicas"},
            "cpu_baseline": {"value": value, "unit": "samples/s", "cores": cores, "kind": "port", "sample": sample},
            "c1_langevin": cpu_c1(threads, 2000),
            "e2e": {"value": value, "unit": "samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--fp64-steps", type=int, default=2, help="samples timed on the plain FP64 path (0 skips it)")
    ap.add_argument("--L", type=int, default=16, help="cells per axis (16 is the benchmark; smaller for profiling)")
    ap.add_argument("--nrep", type=int, default=8, help="replicas sampled per batched add_sample")
    ap.add_argument("--nomega", type=int, default=200, help="energy bins (200 is the benchmark; fewer for profiling)")
    ap.add_argument("--no-extra", action="store_true", help="skip the tempering and Langevin site-step arms")
    ap.add_argument("--no-error", action="store_true", help="skip the stated-error measurement (FP32 vs FP64)")
    ap.add_argument("--error-samples", type=int, default=32, help="samples per path of the stated-error measurement")
    ap.add_argument("--tol", type=float, default=1e-6, help="FP32 batched midpoint tolerance (per-site RMS)")
    ap.add_argument("--first-accept", action="store_true",
                    help="batched midpoint: convergence test from the extrapolated first iterate on")
    ap.add_argument("--mid-shape", type=int, default=None,
                    help="batched midpoint launch shape (row of the autotuner's table) after the first warm-up sample")
    ap.add_argument("--predictor", type=int, default=None,
                    help="first-iterate extrapolation order of the batched midpoint (library default if omitted)")
    args = ap.parse_args()
    global L, NOMEGA
    L = args.L
    NOMEGA = args.nomega
    if args.warmup < 3:
        args.warmup = 3
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as tdist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        tdist.init_process_group("gloo")
        dist = tdist
    if args.impl == "reference":
        reference_arm(args, rank, world)
        if dist:
            dist.barrier()
        return
    import __graft_entry__ as ge
    sg = ge.package()

    def barrier():
        if dist:
            dist.barrier()

    def maxall(x):
        if not dist:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    barrier()
    rb = run_batched(sg, local, args.nrep, args.warmup, args.steps, tol=args.tol, predictor=args.predictor,
                     mid_shape=args.mid_shape, first_accept=args.first_accept)
    barrier()
    r32 = run_arm(sg, "fp32", local, args.warmup, max(2, args.steps // 2), tol=1e-6)
    # (single-system FP32 path: one replica per add_sample)
    barrier()
    r64 = run_arm(sg, "fp64", local, 1, args.fp64_steps, tol=1e-12) if args.fp64_steps > 0 else None
    extra = {}
    pt = None
    if not args.no_extra:
        for kind, n in (("sc", 10000), ("tri", 2000)):
            a = dynamics_rate(sg, kind, "fp32", local, n)
            bb = dynamics_rate(sg, kind, "fp64", local, n // 4)
            extra[kind] = {"fp32": a, "fp64": bb, "speedup": a["site_steps_per_s"] / bb["site_steps_per_s"]}
            if kind == "sc":
                bt = batched_langevin_rate(sg, local)
                extra[kind]["fp32_batch64"] = bt
                extra[kind]["speedup_batch64_vs_fp64"] = bt["site_steps_per_s"] / bb["site_steps_per_s"]
        extra["local_sampler_sc"] = {p: local_sampler_rate(sg, p, local) for p in ("fp32", "fp64")}
        pt = run_tempering(sg, local)
        extra["adjoint"] = run_adjoint(sg, local)
        c3 = {"fp32": run_c3_sqw(sg, local, "fp32", 2), "fp64": run_c3_sqw(sg, local, "fp64", 1)}
        c3["speedup"] = c3["fp32"]["samples_per_s"] / c3["fp64"]["samples_per_s"]
        c3["fp32_group8"] = run_c3_group(sg, local)
        c3["speedup_group8_vs_fp64"] = c3["fp32_group8"]["samples_per_s"] / c3["fp64"]["samples_per_s"]
        extra["c3_sqw"] = c3
    err = None
    if not args.no_error:
        err = stated_error(sg, local, L_=L, nomega=NOMEGA, nrep=args.nrep, nsamples=args.error_samples, tol32=args.tol,
                           first_accept=args.first_accept, predictor=args.predictor)
    barrier()
    ms = maxall(rb["ms"])
    value = world * args.steps * rb["nrep"] / (ms / 1000.0)
    nsteps_sample = rb["nsteps_per_sample"]
    site_steps = value * rb["ns"] * nsteps_sample
    v32 = world * max(2, args.steps // 2) / (maxall(r32["ms"]) / 1000.0)
    v64 = world * args.fp64_steps / (maxall(r64["ms"]) / 1000.0) if r64 else None
    e2e_s = maxall(rb["e2e_s"])
    e2e_val = world * rb["e2e_steps"] * rb["nrep"] / e2e_s
    # roofline of the dominant phase, from the live per-phase CUDA events
    hbm, peak_kind = peaks()
    ph = rb["phase_ms"]
    R = rb["nrep"]
    ncorr, npos, ncell, nw = 6, 16, L**3, rb["n_all_omega"]
    bytes_accum = 2 * 16 * ncorr * npos * npos * ncell * nw + R * 8 * 3 * npos * ncell * nw
    bytes_traj = R * 24 * rb["ns"] * nsteps_sample
    kernels = [
        {"kernel": f"k_batch_midpoint ({R} replicas: trajectories + snapshots)", "ms_per_launch": ph[0],
         "alg_bytes": bytes_traj, "achieved_gbs": bytes_traj / (ph[0] * 1e6) if ph[0] else None},
        {"kernel": f"cuFFT space (3-D, {R} x 200 x 48 transforms)", "ms_per_launch": ph[1]},
        {"kernel": f"cuFFT time (1-D n=398, {R} x 196,608 transforms)", "ms_per_launch": ph[2]},
        {"kernel": f"k_corr_accum_bulk (rank-{R} FP64 accumulator stream, bulk-copy rows)", "ms_per_launch": ph[3], "alg_bytes": bytes_accum,
         "achieved_gbs": bytes_accum / (ph[3] * 1e6) if ph[3] else None},
    ]
    dom = max((k for k in kernels if "alg_bytes" in k), key=lambda k: k["ms_per_launch"])
    traffic = DRAM_BYTES_PER_LAUNCH.get(dom["kernel"].split()[0]) if (L, NOMEGA, R) == (16, 200, 8) else None
    roof = {"bound": "hbm", "kernel": dom["kernel"], "achieved": dom["achieved_gbs"], "peak": hbm, "unit": "GB/s",
            "frac": dom["achieved_gbs"] / hbm, "traffic": traffic, "peak_source": f"{peak_kind} hbm_gbs"}
    # the midpoint kernel's actual bound is L2 (state L2-resident): its L2 bytes per
    # site-iteration (ncu) times the iterations of this run over the trajectory time
    shapes = rb["midpoint_shapes"]["shapes"]
    ch = rb["midpoint_shapes"]["chosen"]
    idx = shapes[ch].get("nbr_index_bytes_smem") if 0 <= ch < len(shapes) else None
    if idx in L2_BYTES_PER_SITE_ITER and ph[0]:
        l2_bytes = L2_BYTES_PER_SITE_ITER[idx] * rb["ns"] * R * rb["iters_per_step"] * nsteps_sample
        l2_gbs = l2_bytes / (ph[0] * 1e6)
        roof["l2"] = {"achieved": l2_gbs, "peak": L2_PEAK_GBS_NCU, "unit": "GB/s", "frac": l2_gbs / L2_PEAK_GBS_NCU,
                      "bytes_per_site_iteration": L2_BYTES_PER_SITE_ITER[idx],
                      "source": "L2 sectors per site-iteration and the L2 peak from one ncu capture of this shape "
                                "(L = 16, 8 replicas, nomega = 20)"}
    line = {"metric": METRIC, "value": value, "unit": "samples/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "pyrochlore 16x16x16x16 (65,536 spins, s=3/2, J1=1, J2=0.05) S(q,w) sampling: "
                                   "ImplicitMidpoint dt=0.024933, 21 steps per snapshot, 200 snapshots, nw=200 to 6 meV, "
                                   "6 correlation pairs x 16 x 16 sublattices, FP64 accumulator; "
                                   f"{R} replicas per batched add_sample ({R * args.steps} samples timed)",
                       "global_batch": world * R, "seq_len": nsteps_sample, "parallelism": f"replicas x{world * R}",
                       "l2": "inputs larger than L2 (40 GB accumulator streamed every step)",
                       "midpoint_tol": {"fp32": args.tol, "fp64": 1e-12}, "first_accept": args.first_accept},
            "site_steps_per_s": site_steps,
            "fp32_single": {"value": v32, "unit": "samples/s", "ms_per_step": r32["ms"] / max(2, args.steps // 2),
                            "phase_ms": r32["phase_ms"], "iters_per_step": r32["iters_per_step"]},
            "fp64_plain": None if r64 is None else
            {"value": v64, "unit": "samples/s", "site_steps_per_s": v64 * r32["ns"] * nsteps_sample,
             "ms_per_step": r64["ms"] / args.fp64_steps, "phase_ms": r64["phase_ms"]},
            "phase_ms": {"trajectory": ph[0], "space_fft": ph[1], "time_fft": ph[2], "accumulate": ph[3]},
            "midpoint_iters_per_step": {"fp32_batched": rb["iters_per_step"], "fp32": r32["iters_per_step"],
                                        "fp64": None if r64 is None else r64["iters_per_step"]},
            "us_per_midpoint_iteration": 1000.0 * ph[0] / (rb["iters_per_step"] * nsteps_sample),
            "midpoint_autotune": rb["midpoint_shapes"],
            "kernels": kernels,
            "langevin_site_steps": {"simple_cubic_16^3_dipole": extra.get("sc"), "triangular_48x48x4_SU3": extra.get("tri"),
                                    "tempering_256_replicas": pt},
            "adjoint_c5": extra.get("adjoint"),
            "sqw_su3_triangular_48x48x4": extra.get("c3_sqw"),
            "local_sampler_simple_cubic_16^3": extra.get("local_sampler_sc"),
            "error_detail": err,
            "roofline": roof,
            "gpu_launches": rb["launches"],
            "clocks": rb["clocks"],
            "e2e": {"value": e2e_val, "unit": "samples/s", "h2d_bytes_per_step": rb["h2d"],
                    "d2h_bytes_per_step": rb["d2h"]},
            "speedup_vs_fp64_plain": None if r64 is None else value / v64,
            "error": None if err is None else
            {"energy_rel_err_per_sample_max": err["energy_rel_err_per_sample_max"],
             "fp64_energy_rel_err_per_sample_max": err["fp64_energy_rel_err_per_sample_max"],
             "energy_rel_err_per_step": err["energy_rel_err_per_step"],
             "sqw_chi2_ratio_vs_fp64": [h["chi2_ratio"] for h in err["sqw_vs_fp64_halves"]],
             "sqw_rel_rms_diff_vs_fp64": [h["rel_rms_diff"] for h in err["sqw_vs_fp64_halves"]],
             "sqw_systematic_rel_rms": err["sqw_systematic_rel_rms"],
             "sqw_systematic_rel_rms_upper": err["sqw_systematic_rel_rms_upper"],
             "limits": err["limits"]}}
    if L != 16 or NOMEGA != 200:
        line["config"]["workload"] = (f"REDUCED SIZE L={L}, nw={NOMEGA} (profiling case, not the benchmark): "
                                      + line["config"]["workload"])
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, cores, t_step = cpu_baseline(1, 20, 12)
        line["cpu_baseline"] = {"value": v, "unit": "samples/s", "cores": cores, "kind": "port",
                                "sample": "20 FP64 implicit-midpoint steps of the 65,536-spin pyrochlore and 12 of "
                                          "the 1,536 (c,i,j) correlation blocks plus the sample FFTs on one core, "
                                          "extrapolated to one full add_sample",
                                "midpoint_step_s": t_step}
    for k in ("speedup_vs_fp64_plain", "error"):      # the summary keys last, where a tail shows them
        line[k] = line.pop(k)
    barrier()
    if rank == 0:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
