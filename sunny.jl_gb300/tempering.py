"""Replica batches and parallel tempering on the GPU.

`ReplicaBatch` holds many independent dipole-mode replicas that share the couplings of a
prototype `System` but may differ in supercell size and temperature; they advance
together in one persistent launch. `ParallelTempering` mirrors Sunny's
(src/MonteCarlo/ParallelTempering.jl:2-95): replica exchange over a kT ladder, here one
ladder per group of equal-size replicas, with step_ensemble! replayed from a captured
CUDA graph.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _abi
from .system import System, LocalSampler, clone_system, energy, magnetization, step


class ReplicaBatch:
    """Replicas of a prototype System advanced together.

    Dipole-mode prototypes with per-sublattice couplings become one batch of concatenated
    states (replicas may differ in dims) driven by persistent batch kernels. Any other
    prototype (SU(N) mode, dipole-dipole interactions, inhomogeneous or general
    couplings) becomes a replica group: `nrep` device clones of the prototype
    (clone_system, as ParallelTempering.jl:20-37 makes them) whose persistent launches run
    concurrently, each on its own stream with an equal share of the SMs; replicas then
    have the prototype's dims, and `members[r]` is replica r's System."""

    def __init__(self, proto: System, dims_list, kT=None, precision: str | None = None, device: int = 0, seed: int = 0):
        self.proto = proto
        self.dims_list = [tuple(int(x) for x in d) for d in dims_list]
        self.nrep = len(self.dims_list)
        self.natoms = proto.natoms
        self.N = proto.N
        self.precision = precision or proto.precision
        self.seed = int(seed)
        self.noise_step = 0
        self._lib = _abi.load()
        self.members = None
        if proto.N or getattr(proto, "_ewald", None) is not None or proto._site_pairs is not None or proto._general:
            self._init_group(device, kT)
            return
        d = _abi.Desc()
        d.dims[:] = self.dims_list[0]
        d.natoms, d.N = proto.natoms, 0
        d.mode = {"dipole": _abi.MODE_DIPOLE, "dipole_uncorrected": _abi.MODE_DIPOLE_UNCORRECTED}[proto.mode]
        d.precision = _abi.FP32 if self.precision == "fp32" else _abi.FP64
        d.device = device
        dims = (C.c_int32 * (3 * self.nrep))(*[x for dd in self.dims_list for x in dd])
        h = C.c_void_p()
        self._check(self._lib.sgb_batch_create(C.byref(d), self.nrep, dims, C.byref(h)), None)
        self._h = h
        self._upload_couplings()
        self.rng = np.random.default_rng(seed)
        self.kT = np.zeros(self.nrep) if kT is None else np.asarray(kT, dtype=float)
        self.set_kT(self.kT)

    def _init_group(self, device, kT):
        if any(d != self.proto.dims for d in self.dims_list):
            raise ValueError("a replica group (SU(N) mode, dipole-dipole, inhomogeneous or general couplings) "
                             "needs replicas with the prototype's dims")
        self.members = [clone_system(self.proto, seed=self.seed + r, device=device, precision=self.precision)
                        for r in range(self.nrep)]
        for m in self.members:
            m._sync_to_device()
        hs = (C.c_void_p * self.nrep)(*[m.handle.value if isinstance(m.handle, C.c_void_p) else m.handle
                                        for m in self.members])
        h = C.c_void_p()
        self._check(self._lib.sgb_batch_create_group(hs, self.nrep, C.byref(h)), None)
        self._h = h
        self.rng = np.random.default_rng(self.seed)
        self.kT = np.zeros(self.nrep) if kT is None else np.asarray(kT, dtype=float)
        self.set_kT(self.kT)

    def _touch(self):
        """The members' device states changed: their host copies refresh on next read."""
        if self.members:
            for m in self.members:
                m._dev_newer = True

    def _sync_members(self):
        if self.members:
            for m in self.members:
                m._sync_to_device()

    def _check(self, rc, h="self"):
        if rc != _abi.SGB_OK:
            hh = self._h if h == "self" else h
            msg = self._lib.sgb_batch_last_error(hh)
            raise _abi.SunnyGPUError(rc, (msg or b"").decode() or f"error {rc}")

    def close(self):
        if getattr(self, "_h", None):
            self._lib.sgb_batch_destroy(self._h)
            self._h = None
        for m in getattr(self, "members", None) or []:
            m.close()
        self.members = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def nsites(self, r: int) -> int:
        return int(self._lib.sgb_batch_nsites(self._h, r))

    def _upload_couplings(self):
        p = self.proto
        na = p.natoms
        # couplings are per sublattice: take the first cell's values
        first = np.arange(na) * p.ncell
        kap = np.ascontiguousarray(p._kappa[first])
        g = np.ascontiguousarray(p._g[first].transpose(0, 2, 1)).reshape(-1)
        field = np.ascontiguousarray(p._field[first]).reshape(-1)
        onsite = np.concatenate([p._onsite[a] if p._onsite[a] is not None else np.zeros(28) for a in range(na)])
        bonds = p.bond_table()
        arr = (_abi.BondC * max(1, len(bonds)))()
        for k, b in enumerate(bonds):
            arr[k] = b
        self._check(self._lib.sgb_batch_set_couplings(self._h, _abi.dptr(kap), _abi.dptr(g), _abi.dptr(field),
                                                      _abi.dptr(np.ascontiguousarray(onsite)), arr, len(bonds)))
        self._kappa_a = kap

    def set_kT(self, kT):
        self.kT = np.ascontiguousarray(kT, dtype=float)
        self._check(self._lib.sgb_batch_set_kT(self._h, _abi.dptr(self.kT)))

    def get_kT(self) -> np.ndarray:
        out = np.zeros(self.nrep)
        self._check(self._lib.sgb_batch_get_kT(self._h, _abi.dptr(out)))
        return out

    def set_state(self, r: int, state: np.ndarray):
        """Replica r's dipoles (ns, 3), or in SU(N) mode its coherent states (ns, N)."""
        if self.members:
            m = self.members[r]
            if m.N:
                m.set_state_flat(coherents=state)
            else:
                m.set_state_flat(dipoles=state)
            m._sync_to_device()
            return
        self._check(self._lib.sgb_batch_set_state(self._h, r, _abi.dptr(np.ascontiguousarray(state, dtype=float).reshape(-1))))

    def get_state(self, r: int) -> np.ndarray:
        """Replica r's dipoles (ns, 3), or in SU(N) mode its coherent states (ns, N)."""
        if self.members:
            m = self.members[r]
            return m.coherents_flat() if m.N else m.dipoles_flat()
        out = np.zeros((self.nsites(r), 3))
        self._check(self._lib.sgb_batch_get_state(self._h, r, _abi.dptr(out)))
        return out

    def randomize_spins(self):
        """randomize_spins! on every replica (System.jl:513-517)."""
        if self.members:
            for m in self.members:
                m.randomize_spins()
                m._sync_to_device()
            return
        for r in range(self.nrep):
            ns = self.nsites(r)
            v = self.rng.standard_normal((ns, 3))
            kap = np.repeat(self._kappa_a, ns // self.natoms)
            self.set_state(r, kap[:, None] * v / np.linalg.norm(v, axis=1)[:, None])

    def langevin(self, dt: float, damping: float, nsteps: int):
        self._sync_members()
        self._check(self._lib.sgb_batch_langevin(self._h, dt, damping, self.seed, self.noise_step, nsteps))
        self._touch()
        self.noise_step += nsteps

    def noise(self, r: int, step: int) -> np.ndarray:
        if self.members and self.N:
            out = np.zeros((self.nsites(r), self.N, 2))
            self._check(self._lib.sgb_batch_langevin_noise(self._h, r, self.seed, step, _abi.dptr(out)))
            return out[..., 0] + 1j * out[..., 1]
        out = np.zeros((self.nsites(r), 3))
        self._check(self._lib.sgb_batch_langevin_noise(self._h, r, self.seed, step, _abi.dptr(out)))
        return out

    def set_wait_limit(self, seconds: float):
        """Wall-clock limit of the device-side waits of the batch's persistent kernels (0:
        the default, 4 s)."""
        self._check(self._lib.sgb_batch_set_wait_limit(self._h, float(seconds)))

    def set_midpoint_first_accept(self, on: bool):
        """Apply the midpoint convergence test from the first (extrapolated) iterate on."""
        self._check(self._lib.sgb_batch_set_midpoint_first_accept(self._h, 1 if on else 0))

    def set_midpoint_chunk(self, replicas: int):
        """Replicas per launch of batched add_sample! trajectories (0: as many as keep a
        launch's working set in L2); every replica's sample still goes into one pass."""
        self._check(self._lib.sgb_batch_set_midpoint_chunk(self._h, int(replicas)))

    def set_midpoint_predictor(self, order: int):
        """First iterate of each batched midpoint step: 0 S' = S (the reference's choice),
        k in 1..4 the degree-k extrapolation of the last k+1 states (fewer iterations, same
        convergence test). Default 4 for FP32, 0 for FP64."""
        self._check(self._lib.sgb_batch_set_midpoint_predictor(self._h, int(order)))

    def energies(self) -> np.ndarray:
        self._sync_members()
        out = np.zeros(self.nrep)
        self._check(self._lib.sgb_batch_energy(self._h, _abi.dptr(out)))
        return out


def exchange_round(E, kT, system_ids, exch_start, uniform):
    """The swap decisions of replica_exchange! (ParallelTempering.jl:40-73) on one ladder.
    E[k]: energy at ladder position k; exch_start is 1-based (1 or 2); uniform(k) draws
    the acceptance uniform of pair (k, k+1). Returns the new ids and, per position, whether
    an exchange was attempted and accepted."""
    n = len(kT)
    ids = list(system_ids)
    E = list(E)
    tried = np.zeros(n, dtype=bool)
    acc = np.zeros(n, dtype=bool)
    for k in range(exch_start - 1, n - 1, 2):
        E1, E2 = E[k], E[k + 1]
        lnP = (E1 / kT[k] - E2 / kT[k]) + (E2 / kT[k + 1] - E1 / kT[k + 1])
        tried[k] = True
        if lnP >= 0 or uniform(k) < math.exp(lnP):
            ids[k], ids[k + 1] = ids[k + 1], ids[k]
            E[k], E[k + 1] = E[k + 1], E[k]
            acc[k] = True
    return ids, tried, acc


class ParallelTempering:
    """ParallelTempering(system, Langevin, kT_sched) over replicas of (possibly) several
    sizes (ParallelTempering.jl:18-37). Each group of equal dims has its own ladder.

    ParallelTempering(system, sampler, kT_sched) with a `System` builds the reference's
    own form instead: clones of one system, one sampler per temperature
    (SystemParallelTempering)."""

    def __new__(cls, *args, **kw):
        if cls is ParallelTempering and args and isinstance(args[0], System):
            return super().__new__(SystemParallelTempering)
        return super().__new__(cls)

    def __init__(self, batch: ReplicaBatch, dt: float, damping: float):
        self.batch = batch
        self.dt, self.damping = float(dt), float(damping)
        self.n_accept = np.zeros(batch.nrep, dtype=np.int64)
        self.n_exch_rounds = 0

    def replica_exchange(self, exch_start: int, uniforms=None, round_index: int = 0):
        """replica_exchange!(PT, exch_start) (ParallelTempering.jl:40-73); `uniforms`
        (indexed by ladder position) replaces the device generator."""
        b = self.batch
        na = np.zeros(b.nrep, dtype=np.int64)
        u = None if uniforms is None else np.ascontiguousarray(uniforms, dtype=float)
        b._check(b._lib.sgb_batch_exchange(b._h, exch_start, b.seed, round_index, _abi.dptr(u),
                                           na.ctypes.data_as(C.POINTER(C.c_int64))))
        self.n_accept = na

    def step_ensemble(self, nsteps: int, exch_interval: int):
        """step_ensemble!(PT, nsteps, exch_interval) (ParallelTempering.jl:80-95)."""
        b = self.batch
        na = np.zeros(b.nrep, dtype=np.int64)
        b._check(b._lib.sgb_batch_step_ensemble(b._h, self.dt, self.damping, b.seed, nsteps, exch_interval,
                                                na.ctypes.data_as(C.POINTER(C.c_int64))))
        rounds = -(-nsteps // exch_interval)
        b.noise_step += rounds * exch_interval
        self.n_exch_rounds += rounds
        self.n_accept = na

    @property
    def graph_active(self) -> bool:
        return bool(self.batch._lib.sgb_batch_graph_active(self.batch._h))


class SystemParallelTempering(ParallelTempering):
    """ParallelTempering(system, sampler, kT_sched) (ParallelTempering.jl:2-95) over device
    clones of one System.

    - Each ladder position has its own copy of `sampler` at its temperature; with a
      LocalSampler its ΔE/ΔS start at the clone's energy and net dipole and are swapped
      with the systems, so exchanges need no energy evaluation (ParallelTempering.jl:28-34,
      45-46, 64-66); other samplers (Langevin) use energy(system).
    - Clone r uses seed system.seed + r for its device random streams (Sunny copies the
      RNG); the exchange uniforms come from a host generator seeded by system.seed.
    """

    def __init__(self, system: System, sampler, kT_sched):
        self.n_replicas = len(kT_sched)
        self.kT_sched = [float(k) for k in kT_sched]
        self.samplers = []
        for kT in self.kT_sched:
            smp = sampler.copy()
            smp.kT = kT
            self.samplers.append(smp)
        self.systems = [clone_system(system, seed=system.seed + r) for r in range(self.n_replicas)]
        self.system_ids = list(range(self.n_replicas))
        self.n_accept = np.zeros(self.n_replicas, dtype=np.int64)
        self.n_exch = np.zeros(self.n_replicas, dtype=np.int64)
        self.rng = np.random.default_rng(system.seed)
        self.local = isinstance(sampler, LocalSampler)
        if self.local:
            for rank in range(self.n_replicas):
                self.samplers[rank].ΔE = energy(self.systems[rank])
                self.samplers[rank].ΔS = magnetization(self.systems[rank])
                self.samplers[rank].nsweeps = 1.0

    def energies(self):
        """Energy at each ladder position, as the exchange sees it."""
        if self.local:
            return [s.ΔE for s in self.samplers]
        return [energy(self.systems[i]) for i in self.system_ids]

    def replica_exchange(self, exch_start: int):
        """replica_exchange!(PT, exch_start) (ParallelTempering.jl:40-73)."""
        ids, tried, acc = exchange_round(self.energies(), self.kT_sched, self.system_ids, exch_start,
                                         lambda k: self.rng.random())
        if self.local:
            for k in np.nonzero(acc)[0]:
                a, b = self.samplers[k], self.samplers[k + 1]
                a.ΔE, b.ΔE = b.ΔE, a.ΔE
                a.ΔS, b.ΔS = b.ΔS, a.ΔS
        self.system_ids = ids
        self.n_accept += acc
        self.n_exch += tried

    def step_ensemble(self, nsteps: int, exch_interval: int):
        """step_ensemble!(PT, nsteps, exch_interval) (ParallelTempering.jl:80-95)."""
        for i in range(1, -(-nsteps // exch_interval) + 1):
            for rank in range(self.n_replicas):
                step(self.systems[self.system_ids[rank]], self.samplers[rank], exch_interval)
            self.replica_exchange((i % 2) + 1)

    def close(self):
        for s in self.systems:
            s.close()
