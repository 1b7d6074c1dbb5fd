"""TEST INFRASTRUCTURE ONLY -- the FP64 CPU oracle for parity checks.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm use this
module. It binds the C restatement in sunny_oracle.c (dynamics, gradients, energy) and
restates Sunny's SampledCorrelations accumulation (CorrelationSampling.jl:21-139) and
replica exchange (ParallelTempering.jl:40-95) in numpy, in the reference's own order:
per-sample windowed correlations folded into a running mean.

Parity pins: the known answers of the reference's own tests that do not depend on
Julia's random stream (see tests/golden/make_golden.py).
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libsunny_oracle.so"

MODE_DIPOLE, MODE_DIPOLE_UNCORRECTED, MODE_SUN = 0, 1, 2


class BondC(C.Structure):
    _fields_ = [("i", C.c_int32), ("j", C.c_int32), ("n", C.c_int32 * 3), ("scalar", C.c_double),
                ("bilin", C.c_double * 9), ("biquad_kind", C.c_int32), ("biquad", C.c_double * 25)]


class SiteBondC(C.Structure):
    _fields_ = [("cell", C.c_int32 * 3), ("pad", C.c_int32), ("bond", BondC)]


class OrSys(C.Structure):
    _fields_ = [("L", C.c_int * 3), ("na", C.c_int), ("N", C.c_int), ("mode", C.c_int),
                ("kappa", C.POINTER(C.c_double)), ("g", C.POINTER(C.c_double)), ("field", C.POINTER(C.c_double)),
                ("onsite", C.POINTER(C.c_double)), ("bonds", C.POINTER(BondC)), ("nbonds", C.c_int),
                ("onsite_site", C.POINTER(C.c_double)), ("site_bonds", C.POINTER(SiteBondC)),
                ("nsite_bonds", C.c_int64), ("gen_bond", C.POINTER(C.c_int)), ("gen_A", C.POINTER(C.c_double)),
                ("gen_B", C.POINTER(C.c_double)), ("ngen", C.c_int), ("ewA", C.POINTER(C.c_double))]


_D = C.POINTER(C.c_double)
_lib = None


def build() -> Path:
    r = subprocess.run(["make", "-s"], cwd=HERE, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        lib = C.CDLL(str(LIB))
        P = C.POINTER(OrSys)
        sig = {
            "or_grad_dipoles": (None, [P, _D, _D]),
            "or_grad_coherents": (None, [P, _D, _D]),
            "or_energy": (C.c_double, [P, _D, _D]),
            "or_langevin_steps": (None, [P, _D, _D, C.c_double, C.c_double, C.c_double, C.c_int, _D]),
            "or_midpoint_steps": (C.c_int, [P, _D, _D, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int,
                                            C.POINTER(C.c_int64)]),
            "or_observables": (None, [P, _D, _D, C.c_int, _D, _D]),
            "or_langevin_replicas": (C.c_int, [P, C.c_int, _D, _D, C.c_double, C.c_double, C.c_int, C.c_uint64]),
            "or_expected_spin": (None, [C.c_int, _D, _D]),
            "or_local_energy_change": (C.c_double, [P, _D, C.c_int64, _D]),
            "or_local_energy_change_sun": (C.c_double, [P, _D, _D, C.c_int64, _D]),
            "or_local_sweeps_sun": (None, [P, _D, _D, C.c_double, C.c_int, C.c_double, C.POINTER(C.c_int), C.c_int,
                                           C.POINTER(C.c_int), _D, _D, _D, _D, _D]),
            "or_ewald_matrices": (None, [C.c_int, C.c_int, C.c_int, C.c_int, _D, _D, _D, C.c_double, _D]),
            "or_local_sweeps": (None, [P, _D, C.c_double, C.c_int, C.c_double, C.POINTER(C.c_int), C.c_int,
                                       C.POINTER(C.c_int), _D, _D, _D, _D, _D]),
        }
        for k, (res, args) in sig.items():
            f = getattr(lib, k)
            f.restype, f.argtypes = res, args
        _lib = lib
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(_D)


class OracleSystem:
    """FP64 CPU model built from the same host tables the GPU library receives."""

    def __init__(self, dims, natoms, N, mode, kappa, g_colmajor, field, onsite, bonds, onsite_site=None,
                 site_bonds=None, general=None):
        """onsite_site / site_bonds: the per-site onsite couplings and the non-culled per-site
        pair couplings (SiteBondC) of an inhomogeneous system, else None. general: SU(N)
        general pair couplings as (bond indices, A, B) with A, B [nterms][N][N] complex."""
        self.lib = load()
        self.dims, self.na, self.N, self.mode = tuple(dims), natoms, N, mode
        self.ns = int(np.prod(dims)) * natoms
        self._keep = [np.ascontiguousarray(kappa, dtype=float), np.ascontiguousarray(g_colmajor, dtype=float),
                      None if field is None else np.ascontiguousarray(field, dtype=float),
                      None if onsite is None else np.ascontiguousarray(onsite, dtype=float)]
        arr = (BondC * max(1, len(bonds)))()
        for k, b in enumerate(bonds):
            C.memmove(C.byref(arr[k]), C.byref(b), C.sizeof(BondC))
        self._bonds = arr
        s = OrSys()
        s.L[:] = dims
        s.na, s.N, s.mode = natoms, N, mode
        s.kappa, s.g = _p(self._keep[0]), _p(self._keep[1])
        s.field = _p(self._keep[2])
        s.onsite = _p(self._keep[3])
        s.bonds = arr
        s.nbonds = len(bonds)
        if onsite_site is not None:
            self._onsite_site = np.ascontiguousarray(onsite_site, dtype=float).reshape(-1)
            s.onsite_site = _p(self._onsite_site)
        if site_bonds is not None:
            sb = (SiteBondC * max(1, len(site_bonds)))()
            for k, b in enumerate(site_bonds):
                C.memmove(C.byref(sb[k]), C.byref(b), C.sizeof(SiteBondC))
            self._site_bonds = sb
            s.site_bonds = sb
            s.nsite_bonds = len(site_bonds)
        if general is not None and len(general[0]):
            gb, A, B = general
            self._gen = (np.ascontiguousarray(gb, dtype=np.int32),
                         np.ascontiguousarray(np.stack([np.swapaxes(A, -1, -2).real, np.swapaxes(A, -1, -2).imag], -1)).reshape(-1),
                         np.ascontiguousarray(np.stack([np.swapaxes(B, -1, -2).real, np.swapaxes(B, -1, -2).imag], -1)).reshape(-1))
            s.gen_bond = self._gen[0].ctypes.data_as(C.POINTER(C.c_int))
            s.gen_A = _p(self._gen[1])
            s.gen_B = _p(self._gen[2])
            s.ngen = len(gb)
        self.s = s

    def set_ewald(self, A):
        """Include the dipole-dipole term in local energy changes: A[cell, i, j] (3x3) from
        ewald_matrices (or None to drop it)."""
        if A is None:
            self.s.ewA = None
            return
        self._ewA = np.ascontiguousarray(np.asarray(A, dtype=float).transpose(0, 1, 2, 4, 3)).reshape(-1)
        self.s.ewA = _p(self._ewA)

    @classmethod
    def from_system(cls, sys):
        """Copy the couplings of a sunny_gb300 System (its host tables)."""
        na = sys.natoms
        if sys.N:
            on = []
            for a in range(na):
                M = sys._onsite[a] if sys._onsite[a] is not None else np.zeros((sys.N, sys.N), complex)
                on.append(np.stack([M.T.real, M.T.imag], -1).reshape(-1))
            onsite = np.concatenate(on)
        else:
            onsite = np.concatenate([sys._onsite[a] if sys._onsite[a] is not None else np.zeros(28) for a in range(na)])
        gcm = np.ascontiguousarray(sys._g.transpose(0, 2, 1)).reshape(-1)
        field = sys._field.reshape(-1) if np.any(sys._field) else None
        mode = {"dipole": MODE_DIPOLE, "dipole_uncorrected": MODE_DIPOLE_UNCORRECTED, "SUN": MODE_SUN}[sys.mode]
        if sys.is_homogeneous():
            return cls(sys.dims, na, sys.N, mode, sys._kappa, gcm, field, onsite, sys.bond_table(),
                       general=sys.general_table())
        return cls(sys.dims, na, sys.N, mode, sys._kappa, gcm, field, onsite, [], onsite_site=sys.onsite_site_table(),
                   site_bonds=[SiteBondC.from_buffer_copy(bytes(b)) for b in sys.site_bond_table()])

    # ---- state helpers: S (ns, 3) float; Z (ns, N) complex --------------------------------
    def _zbuf(self, Z):
        return None if Z is None else np.ascontiguousarray(np.stack([Z.real, Z.imag], -1)).reshape(-1)

    def expected_spin(self, Z):
        zb = self._zbuf(Z)
        out = np.zeros((self.ns, 3))
        for i in range(self.ns):
            self.lib.or_expected_spin(self.N, zb[2 * self.N * i:].ctypes.data_as(_D), out[i].ctypes.data_as(_D))
        return out

    def grad(self, S=None, Z=None):
        if self.N:
            zb = self._zbuf(Z)
            out = np.zeros(2 * self.N * self.ns)
            self.lib.or_grad_coherents(C.byref(self.s), _p(zb), _p(out))
            o = out.reshape(self.ns, self.N, 2)
            return o[..., 0] + 1j * o[..., 1]
        S = np.ascontiguousarray(S, dtype=float)
        out = np.zeros((self.ns, 3))
        self.lib.or_grad_dipoles(C.byref(self.s), _p(S), _p(out))
        return out

    def local_energy_change(self, S, site, S_new, Z=None):
        """local_energy_change (Interactions.jl:311-373). SU(N) mode: Z (ns, N) complex kets,
        S their expected dipoles, S_new the new ket (N,) complex."""
        S = np.ascontiguousarray(S, dtype=float)
        if self.N:
            zn = np.ascontiguousarray(np.stack([np.real(S_new), np.imag(S_new)], -1), dtype=float).reshape(-1)
            return self.lib.or_local_energy_change_sun(C.byref(self.s), _p(S), _p(self._zbuf(Z)), int(site), _p(zn))
        Sn = np.ascontiguousarray(S_new, dtype=float)
        return self.lib.or_local_energy_change(C.byref(self.s), _p(S), int(site), _p(Sn))

    def local_sweeps(self, S, kT, nsweeps, frac, order, proposal, rand):
        """LocalSampler updates in the site order `order` (each sweep), with caller randoms
        rand [nsweeps][ns][6]; proposal: list of (kind, weight, magnitude). Returns
        (S, dE, dS)."""
        S = np.ascontiguousarray(S, dtype=float).copy()
        perm = np.ascontiguousarray(order, dtype=np.int32)
        w = np.array([p[1] for p in proposal], dtype=float)
        cum = np.cumsum(w / w.sum())
        kind = np.array([p[0] for p in proposal], dtype=np.int32)
        mag = np.array([p[2] for p in proposal], dtype=float)
        rnd = np.ascontiguousarray(rand, dtype=float).reshape(-1)
        dE = C.c_double()
        dS = np.zeros(3)
        IP = C.POINTER(C.c_int)
        self.lib.or_local_sweeps(C.byref(self.s), _p(S), float(kT), int(nsweeps), float(frac), perm.ctypes.data_as(IP),
                                 len(proposal), kind.ctypes.data_as(IP), _p(cum), _p(mag), _p(rnd), C.byref(dE), _p(dS))
        return S, dE.value, dS

    def local_sweeps_sun(self, S, Z, kT, nsweeps, frac, order, proposal, rand):
        """SU(N) LocalSampler updates (see local_sweeps); rand [nsweeps][ns][2N+3].
        Returns (S, Z, dE, dS)."""
        S = np.ascontiguousarray(S, dtype=float).copy()
        zb = self._zbuf(Z).copy()
        perm = np.ascontiguousarray(order, dtype=np.int32)
        w = np.array([p[1] for p in proposal], dtype=float)
        cum = np.cumsum(w / w.sum())
        kind = np.array([p[0] for p in proposal], dtype=np.int32)
        mag = np.array([p[2] for p in proposal], dtype=float)
        rnd = np.ascontiguousarray(rand, dtype=float).reshape(-1)
        dE = C.c_double()
        dS = np.zeros(3)
        IP = C.POINTER(C.c_int)
        self.lib.or_local_sweeps_sun(C.byref(self.s), _p(S), _p(zb), float(kT), int(nsweeps), float(frac),
                                     perm.ctypes.data_as(IP), len(proposal), kind.ctypes.data_as(IP), _p(cum), _p(mag),
                                     _p(rnd), C.byref(dE), _p(dS))
        return S, self._unz(zb), dE.value, dS

    def energy(self, S, Z=None):
        S = np.ascontiguousarray(S, dtype=float)
        return self.lib.or_energy(C.byref(self.s), _p(S), _p(self._zbuf(Z)))

    def langevin(self, S, Z, dt, damping, kT, nsteps, noise=None):
        """Returns updated (S, Z). noise: standard normals, (nsteps, ns, 3) or complex (nsteps, ns, N)."""
        S = np.ascontiguousarray(S, dtype=float).copy()
        zb = self._zbuf(Z)
        nz = None
        if noise is not None:
            noise = np.asarray(noise)
            if self.N:
                noise = np.stack([noise.real, noise.imag], -1)
            nz = np.ascontiguousarray(noise, dtype=float).reshape(-1)
        self.lib.or_langevin_steps(C.byref(self.s), _p(S), _p(zb), dt, damping, kT, nsteps, _p(nz))
        return S, self._unz(zb)

    def midpoint(self, S, Z, dt, damping, tol, max_iters, nsteps):
        S = np.ascontiguousarray(S, dtype=float).copy()
        zb = self._zbuf(Z)
        it = C.c_int64(0)
        st = self.lib.or_midpoint_steps(C.byref(self.s), _p(S), _p(zb), dt, damping, tol, max_iters, nsteps, C.byref(it))
        return st, S, self._unz(zb), it.value

    def observables(self, S, Z, obs_flat, nobs):
        out = np.zeros(nobs * self.ns)
        self.lib.or_observables(C.byref(self.s), _p(np.ascontiguousarray(S, dtype=float)), _p(self._zbuf(Z)), nobs,
                                _p(np.ascontiguousarray(obs_flat, dtype=float)), _p(out))
        return out.reshape(nobs, self.ns)

    def _unz(self, zb):
        if zb is None:
            return None
        z = zb.reshape(self.ns, self.N, 2)
        return z[..., 0] + 1j * z[..., 1]


# ---- SampledCorrelations (CorrelationSampling.jl:21-139) -----------------------------------

class OracleCorrelations:
    """Per-sample accumulation in the reference's order (running mean of windowed
    correlations). Layout of `data`: [c, i, j, q1, q2, q3, ω] like Sunny."""

    def __init__(self, osys: OracleSystem, obs_flat, nobs, corr_pairs, n_all_omega, measperiod, dt, tol,
                 damping=0.0, max_iters=100, calculate_errors=False):
        self.o = osys
        self.obs_flat = obs_flat
        self.nobs = nobs
        self.pairs = [(a - 1, b - 1) for a, b in corr_pairs]
        self.n = n_all_omega
        self.measperiod = measperiod
        self.dt, self.tol, self.damping, self.max_iters = dt, tol, damping, max_iters
        L1, L2, L3 = osys.dims
        self.data = np.zeros((len(self.pairs), osys.na, osys.na, L1, L2, L3, n_all_omega), dtype=complex)
        self.M = np.zeros(self.data.shape) if calculate_errors else None
        self.nsamples = 0

    def trajectory(self, S, Z):
        """new_sample!/trajectory! (CorrelationSampling.jl:21-46): returns the sample buffer
        [nobs, L1, L2, L3, npos, n] (zero-padded) and the final state."""
        L1, L2, L3 = self.o.dims
        na, ns = self.o.na, self.o.ns
        nsnaps = self.n // 2 + 1
        buf = np.zeros((self.nobs, L1, L2, L3, na, self.n), dtype=complex)

        def record(t, S, Z):
            v = self.o.observables(S, Z, self.obs_flat, self.nobs)   # (nobs, ns) in site order
            buf[..., t] = v.reshape(self.nobs, na, L3, L2, L1).transpose(0, 4, 3, 2, 1)

        record(0, S, Z)
        for t in range(1, nsnaps):
            st, S, Z, _ = self.o.midpoint(S, Z, self.dt, self.damping, self.tol, self.max_iters, self.measperiod)
            if st != 0:
                raise RuntimeError("oracle midpoint did not converge")
            record(t, S, Z)
        return buf, S, Z

    def accum(self, buf, window="cosine"):
        """accum_sample! (CorrelationSampling.jl:48-139)."""
        n = self.n
        L1, L2, L3 = self.o.dims
        ncell = L1 * L2 * L3
        T = n // 2 + 1
        # A(q) = sum_r exp(iqr) A(r) / sqrt(Ncell): conj -> FFT -> conj
        A = np.conj(np.fft.fftn(np.conj(buf), axes=(1, 2, 3))) / np.sqrt(ncell)
        A = np.fft.fft(A, axis=5)
        offs = np.fft.fftfreq(n, 1.0 / n)
        ncontrib = (T - np.abs(offs)).astype(float)
        ncontrib[ncontrib == 0] = np.inf
        self.nsamples += 1
        count = self.nsamples
        win = np.cos(np.linspace(0, np.pi, n + 1)[:-1]) ** 2
        for j in range(self.o.na):
            for i in range(self.o.na):
                for c, (a, b) in enumerate(self.pairs):
                    corr = np.conj(A[a, :, :, :, i, :]) * A[b, :, :, :, j, :]
                    corr = np.fft.ifft(corr, axis=3) / ncontrib
                    if window == "cosine":
                        corr = corr * win
                    corr = np.fft.fft(corr, axis=3)
                    d = self.data[c, i, j]
                    if self.M is None:
                        d += (corr - d) * (1.0 / count)
                    else:
                        # Welford update (CorrelationSampling.jl:117-134)
                        mu_old = d.copy()
                        d += (corr - d) / count
                        self.M[c, i, j] += np.real((corr - mu_old) * np.conj(corr - d))

    def add_sample(self, S, Z, window="cosine"):
        buf, S, Z = self.trajectory(S, Z)
        self.accum(buf, window)
        return S, Z


def merge_with_errors(datas, Ms, counts):
    """merge_correlations with M (SampledCorrelations.jl:128-142)."""
    d, M, n = datas[0].copy(), Ms[0].copy(), counts[0]
    for d2, M2, m in zip(datas[1:], Ms[1:], counts[1:]):
        mu = (n / (n + m)) * d + (m / (n + m)) * d2
        M = (M + n * np.abs(mu - d) ** 2) + (M2 + m * np.abs(mu - d2) ** 2)
        d = mu
        n += m
    return d, M, n


def merge_means(datas, counts):
    """merge_correlations' weighted mean (SampledCorrelations.jl:128-142), data only."""
    mu = datas[0].copy()
    n = counts[0]
    for d, m in zip(datas[1:], counts[1:]):
        mu = (n / (n + m)) * mu + (m / (n + m)) * d
        n += m
    return mu, n


# ---- replica exchange (ParallelTempering.jl:40-73) -----------------------------------------

def replica_exchange(E, kT, system_ids, exch_start, uniforms):
    """One exchange sweep on the ladder; E[k] is the energy of system_ids[k] (0-based
    ladder positions). exch_start is 1-based as in the reference. Returns accepted flags."""
    nrep = len(kT)
    acc = np.zeros(nrep, dtype=bool)
    ids = list(system_ids)
    for rank in range(exch_start - 1, nrep - 1, 2):
        i1, i2 = rank, rank + 1
        E1, E2 = E[ids[i1]], E[ids[i2]]
        dS1 = E1 / kT[i1] - E2 / kT[i1]
        dS2 = E2 / kT[i2] - E1 / kT[i2]
        lnP = dS1 + dS2
        if lnP >= 0 or uniforms[i1] < np.exp(lnP):
            ids[i1], ids[i2] = ids[i2], ids[i1]
            acc[i1] = True
    return ids, acc


# ---- dipole-dipole (Ewald.jl) in pairwise form ------------------------------------------

def ewald_matrices(dims, latvecs, positions, demag, mu0_muB2):
    """A[cell, i, j] (3x3, [row, col]) of precompute_dipole_ewald (Ewald.jl:40-146), from the
    C restatement; cell = c1 + L1*(c2 + L2*c3) is the offset of atom j's cell."""
    lib = load()
    L1, L2, L3 = dims
    na = len(positions)
    out = np.zeros(L1 * L2 * L3 * na * na * 9)
    lat = np.ascontiguousarray(np.asarray(latvecs, dtype=float).T.reshape(-1))
    pos = np.ascontiguousarray(np.asarray(positions, dtype=float).reshape(-1))
    dm = np.ascontiguousarray(np.asarray(demag, dtype=float).T.reshape(-1))
    lib.or_ewald_matrices(L1, L2, L3, na, _p(lat), _p(pos), _p(dm), float(mu0_muB2), _p(out))
    return out.reshape(L1 * L2 * L3, na, na, 3, 3).transpose(0, 1, 2, 4, 3)


def ewald_pairwise_grad(A, dims, na, S, g):
    """dE/dS of the dipole-dipole energy as a sum over pairs (Ewald.jl:210-228):
    ∇E_1 = Σ_2 g_1ᵀ A[cell_2 - cell_1, i_1, i_2] g_2 S_2. S: [ns][3]; g: [ns][3][3]."""
    L1, L2, L3 = dims
    ncell = L1 * L2 * L3
    ns = ncell * na
    cells = np.arange(ns) % ncell
    atoms = np.arange(ns) // ncell
    c = np.stack([cells % L1, (cells // L1) % L2, cells // (L1 * L2)], 1)
    mu = np.einsum("sab,sb->sa", g, S)
    grad = np.zeros((ns, 3))
    for s1 in range(ns):
        off = (c - c[s1]) % np.array(dims)
        oi = off[:, 0] + L1 * (off[:, 1] + L2 * off[:, 2])
        phi = np.einsum("sab,sb->a", A[oi, atoms[s1], atoms], mu)
        grad[s1] = g[s1].T @ phi
    return grad


# ---- S(q,w) loss of one sample, for finite-difference reference gradients -----------------

def sqw_loss(osys: OracleSystem, obs_flat, nobs, corr_pairs, n_all_omega, measperiod, dt, tol, S0, target):
    """mean over all complex bins of |data - target|^2, data = one add_sample! from S0
    (CorrelationSampling.jl:1-139, cosine window), in FP64. Returns (loss, data)."""
    oc = OracleCorrelations(osys, obs_flat, nobs, corr_pairs, n_all_omega, measperiod, dt, tol)
    oc.add_sample(np.asarray(S0, dtype=float), None)
    d = oc.data
    return float(np.mean(np.abs(d - target) ** 2)), d


# ---- intensities (DataRetrieval.jl:1-181, PhaseAveraging.jl) -------------------------------

def intensities(data, recipvecs, positions, dims, qs, widx, combiner, n_all_omega, dw, kT=None, ws=None,
                formfactors=None):
    """intensities_aux! and the density / classical-to-quantum post-processing, on the raw
    data [c, i, j, q1, q2, q3, w]. qs in RLU; widx are energy indices; combiner(q_abs,
    elems) is the MeasureSpec combiner. Returns [w, q]."""
    Ls = np.asarray(dims)
    npos = data.shape[1]
    out = np.zeros((len(widx), len(qs)))
    for k, q in enumerate(qs):
        m = np.rint(np.asarray(q) * Ls).astype(int)
        i1, i2, i3 = np.mod(m, Ls)
        qabs = recipvecs @ (m / Ls)
        ff = np.ones(npos) if formfactors is None else np.array([f(qabs @ qabs) for f in formfactors])
        pref = ff * np.exp(-2j * np.pi * ((m / Ls) @ np.asarray(positions).T))
        for t, w in enumerate(widx):
            elems = np.zeros(data.shape[0], dtype=complex)
            for j in range(npos):
                for i in range(npos):
                    elems += (pref[i] * np.conj(pref[j])) * data[:, i, j, i1, i2, i3, w]
            out[t, k] = combiner(qabs, elems)
    if dw is not None and not np.isnan(dw):
        out /= n_all_omega * dw
        if kT is not None:
            c2q = np.array([1.0 if w == 0 else abs((w / kT) / (1 - np.exp(-w / kT))) for w in ws])
            out *= c2q[:, None]
    return out
