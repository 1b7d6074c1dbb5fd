"""`System`, integrators and `step` -- a host-side mirror of Sunny.jl's API whose hot path
runs in libsunnygb300.so.

Names, argument meanings and error messages follow Sunny.jl v0.9.2
(src/System/System.jl, src/System/Interactions.jl, src/System/PairExchange.jl,
src/System/OnsiteCoupling.jl, src/Integrators.jl). Julia's `!` suffix is dropped:
`step!(sys, integrator)` is `step(sys, integrator)`. Atom indices are 1-based, as in Sunny.

The spin state lives on the GPU. `sys.dipoles` / `sys.coherents` return numpy views of a
host copy that is refreshed from the device on access; writes through those views are
uploaded before the next device call (the host copy is treated as modified whenever it
has been handed out).
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import _abi
from .crystal import Bond, Crystal
from .operators import (rcs_factors, spin_matrices_of_dim, stevens_expansion_for_dipole, expected_spin,
                        tensor_decomposition,
                        ket_from_dipole)

_MODES = {"dipole": _abi.MODE_DIPOLE, "dipole_uncorrected": _abi.MODE_DIPOLE_UNCORRECTED, "SUN": _abi.MODE_SUN}


@dataclass
class Moment:
    """Moment(s, g) (src/System/Moment.jl:13-23)."""
    s: float
    g: object = 2.0

    def gmat(self) -> np.ndarray:
        g = np.asarray(self.g, dtype=float)
        return g * np.eye(3) if g.ndim == 0 else g.reshape(3, 3)


class Langevin:
    """Langevin(dt; damping, kT) (src/Integrators.jl:56-74)."""

    def __init__(self, dt=math.nan, *, damping=None, kT):
        if damping is None:
            raise ValueError("`damping` parameter required")
        if damping == 0:
            raise ValueError("Use ImplicitMidpoint instead for energy-conserving dynamics")
        if dt <= 0:
            raise ValueError("Select positive dt")
        if kT < 0:
            raise ValueError("Select nonnegative kT")
        if damping <= 0:
            raise ValueError("Select positive damping")
        self.dt, self.damping, self.kT = float(dt), float(damping), float(kT)

    def copy(self):
        return Langevin(self.dt, damping=self.damping, kT=self.kT)


class ImplicitMidpoint:
    """ImplicitMidpoint(dt; damping=0, kT=0, tol=1e-12) (src/Integrators.jl:107-131)."""

    def __init__(self, dt=math.nan, *, damping=0.0, kT=0.0, tol=1e-12):
        if dt <= 0:
            raise ValueError("Select positive dt")
        if kT < 0:
            raise ValueError("Select nonnegative kT")
        if damping < 0:
            raise ValueError("Select nonnegative damping")
        if kT != 0:
            raise ValueError("ImplicitMidpoint with a Langevin thermostat is not currently supported.")
        self.dt, self.damping, self.kT, self.tol = float(dt), float(damping), float(kT), float(tol)

    def copy(self):
        return ImplicitMidpoint(self.dt, damping=self.damping, kT=self.kT, tol=self.tol)


class Proposal:
    """A LocalSampler proposal function, or a mixture of them (Samplers.jl:1-98):
    `terms` holds (kind, weight, magnitude) with kind one of _abi.PROPOSE_*."""

    def __init__(self, terms):
        self.terms = [(int(k), float(w), float(m)) for k, w, m in terms]

    def cstruct(self) -> _abi.Proposal:
        p = _abi.Proposal()
        p.n = len(self.terms)
        for i, (k, w, m) in enumerate(self.terms):
            p.kind[i], p.weight[i], p.magnitude[i] = k, w, m
        return p


propose_uniform = Proposal([(_abi.PROPOSE_UNIFORM, 1.0, 0.0)])   # Samplers.jl:14 (randspin)
propose_flip = Proposal([(_abi.PROPOSE_FLIP, 1.0, 0.0)])         # Samplers.jl:23


def propose_delta(magnitude) -> Proposal:
    """propose_delta(magnitude) (Samplers.jl:46-48): S + |S| ξ with ξ ~ N(0, magnitude²),
    renormalised; an infinite magnitude is propose_uniform (System.jl:455)."""
    return Proposal([(_abi.PROPOSE_DELTA, 1.0, float(magnitude))])


def mix_proposals(*terms) -> Proposal:
    """@mix_proposals weight1 propose1 weight2 propose2 ... (Samplers.jl:64-98)."""
    if len(terms) % 2:
        raise ValueError("Alternate weights and proposal functions.")
    out = []
    for w, p in zip(terms[0::2], terms[1::2]):
        if len(p.terms) != 1:
            raise ValueError("mix_proposals takes single proposal functions")
        k, _, m = p.terms[0]
        out.append((k, float(w), m))
    if not 1 <= len(out) <= 4:
        raise ValueError("a proposal mixture has 1 to 4 functions")
    return Proposal(out)


class LocalSampler:
    """LocalSampler(; kT, nsweeps=1.0, propose=propose_uniform) (Samplers.jl:101-137).

    `ΔE` and `ΔS` accumulate the energy and net dipole changes of accepted updates."""

    def __init__(self, *, kT, nsweeps=1.0, propose=None):
        self.kT = float(kT)
        self.nsweeps = float(nsweeps)
        self.propose = propose if propose is not None else propose_uniform
        self.ΔE = 0.0
        self.ΔS = np.zeros(3)

    def copy(self):
        return LocalSampler(kT=self.kT, nsweeps=self.nsweeps, propose=self.propose)


@dataclass
class PairCoupling:
    scalar: float
    bilin: np.ndarray        # 3x3
    biquad: object           # 0.0, float, or 5x5


class System:
    """System(crystal, moments, mode; dims, seed) (src/System/System.jl:33-93)."""

    def __init__(self, crystal: Crystal, moments, mode: str, dims=(1, 1, 1), seed=None,
                 precision: str = "fp64", device: int | None = 0):
        """`device=None` builds the host tables only (no GPU handle); such a System can
        feed the CPU oracle but cannot step."""
        mode = mode.lstrip(":")
        if mode not in _MODES:
            raise ValueError("Mode must be `:SUN`, `:dipole`, or `:dipole_uncorrected`")
        self.crystal = crystal
        self.mode = mode
        self.dims = tuple(int(x) for x in dims)
        na = crystal.natoms
        self.natoms = na
        mom = dict(moments)
        if len(mom) == 1 and na > 1 and 1 in mom:
            mom = {i: mom[1] for i in range(1, na + 1)}
        if sorted(mom) != list(range(1, na + 1)):
            raise ValueError("a Moment is required for every atom (or one Moment for all)")
        self.moments = [mom[i] for i in range(1, na + 1)]
        Ns = [int(round(2 * m.s + 1)) for m in self.moments]
        if mode == "SUN":
            if len(set(Ns)) != 1:
                raise ValueError("Currently all spins S must be equal in SU(N) mode")
            self.N = Ns[0]
        else:
            self.N = 0
        L1, L2, L3 = self.dims
        self.ncell = L1 * L2 * L3
        self.nsites = self.ncell * na
        ns = self.nsites
        self.precision = precision
        atom = np.repeat(np.arange(na), self.ncell)
        self._atom_of_site = atom
        kap = np.array([m.s for m in self.moments]) if mode != "SUN" else np.ones(na)
        self._kappa = np.ascontiguousarray(kap[atom].astype(float))
        self._g = np.ascontiguousarray(np.stack([self.moments[a].gmat() for a in atom]))     # (ns, 3, 3)
        self._field = np.zeros((ns, 3))
        self._pairs: dict[Bond, PairCoupling] = {}
        self._onsite = [None] * na
        # inhomogeneous systems: per site, Sunny's pair list [Bond, PairCoupling, isculled]
        # and its onsite coupling (None while the system is homogeneous)
        self._site_pairs: list | None = None
        self._site_onsite: list | None = None
        # SU(N) general pair couplings: bond -> [(A, B), ...] (Types.jl:23-30)
        self._general: dict[Bond, list] = {}
        self._base_dip = np.zeros((na, L3, L2, L1, 3))
        self._base_coh = np.zeros((na, L3, L2, L1, max(self.N, 1)), dtype=complex)
        self.rng = np.random.default_rng(seed)
        self.seed = int(seed) if seed is not None else int(self.rng.integers(0, 2**62))
        self.noise_step = 0
        self.mc_sweep = 0
        self._ewald = None            # (μ0 μB², demag 3x3) when dipole-dipole is enabled
        self._ewald_dirty = False
        self._couplings_dirty = True
        self._host_newer = True
        self._dev_newer = False
        self._h = None
        self._lib = None
        self.device = device
        if device is None:
            self.polarize_spins((0, 0, 1))
            return
        self._lib = _abi.load()
        d = _abi.Desc()
        d.dims[:] = self.dims
        d.natoms, d.N, d.mode = na, self.N, _MODES[mode]
        d.precision = _abi.FP32 if precision == "fp32" else _abi.FP64
        d.device = device
        h = C.c_void_p()
        _abi.check(self._lib.sgb_create(C.byref(d), C.byref(h)), self._lib, None)
        self._h = h
        self.polarize_spins((0, 0, 1))

    # ---- lifetime -------------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None) and self._lib is not None:
            self._lib.sgb_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    # ---- state views ------------------------------------------------------------------
    def _sync_to_host(self):
        if self._dev_newer:
            dip = np.empty((self.nsites, 3))
            coh = np.empty((self.nsites, self.N, 2)) if self.N else None
            _abi.check(self._lib.sgb_get_state(self._h, _abi.dptr(dip), _abi.dptr(coh)), self._lib, self._h)
            self._base_dip.reshape(-1, 3)[:] = dip
            if self.N:
                self._base_coh.reshape(-1, self.N)[:] = coh[..., 0] + 1j * coh[..., 1]
            self._dev_newer = False

    def _sync_to_device(self):
        if self._h is None:
            raise RuntimeError("this System was built without a device (device=None)")
        if self._couplings_dirty:
            self._upload_couplings()
        if self._host_newer:
            if self.N:
                coh = np.ascontiguousarray(np.stack([self._base_coh.real, self._base_coh.imag], -1).reshape(-1))
                _abi.check(self._lib.sgb_set_state(self._h, None, _abi.dptr(coh)), self._lib, self._h)
            else:
                dip = np.ascontiguousarray(self._base_dip.reshape(-1))
                _abi.check(self._lib.sgb_set_state(self._h, _abi.dptr(dip), None), self._lib, self._h)
            self._host_newer = False

    @property
    def dipoles(self) -> np.ndarray:
        """Array indexed [c1, c2, c3, atom, component] (0-based), like Sunny's sys.dipoles."""
        self._sync_to_host()
        self._host_newer = True
        return self._base_dip.transpose(3, 2, 1, 0, 4)

    @property
    def coherents(self) -> np.ndarray:
        self._sync_to_host()
        self._host_newer = True
        return self._base_coh.transpose(3, 2, 1, 0, 4)

    def dipoles_flat(self) -> np.ndarray:
        """Copy of the dipoles in site order (ns, 3)."""
        self._sync_to_host()
        return self._base_dip.reshape(-1, 3).copy()

    def coherents_flat(self) -> np.ndarray:
        self._sync_to_host()
        return self._base_coh.reshape(-1, self.N).copy()

    def set_state_flat(self, dipoles=None, coherents=None):
        """Overwrite the state from site-ordered arrays (dipoles (ns, 3) or coherents (ns, N))."""
        full = (self.N == 0 and dipoles is not None) or (self.N > 0 and coherents is not None)
        if not full:
            self._sync_to_host()
        self._dev_newer = False
        if dipoles is not None:
            self._base_dip.reshape(-1, 3)[:] = dipoles
        if coherents is not None:
            self._base_coh.reshape(-1, self.N)[:] = coherents
            self._base_dip.reshape(-1, 3)[:] = expected_spin(np.asarray(coherents))
        self._host_newer = True

    @property
    def kappas(self) -> np.ndarray:
        return self._kappa

    def set_kappas(self, kappa):
        """Rescale |S| = κ (dipole) or |Z|² = κ (SU(N)) per site, keeping directions."""
        self._sync_to_host()
        self._kappa[:] = np.broadcast_to(np.asarray(kappa, dtype=float), self._kappa.shape)
        flatd = self._base_dip.reshape(-1, 3)
        if self.N:
            flatz = self._base_coh.reshape(-1, self.N)
            nz = np.linalg.norm(flatz, axis=1)
            flatz[:] = np.where(self._kappa[:, None] == 0, 0, flatz / np.where(nz == 0, 1, nz)[:, None] * np.sqrt(self._kappa)[:, None])
            flatd[:] = expected_spin(flatz)
        else:
            nd = np.linalg.norm(flatd, axis=1)
            flatd[:] = np.where(self._kappa[:, None] == 0, 0, flatd / np.where(nd == 0, 1, nd)[:, None] * self._kappa[:, None])
        self._host_newer = True
        self._couplings_dirty = True

    # ---- site helpers -------------------------------------------------------------------
    def site_index(self, c1, c2, c3, a) -> int:
        """0-based linear site of (c1, c2, c3, atom), all 1-based as Sunny's Site."""
        L1, L2, L3 = self.dims
        return (c1 - 1) + L1 * ((c2 - 1) + L2 * ((c3 - 1) + L3 * (a - 1)))

    def spin_label(self, i: int) -> float:
        return self.moments[i - 1].s

    # ---- couplings --------------------------------------------------------------------
    def _upload_couplings(self):
        lib, h = self._lib, self._h
        _abi.check(lib.sgb_set_sites(h, _abi.dptr(self._kappa), _abi.dptr(np.ascontiguousarray(self._g.transpose(0, 2, 1)).reshape(-1)),
                                     _abi.dptr(np.ascontiguousarray(self._field.reshape(-1)))), lib, h)
        if self._ewald_dirty:
            if self._ewald is None:
                _abi.check(lib.sgb_set_dipole_dipole(h, 0.0, None, None, None), lib, h)
            else:
                mu0, demag = self._ewald
                lat = np.ascontiguousarray(np.asarray(self.crystal.latvecs, dtype=float).T.reshape(-1))   # column-major
                pos = np.ascontiguousarray(np.array([self.crystal.position(i) for i in range(1, self.natoms + 1)],
                                                    dtype=float).reshape(-1))
                dm = np.ascontiguousarray(np.asarray(demag, dtype=float).T.reshape(-1))
                _abi.check(lib.sgb_set_dipole_dipole(h, float(mu0), _abi.dptr(dm), _abi.dptr(lat), _abi.dptr(pos)), lib, h)
            self._ewald_dirty = False
        if self._site_pairs is not None:
            _abi.check(lib.sgb_set_onsite_at(h, _abi.dptr(self.onsite_site_table())), lib, h)
            sb = self.site_bond_table()
            arr = (_abi.SiteBondC * max(1, len(sb)))()
            for k, b in enumerate(sb):
                arr[k] = b
            _abi.check(lib.sgb_set_bonds_at(h, arr, len(sb)), lib, h)
            self._couplings_dirty = False
            return
        for a in range(self.natoms):
            _abi.check(lib.sgb_set_onsite(h, a, _abi.dptr(self._onsite_row(self._onsite[a]))), lib, h)
        bonds = self.bond_table()
        arr = (_abi.BondC * max(1, len(bonds)))()
        for k, b in enumerate(bonds):
            arr[k] = b
        _abi.check(lib.sgb_set_bonds(h, arr, len(bonds)), lib, h)
        if self.N:
            gb, A, B = self.general_table()
            cm = lambda M: np.ascontiguousarray(np.stack([np.swapaxes(M, -1, -2).real, np.swapaxes(M, -1, -2).imag], -1)).reshape(-1)
            ga, gbm = (cm(A), cm(B)) if len(gb) else (None, None)
            _abi.check(lib.sgb_set_general(h, gb.ctypes.data_as(C.POINTER(C.c_int32)) if len(gb) else None, len(gb),
                                           _abi.dptr(ga), _abi.dptr(gbm)), lib, h)
        self._couplings_dirty = False

    def _onsite_row(self, oc) -> np.ndarray:
        """One onsite coupling in the C layout: 28 Stevens coefficients (dipole modes) or
        the N x N matrix column-major as (re, im) (SU(N) mode)."""
        if self.N:
            M = np.zeros((self.N, self.N), dtype=complex) if oc is None else oc
            return np.ascontiguousarray(np.stack([M.T.real, M.T.imag], -1).reshape(-1))
        return np.zeros(28) if oc is None else np.ascontiguousarray(oc, dtype=float)

    @staticmethod
    def _bond_c(b: Bond, pc: PairCoupling):
        e = _abi.BondC()
        e.i, e.j = b.i - 1, b.j - 1
        e.n[:] = b.n
        e.scalar = pc.scalar
        e.bilin[:] = list(np.asarray(pc.bilin, dtype=float).T.reshape(-1))
        if isinstance(pc.biquad, np.ndarray):
            e.biquad_kind = 2
            e.biquad[:] = list(pc.biquad.T.reshape(-1))
        elif pc.biquad != 0:
            e.biquad_kind = 1
            e.biquad[0] = float(pc.biquad)
        return e

    def bond_table(self):
        """Non-culled pair couplings in the C layout (0-based atoms, column-major J)."""
        return [self._bond_c(b, pc) for b, pc in self._pairs.items()]

    def general_table(self):
        """SU(N) general pair couplings: (bond index into bond_table(), A [n][N][N], B [n][N][N])."""
        idx = {b: k for k, b in enumerate(self._pairs)}
        gb, A, B = [], [], []
        for b, terms in self._general.items():
            for a_, b_ in terms:
                gb.append(idx[b])
                A.append(a_)
                B.append(b_)
        N = max(self.N, 1)
        return (np.array(gb, dtype=np.int32), np.array(A, dtype=complex).reshape(-1, N, N),
                np.array(B, dtype=complex).reshape(-1, N, N))

    def set_pair_coupling_op(self, op, bond: Bond):
        """set_pair_coupling!(sys, op, bond) in SU(N) mode on this one bond (and its
        reverse; no symmetry propagation): `op` is a Hermitian operator on the product
        space of the two sites (N² x N²), or a function of the two sites' spin matrices in
        that space as in Sunny ((Si, Sj) -> op). Stored as the general tensor
        decomposition Σ_k A_k ⊗ B_k of the whole operator (PairExchange.jl:185-244 keeps
        scalar, bilinear and biquadratic parts apart; the sum is the same operator)."""
        from .crystal import bond_parity
        if self.mode != "SUN":
            raise ValueError("General couplings require mode :SUN")
        if bond.i == bond.j and all(x == 0 for x in bond.n):
            raise ValueError("Bond must connect different atoms.")
        N = self.N
        if callable(op):
            I = np.eye(N)
            Sm = spin_matrices_of_dim(N)
            op = op([np.kron(S, I) for S in Sm], [np.kron(I, S) for S in Sm])
        terms = tensor_decomposition(op, N, N)
        if not bond_parity(bond):
            bond = bond.reverse()
            terms = [(b_, a_) for a_, b_ in terms]
        if bond not in self._pairs:
            self._pairs[bond] = PairCoupling(0.0, np.zeros((3, 3)), 0.0)
        self._general[bond] = terms
        self._couplings_dirty = True

    # ---- inhomogeneous systems (Interactions.jl:81-100, 237-257; PairExchange.jl:431-605) ----
    def is_homogeneous(self) -> bool:
        return self._site_pairs is None

    def _site_of(self, site) -> int:
        """0-based linear site of a Sunny Site (c1, c2, c3, atom), all 1-based, or of an int."""
        if isinstance(site, (int, np.integer)):
            return int(site)
        c1, c2, c3, a = (int(x) for x in site)
        return self.site_index(c1, c2, c3, a)

    def _cell_atom(self, i: int):
        L1, L2, L3 = self.dims
        return (i % L1, (i // L1) % L2, (i // (L1 * L2)) % L3), i // self.ncell

    def bonded_site(self, i: int, b: Bond) -> int:
        """bonded_site (System.jl:204-212), 0-based linear sites."""
        (c1, c2, c3), _ = self._cell_atom(i)
        L1, L2, L3 = self.dims
        return self.site_index((c1 + b.n[0]) % L1 + 1, (c2 + b.n[1]) % L2 + 1, (c3 + b.n[2]) % L3 + 1, b.j)

    def _make_inhomogeneous(self):
        from .crystal import bond_parity
        if self._general:
            raise ValueError("general (tensor-decomposed) pair couplings are supported on homogeneous systems only")
        per_atom = [[] for _ in range(self.natoms)]
        for b, pc in self._pairs.items():
            per_atom[b.i - 1].append([b, pc, not bond_parity(b)])
            rb = b.reverse()
            rq = pc.biquad.T if isinstance(pc.biquad, np.ndarray) else pc.biquad
            per_atom[b.j - 1].append([rb, PairCoupling(pc.scalar, np.asarray(pc.bilin, dtype=float).T, rq),
                                      not bond_parity(rb)])
        for lst in per_atom:
            lst.sort(key=lambda e: e[2])          # non-culled first (Interactions.jl:38-41)
        ns = self.nsites
        self._site_pairs = [[list(e) for e in per_atom[i // self.ncell]] for i in range(ns)]
        self._site_onsite = [self._onsite[i // self.ncell] for i in range(ns)]
        self._couplings_dirty = True

    def _require_inhomogeneous(self):
        if self._site_pairs is None:
            raise ValueError("Use `to_inhomogeneous` first.")

    def _site_bond(self, i: int, k: int, offset):
        """sites_to_internal_bond (PairExchange.jl:390-430), 0-based linear sites."""
        (ca, a), (cb, b) = self._cell_atom(i), self._cell_atom(k)
        n0 = np.array(cb) - np.array(ca)
        dims = np.array(self.dims)
        if offset is not None:
            n = np.array(offset, dtype=int)
            if np.all(np.mod(n - n0, dims) == 0):
                return Bond(a + 1, b + 1, tuple(int(x) for x in n))
            raise ValueError(f"Cells {tuple(int(x) + 1 for x in ca)} and {tuple(int(x) + 1 for x in cb)} are not "
                             f"compatible with the offset {tuple(int(x) for x in n)} for a system with dimensions "
                             f"{self.dims}.")
        cands = [Bond(a + 1, b + 1, tuple(int(x) for x in n0 + dims * np.array((w1, w2, w3))))
                 for w3 in (-1, 0, 1) for w2 in (-1, 0, 1) for w1 in (-1, 0, 1)]
        d = np.array([self.crystal.distance(c) for c in cands])
        perm = np.argsort(d, kind="stable")
        if 4 * d[perm[0]] < d[perm[1]] - 1e-12:
            return cands[perm[0]]
        raise ValueError(f"Ambiguous offset vector. Possibilities include {cands[perm[0]].n} and {cands[perm[1]].n}. "
                         "Try using a bigger system size, or pass an explicit offset.")

    @staticmethod
    def _replace_in_list(lst, b: Bond, pc: PairCoupling | None):
        """replace_coupling_in_list! (PairExchange.jl:431-445)."""
        from .crystal import bond_parity
        lst[:] = [e for e in lst if e[0] != b]
        if pc is None:
            return
        lst.append([b, pc, not bond_parity(b)])
        lst.sort(key=lambda e: e[2])

    def set_pair_coupling_at(self, scalar: float, bilin, biquad, site1, site2, offset=None):
        """set_pair_coupling_at_aux! (PairExchange.jl:447-468): one coupling on the single
        bond from site1 to site2, stored from both ends, ignoring crystal symmetry."""
        self._require_inhomogeneous()
        i, k = self._site_of(site1), self._site_of(site2)
        if self._kappa[i] == 0 or self._kappa[k] == 0:
            raise ValueError("Cannot couple vacant site")
        J = np.asarray(bilin, dtype=float)
        J = J * np.eye(3) if J.ndim == 0 else J.reshape(3, 3)
        if self.mode == "dipole":
            (_, a), (_, b) = self._cell_atom(i), self._cell_atom(k)
            biquad = biquad * rcs_factors(self.spin_label(a + 1))[2] * rcs_factors(self.spin_label(b + 1))[2]
        bond = self._site_bond(i, k, offset)
        zero = scalar == 0 and not np.any(J) and (np.all(biquad == 0) if isinstance(biquad, np.ndarray) else biquad == 0)
        rq = biquad.T if isinstance(biquad, np.ndarray) else biquad
        self._replace_in_list(self._site_pairs[i], bond, None if zero else PairCoupling(float(scalar), J, biquad))
        self._replace_in_list(self._site_pairs[k], bond.reverse(), None if zero else PairCoupling(float(scalar), J.T, rq))
        self._couplings_dirty = True

    def set_exchange_at(self, J, site1, site2, biquad: float = 0.0, offset=None):
        """set_exchange_at!(sys, J, site1, site2; biquad, offset) (PairExchange.jl:470-490),
        with adapt_for_biquad's scalar and bilinear shifts (PairExchange.jl:300-330)."""
        J = np.asarray(J, dtype=float)
        J = J * np.eye(3) if J.ndim == 0 else J.reshape(3, 3)
        scalar = 0.0
        biquad = float(biquad)
        if biquad != 0:
            (_, a), (_, b) = self._cell_atom(self._site_of(site1)), self._cell_atom(self._site_of(site2))
            s1, s2 = self.spin_label(a + 1), self.spin_label(b + 1)
            if self.mode in ("SUN", "dipole"):
                J = J - (biquad / 2) * np.eye(3)
                scalar += biquad * s1 * (s1 + 1) * s2 * (s2 + 1) / 3
            else:
                scalar += biquad * s1**2 * s2**2 / 3
        self.set_pair_coupling_at(scalar, J, biquad, site1, site2, offset)

    def set_onsite_coupling_at(self, op, site):
        """set_onsite_coupling_at!(sys, op, site) (OnsiteCoupling.jl:222-231)."""
        self._require_inhomogeneous()
        i = self._site_of(site)
        if self._kappa[i] == 0:
            raise ValueError("Cannot couple vacant site")
        _, a = self._cell_atom(i)
        s = self.spin_label(a + 1)
        N = int(round(2 * s + 1))
        if callable(op):
            op = op(*spin_matrices_of_dim(N))
        A = np.asarray(op, dtype=complex)
        if A.shape != (N, N):
            raise ValueError("Invalid matrix size.")
        if not np.allclose(A, A.conj().T):
            raise ValueError("Operator is not Hermitian")
        if self.mode == "SUN":
            self._site_onsite[i] = A
        elif self.mode == "dipole":
            self._site_onsite[i] = stevens_expansion_for_dipole((A + A.conj().T) / 2, s, renormalize=True)
        else:
            raise ValueError("System with mode :dipole_uncorrected requires Stevens coefficients")
        self._couplings_dirty = True

    def set_vacancy_at(self, site):
        """set_vacancy_at!(sys, site) (Interactions.jl:237-257): κ = 0, zero state, no onsite
        coupling, and the site removed from its neighbours' lists (its own list stays)."""
        self._require_inhomogeneous()
        i = self._site_of(site)
        self._sync_to_host()
        self._kappa[i] = 0.0
        self._base_dip.reshape(-1, 3)[i] = 0
        if self.N:
            self._base_coh.reshape(-1, self.N)[i] = 0
        self._site_onsite[i] = None
        for b, _, _ in self._site_pairs[i]:
            k = self.bonded_site(i, b)
            rb = b.reverse()
            lst = self._site_pairs[k]
            hits = [e for e in lst if e[0] == rb]
            if len(hits) != 1:
                raise ValueError("inconsistent pair lists")
            lst.remove(hits[0])
        self._host_newer = True
        self._couplings_dirty = True

    def remove_periodicity(self, flags):
        """remove_periodicity!(sys, flags) (PairExchange.jl:592-605): drops every bond that
        leaves the supercell along a flagged dimension."""
        self._require_inhomogeneous()
        for i in range(self.nsites):
            (c, _) = self._cell_atom(i)
            self._site_pairs[i] = [e for e in self._site_pairs[i]
                                   if all((not f) or 0 <= c[d] + e[0].n[d] < self.dims[d] for d, f in enumerate(flags))]
        self._couplings_dirty = True

    def site_bond_table(self):
        """Every site's non-culled pair couplings in the C layout (sgb_site_bond), in site order."""
        out = []
        for i, lst in enumerate(self._site_pairs):
            (c, _) = self._cell_atom(i)
            for b, pc, culled in lst:
                if culled:
                    continue
                e = _abi.SiteBondC()
                e.cell[:] = [int(x) for x in c]
                e.bond = self._bond_c(b, pc)
                out.append(e)
        return out

    def onsite_site_table(self) -> np.ndarray:
        """Per-site onsite couplings in the C layout, site order."""
        return np.ascontiguousarray(np.concatenate([self._onsite_row(o) for o in self._site_onsite]))

    def set_pair_coupling(self, bond: Bond, scalar: float, bilin, biquad):
        """Set one coupling on `bond` and its equivalents (PairExchange.jl:185-244)."""
        J = np.asarray(bilin, dtype=float)
        J = J * np.eye(3) if J.ndim == 0 else J.reshape(3, 3)
        if bond.i == bond.j and all(x == 0 for x in bond.n):
            raise ValueError("Bond must connect different atoms.")
        for k in (bond.i, bond.j):
            if not 1 <= k <= self.natoms:
                raise ValueError(f"Atom index {k} is out of range.")
        if self.mode == "dipole":
            biquad = biquad * rcs_factors(self.spin_label(bond.i))[2] * rcs_factors(self.spin_label(bond.j))[2]
        for b, Jb in self.crystal.equivalent_bonds(bond, J):
            bq = biquad
            if isinstance(bq, np.ndarray) and not b == bond:
                raise ValueError("matrix biquadratic couplings are set per bond")
            self._pairs[b] = PairCoupling(float(scalar), Jb, bq)
        self._couplings_dirty = True

    def set_bond_coupling(self, bond: Bond, scalar: float, bilin, biquad):
        """Set a coupling on exactly one bond (and its reverse), without propagation. In
        dipole mode the biquadratic part is renormalised by the RCS factors like
        set_pair_coupling_at! (PairExchange.jl:447-468)."""
        from .crystal import bond_parity
        J = np.asarray(bilin, dtype=float)
        J = J * np.eye(3) if J.ndim == 0 else J.reshape(3, 3)
        if bond.i == bond.j and all(x == 0 for x in bond.n):
            raise ValueError("Bond must connect different atoms.")
        if self.mode == "dipole":
            biquad = biquad * rcs_factors(self.spin_label(bond.i))[2] * rcs_factors(self.spin_label(bond.j))[2]
        if not bond_parity(bond):
            bond, J = bond.reverse(), J.T
            if isinstance(biquad, np.ndarray):
                biquad = biquad.T
        self._pairs[bond] = PairCoupling(float(scalar), J, biquad)
        self._couplings_dirty = True

    def set_exchange(self, J, bond: Bond, biquad: float = 0.0):
        """set_exchange!(sys, J, bond; biquad) with adapt_for_biquad (PairExchange.jl:300-385)."""
        J = np.asarray(J, dtype=float)
        J = J * np.eye(3) if J.ndim == 0 else J.reshape(3, 3)
        scalar = 0.0
        biquad = float(biquad)
        if biquad != 0:
            if self.mode in ("SUN", "dipole"):
                s1, s2 = self.spin_label(bond.i), self.spin_label(bond.j)
                J = J - (biquad / 2) * np.eye(3)
                scalar += biquad * s1 * (s1 + 1) * s2 * (s2 + 1) / 3
            else:
                s1, s2 = self.spin_label(bond.i), self.spin_label(bond.j)
                scalar += biquad * s1**2 * s2**2 / 3
        self.set_pair_coupling(bond, scalar, J, biquad)

    def set_onsite_coupling(self, op, i: int, atoms=None):
        """set_onsite_coupling!(sys, op, i) (OnsiteCoupling.jl:159-210). `op` is an N x N
        matrix in the spin-s representation of atom i, or a function of (Sx, Sy, Sz).
        Sunny propagates the coupling to symmetry-equivalent atoms; here the coupling is
        applied to atom i and to any extra `atoms` listed."""
        if not 1 <= i <= self.natoms:
            raise ValueError(f"Atom index {i} is out of range.")
        s = self.spin_label(i)
        N = int(round(2 * s + 1))
        if callable(op):
            op = op(*spin_matrices_of_dim(N))
        A = np.asarray(op, dtype=complex)
        if A.shape != (N, N):
            raise ValueError("Invalid matrix size.")
        if not np.allclose(A, A.conj().T):
            raise ValueError("Operator is not Hermitian")
        if N == 2:
            if self.mode == "dipole":
                raise ValueError("Consider mode :dipole_uncorrected. Onsite coupling is trivial for quantum spin 1/2.")
            if self.mode == "SUN":
                raise ValueError("Onsite coupling is trivial for quantum spin 1/2.")
        if self.mode == "SUN":
            val = A
        elif self.mode == "dipole":
            val = stevens_expansion_for_dipole((A + A.conj().T) / 2, s, renormalize=True)
        else:
            raise ValueError("System with mode :dipole_uncorrected requires Stevens coefficients (use set_onsite_stevens)")
        for a in [i] + list(atoms or []):
            self._onsite[a - 1] = val
        self._couplings_dirty = True

    def set_onsite_stevens(self, coeffs28, i: int, atoms=None):
        """Dipole modes: set the 28 (already renormalised) Stevens coefficients directly."""
        if self.N:
            raise ValueError("Stevens coefficients are for dipole modes")
        c = np.asarray(coeffs28, dtype=float).reshape(28)
        for a in [i] + list(atoms or []):
            self._onsite[a - 1] = c.copy()
        self._couplings_dirty = True

    def enable_dipole_dipole(self, mu0_muB2=None, demag=1 / 3):
        """enable_dipole_dipole!(sys, μ0_μB²; demag=1/3) (Interactions.jl:180-188): Ewald-summed
        dipole-dipole interactions over the periodic supercell; `demag` is a scalar (times
        the identity) or a 3x3 tensor."""
        if mu0_muB2 is None:
            import warnings
            warnings.warn("Deprecated syntax! Consider `enable_dipole_dipole(sys, units.vacuum_permeability)`")
            mu0_muB2 = 0.6745817653   # μ0 μB² in meV Å³ (Units.jl:57)
        dm = np.asarray(demag, dtype=float)
        self._ewald = (float(mu0_muB2), dm * np.eye(3) if dm.ndim == 0 else dm.reshape(3, 3))
        self._ewald_dirty = True
        self._couplings_dirty = True

    def set_field(self, B):
        """set_field!(sys, B) (Interactions.jl:210-214); B already scaled by μB."""
        self._field[:] = np.asarray(B, dtype=float).reshape(3)
        self._couplings_dirty = True

    def set_field_at(self, B, site: int):
        self._field[site] = np.asarray(B, dtype=float).reshape(3)
        self._couplings_dirty = True

    # ---- state initialisation -------------------------------------------------------------
    def polarize_spins(self, direction):
        """polarize_spins!(sys, dir) (System.jl:566-570)."""
        d = np.asarray(direction, dtype=float)
        self._sync_to_host()
        flatd = self._base_dip.reshape(-1, 3)
        if self.N:
            z = ket_from_dipole(d, self.N)
            z = z / np.sqrt(np.vdot(z, z).real)
            flatz = self._base_coh.reshape(-1, self.N)
            flatz[:] = z[None, :] * np.sqrt(self._kappa)[:, None]
            flatd[:] = expected_spin(flatz)
        else:
            flatd[:] = self._kappa[:, None] * (d / np.linalg.norm(d))[None, :]
        self._host_newer = True

    def set_langevin_cluster(self, mode: int):
        """Kernel choice of Langevin steps on dipole lattices: -1 timed choice (default),
        0 persistent grid kernel, 1 one thread-block cluster holding the lattice."""
        self._sync_to_device()
        _abi.check(self._lib.sgb_set_langevin_cluster(self._h, int(mode)), self._lib, self._h)

    def langevin_kernel(self) -> int:
        """The Langevin kernel in use: -1 before the first timed choice, 0 the persistent
        grid kernel, c > 0 the cluster kernel on a cluster of c CTAs."""
        c = C.c_int32(0)
        _abi.check(self._lib.sgb_langevin_kernel(self._h, C.byref(c)), self._lib, self._h)
        return int(c.value)

    def set_wait_limit(self, seconds: float):
        """Wall-clock limit of the device-side waits of this system's persistent kernels
        (0: the default, 4 s). A wait that runs past it fails the call with
        SunnyGPUError(SGB_ERR_TIMEOUT); the system stays usable."""
        _abi.check(self._lib.sgb_set_wait_limit(self._h, float(seconds)), self._lib, self._h)

    def set_midpoint_predictor(self, order: int):
        """First iterate of each dipole midpoint step within one call: 0 S' = S (the
        reference's choice), k in 1..4 the degree-k extrapolation of the last states.
        Default 4 for FP32 dipole systems, 0 otherwise."""
        _abi.check(self._lib.sgb_set_midpoint_predictor(self._h, int(order)), self._lib, self._h)

    def randomize_spins(self):
        """randomize_spins!(sys) (System.jl:444-452, 513-517)."""
        self._sync_to_host()
        ns = self.nsites
        if self.N:
            z = self.rng.standard_normal((ns, self.N)) + 1j * self.rng.standard_normal((ns, self.N))
            nz = np.sqrt(np.sum(np.abs(z) ** 2, axis=1) / np.where(self._kappa == 0, 1, self._kappa))
            z = np.where(self._kappa[:, None] == 0, 0, z / nz[:, None])
            self._base_coh.reshape(-1, self.N)[:] = z
            self._base_dip.reshape(-1, 3)[:] = expected_spin(z)
        else:
            v = self.rng.standard_normal((ns, 3))
            self._base_dip.reshape(-1, 3)[:] = self._kappa[:, None] * v / np.linalg.norm(v, axis=1)[:, None]
        self._host_newer = True


# ---- free functions mirroring Sunny's exported API -----------------------------------------

def set_exchange(sys: System, J, bond: Bond, biquad: float = 0.0):
    sys.set_exchange(J, bond, biquad)


def set_onsite_coupling(sys: System, op, i: int, atoms=None):
    sys.set_onsite_coupling(op, i, atoms)


def set_field(sys: System, B):
    sys.set_field(B)


def randomize_spins(sys: System):
    sys.randomize_spins()


def polarize_spins(sys: System, direction):
    sys.polarize_spins(direction)


def enable_dipole_dipole(sys: System, mu0_muB2=None, demag=1 / 3):
    sys.enable_dipole_dipole(mu0_muB2, demag)


def energy(sys: System) -> float:
    """energy(sys) in FP64 (Interactions.jl:401-432)."""
    sys._sync_to_device()
    E = C.c_double()
    _abi.check(sys._lib.sgb_energy(sys._h, C.byref(E), None), sys._lib, sys._h)
    return E.value


def energy_per_site(sys: System) -> float:
    return energy(sys) / sys.nsites


def magnetization(sys: System) -> np.ndarray:
    """sum(sys.dipoles) in FP64 (ParallelTempering.jl:31)."""
    sys._sync_to_device()
    M = np.zeros(3)
    _abi.check(sys._lib.sgb_energy(sys._h, None, _abi.dptr(M)), sys._lib, sys._h)
    return M


def energy_grad(sys: System) -> np.ndarray:
    """energy_grad_dipoles / energy_grad_coherents (Interactions.jl:689-698), site order."""
    sys._sync_to_device()
    if sys.N:
        out = np.zeros((sys.nsites, sys.N, 2))
        _abi.check(sys._lib.sgb_energy_grad(sys._h, _abi.dptr(out)), sys._lib, sys._h)
        return out[..., 0] + 1j * out[..., 1]
    out = np.zeros((sys.nsites, 3))
    _abi.check(sys._lib.sgb_energy_grad(sys._h, _abi.dptr(out)), sys._lib, sys._h)
    return out


def step(sys: System, integrator, nsteps: int = 1, noise: np.ndarray | None = None, max_iters: int = 100) -> int:
    """step!(sys, integrator), `nsteps` times (Integrators.jl:309-452).

    Langevin noise comes from the device generator keyed by (sys.seed, step counter),
    or from `noise` (standard normals, [nsteps][ns][3] or complex [nsteps][ns][N]).
    Returns the number of midpoint iterations (0 for Langevin)."""
    if isinstance(integrator, LocalSampler):
        return _local_sampler_steps(sys, integrator, nsteps, noise)
    if math.isnan(integrator.dt):
        raise ValueError("Set integration timestep `dt`.")
    sys._sync_to_device()
    lib, h = sys._lib, sys._h
    if isinstance(integrator, Langevin):
        nz = None
        if noise is not None:
            noise = np.asarray(noise)
            if sys.N:
                noise = np.stack([noise.real, noise.imag], -1)
            nz = np.ascontiguousarray(noise, dtype=float).reshape(-1)
            per = sys.nsites * (2 * sys.N if sys.N else 3)
            if nz.size != per * nsteps:
                raise ValueError("noise must hold nsteps x nsites x components normals")
        rc = lib.sgb_langevin(h, integrator.dt, integrator.damping, integrator.kT, sys.seed, sys.noise_step, nsteps,
                              _abi.dptr(nz))
        sys.noise_step += nsteps
        sys._dev_newer = True
        _abi.check(rc, lib, h)
        return 0
    if isinstance(integrator, ImplicitMidpoint):
        iters = C.c_int64()
        rc = lib.sgb_midpoint(h, integrator.dt, integrator.damping, integrator.tol, max_iters, nsteps, C.byref(iters))
        sys._dev_newer = True
        _abi.check(rc, lib, h)
        return iters.value
    raise TypeError(f"unsupported integrator {type(integrator).__name__}")


def to_inhomogeneous(sys: System) -> System:
    """to_inhomogeneous(sys) (Interactions.jl:81-100): a copy whose couplings are held per
    site, to be edited with set_exchange_at, set_pair_coupling_at, set_onsite_coupling_at,
    set_vacancy_at and remove_periodicity."""
    if not sys.is_homogeneous():
        raise ValueError("System is already inhomogeneous.")
    c = clone_system(sys)
    c._make_inhomogeneous()
    return c


def set_exchange_at(sys: System, J, site1, site2, biquad: float = 0.0, offset=None):
    sys.set_exchange_at(J, site1, site2, biquad=biquad, offset=offset)


def set_onsite_coupling_at(sys: System, op, site):
    sys.set_onsite_coupling_at(op, site)


def set_vacancy_at(sys: System, site):
    sys.set_vacancy_at(site)


def remove_periodicity(sys: System, flags):
    sys.remove_periodicity(flags)


def clone_system(sys: System, seed=None, device="same", precision=None) -> System:
    """clone_system(sys) (System.jl:144-175): a new System with copies of the couplings,
    κ, g, field and state, on the same device (or `device`, in `precision`). Sunny copies
    the RNG; the clone keeps sys.seed and its counters unless `seed` is given."""
    if sys._h is not None:
        sys._sync_to_host()
    mom =[(i + 1, m) for i, m in enumerate(sys.moments)]
    c = System(sys.crystal, mom, sys.mode, sys.dims, seed=sys.seed if seed is None else seed,
               precision=precision or sys.precision, device=sys.device if device == "same" else device)
    c._kappa[:] = sys._kappa
    c._g[:] = sys._g
    c._field[:] = sys._field
    c._pairs = {b: PairCoupling(pc.scalar, np.array(pc.bilin, dtype=float),
                                pc.biquad.copy() if isinstance(pc.biquad, np.ndarray) else pc.biquad)
                for b, pc in sys._pairs.items()}
    c._onsite = [None if o is None else np.array(o) for o in sys._onsite]
    c._general = {b: [(np.array(a_), np.array(b_)) for a_, b_ in t] for b, t in sys._general.items()}
    if sys._site_pairs is not None:
        c._site_pairs = [[[e[0], PairCoupling(e[1].scalar, np.array(e[1].bilin, dtype=float),
                                              e[1].biquad.copy() if isinstance(e[1].biquad, np.ndarray) else e[1].biquad),
                           e[2]] for e in lst] for lst in sys._site_pairs]
        c._site_onsite = [None if o is None else np.array(o) for o in sys._site_onsite]
    if sys._ewald is not None:
        c._ewald = (sys._ewald[0], np.array(sys._ewald[1]))
        c._ewald_dirty = True
    c._base_dip[:] = sys._base_dip
    c._base_coh[:] = sys._base_coh
    if seed is None:
        c.noise_step, c.mc_sweep = sys.noise_step, sys.mc_sweep
    c._couplings_dirty = True
    c._host_newer = True
    return c


def _local_sampler_steps(sys: System, sampler: LocalSampler, nsteps: int, rand) -> int:
    """`nsteps` x step!(sys, sampler) (Samplers.jl:139-158). Random numbers come from the
    device generator keyed by (sys.seed, sweep counter), or from `rand`
    ([sweeps][ns][6]: 3 normals, mixture, acceptance and participation uniforms; in SU(N)
    mode [sweeps][ns][2N+3], N complex normals as (re, im) first)."""
    sys._sync_to_device()
    lib, h = sys._lib, sys._h
    per_step = math.ceil(sampler.nsweeps)
    per_site = 2 * sys.N + 3 if sys.N else 6
    if rand is not None:
        rand = np.ascontiguousarray(rand, dtype=float).reshape(-1)
        if rand.size != per_step * nsteps * sys.nsites * per_site:
            raise ValueError(f"rand must hold sweeps x nsites x {per_site} numbers")
    prop = sampler.propose.cstruct()
    # integer sweeps fuse into one launch; a fractional sweep ends every step
    calls = [(sampler.nsweeps * nsteps, 0)] if sampler.nsweeps == per_step else \
        [(sampler.nsweeps, k * per_step) for k in range(nsteps)]
    dE, dS = C.c_double(), np.zeros(3)
    for nsw, k0 in calls:
        r = None if rand is None else rand[k0 * sys.nsites * per_site:]
        rc = lib.sgb_local_sweeps(h, sampler.kT, nsw, C.byref(prop), sys.seed, sys.mc_sweep, _abi.dptr(r), C.byref(dE),
                                  _abi.dptr(dS))
        sys._dev_newer = True
        _abi.check(rc, lib, h)
        sys.mc_sweep += math.ceil(nsw)
        sampler.ΔE += dE.value
        sampler.ΔS = sampler.ΔS + dS
    return 0


@dataclass
class MinimizationResult:
    """MinimizationResult (Optimization.jl:1-10): converged, niters, energy."""
    converged: bool
    niters: int
    energy: float

    def __str__(self):
        # Optimization.jl:12-20
        if self.converged:
            return f"Converged in {self.niters} iterations"
        return f"Non-converged after {self.niters} iterations"


def minimize_energy(sys: System, maxiters: int = 1000, jitter: float = 1e-8) -> MinimizationResult:
    """minimize_energy!(sys; maxiters=1000, jitter=1e-8) (Optimization.jl:102-166), dipole
    modes, FP64 systems: conjugate-gradient descent on the unit spheres on the device.
    Warns when it does not converge, as the reference does."""
    sys._sync_to_device()
    conv, nit, E = C.c_int32(), C.c_int32(), C.c_double()
    seed = (sys.seed * 1000003 + sys.mc_sweep + 17) % (1 << 63)
    rc = sys._lib.sgb_minimize_energy(sys._h, int(maxiters), float(jitter), seed, C.byref(conv), C.byref(nit),
                                      C.byref(E))
    sys._dev_newer = True
    _abi.check(rc, sys._lib, sys._h)
    sys.mc_sweep += 1
    res = MinimizationResult(bool(conv.value), int(nit.value), float(E.value))
    if not res.converged:
        import warnings
        warnings.warn(str(res))
    return res


def local_energy_change(sys: System, site: int, S_new) -> float:
    """local_energy_change(sys, site, state) (Interactions.jl:311-373); `site` is the
    0-based linear index; S_new is a dipole, or a coherent state (N complex) in SU(N) mode."""
    sys._sync_to_device()
    out = C.c_double()
    if sys.N:
        z = np.asarray(S_new, dtype=complex).reshape(sys.N)
        Sn = np.ascontiguousarray(np.stack([z.real, z.imag], -1).reshape(-1))
    else:
        Sn = np.ascontiguousarray(S_new, dtype=float).reshape(3)
    _abi.check(sys._lib.sgb_local_energy_change(sys._h, int(site), _abi.dptr(Sn), C.byref(out)), sys._lib, sys._h)
    return out.value


def local_colors(sys: System):
    """(ncolors, color per site) of the bond-graph colouring the LocalSampler sweeps use."""
    sys._sync_to_device()
    n = C.c_int32()
    col = np.zeros(sys.nsites, dtype=np.int32)
    _abi.check(sys._lib.sgb_local_colors(sys._h, C.byref(n), col.ctypes.data_as(C.POINTER(C.c_int32))), sys._lib,
               sys._h)
    return n.value, col


def langevin_noise(sys: System, step_index: int) -> np.ndarray:
    """The standard normals the device generator uses for step `step_index` of sys.seed."""
    per = sys.nsites * (2 * sys.N if sys.N else 3)
    out = np.zeros(per)
    _abi.check(sys._lib.sgb_langevin_noise(sys._h, sys.seed, step_index, _abi.dptr(out)), sys._lib, sys._h)
    if sys.N:
        o = out.reshape(sys.nsites, sys.N, 2)
        return o[..., 0] + 1j * o[..., 1]
    return out.reshape(sys.nsites, 3)
