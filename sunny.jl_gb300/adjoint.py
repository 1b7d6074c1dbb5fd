"""Gradient of an S(q,ω) loss with respect to coupling parameters, through a
deterministic ImplicitMidpoint trajectory (discrete adjoint on the GPU, FP64).

Sunny.jl has no reverse rule for its dynamics. The parameters follow the labelled-
parameter convention of its fitting code (src/Fitting.jl:123-152,
src/ModelParams.jl:140-150): each parameter is a function f(sys, value) that sets one
coupling of the System, for example ``lambda s, v: s.set_exchange(v, bond)``. The
energy must be linear in every parameter, and different parameters must set different
couplings.

Supported: FP64 dipole-mode systems with bilinear pair couplings and onsite anisotropy
of rank <= 2, undamped midpoint dynamics, one cosine-window sample.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from .correlations import MeasureSpec, adjusted_dt_and_downsampling_factor
from .system import System


def twin_system(sys: System) -> System:
    """A host-only System with the same crystal, moments, mode and dims and no couplings."""
    moments = [(a + 1, m) for a, m in enumerate(sys.moments)]
    return System(sys.crystal, moments, sys.mode, dims=sys.dims, device=None)


def unit_coupling_sets(sys: System, params):
    """For every parameter f, the couplings that f(twin, 1.0) sets on an empty twin of
    `sys`: its non-culled bonds (C layout) and its onsite Stevens coefficients
    [natoms][28]. Returns (all bonds back to back, bond count per parameter, onsite
    coefficients [nparams][natoms][28])."""
    na = sys.natoms
    bonds, counts, onsite = [], [], []
    for f in params:
        twin = twin_system(sys)
        f(twin, 1.0)
        bt = twin.bond_table()
        bonds += bt
        counts.append(len(bt))
        onsite.append(np.stack([twin._onsite[a] if twin._onsite[a] is not None else np.zeros(28) for a in range(na)]))
    return bonds, counts, np.stack(onsite)


class SampledCorrelationsAdjoint:
    """Loss L(θ, S0) = mean over all complex bins of |data - target|², where data is the
    S(q,ω) of one add_sample! from state S0 with couplings θ; dL/dθ and dL/dS0 by the
    discrete adjoint, with checkpoints every `checkpoint` steps."""

    def __init__(self, sys: System, params, *, measure: MeasureSpec, energies, dt: float, tol: float = 1e-12,
                 max_iters: int = 100):
        if sys.N or sys.precision != "fp64":
            raise ValueError("the adjoint supports FP64 dipole-mode systems")
        if sys.handle is None:
            raise ValueError("the System needs a device")
        self.sys = sys
        self.params = list(params)
        self.measure = measure
        energies = np.asarray(energies, dtype=float)
        nw = len(energies)
        if not (energies[0] == 0 and energies[-1] > 0) or not np.allclose(np.diff(energies), energies[1] - energies[0]):
            raise ValueError("`energies` must be an equally spaced range from 0 to a positive value")
        self.dt, self.measperiod = adjusted_dt_and_downsampling_factor(dt, nw, energies[-1])
        self.n_all_omega = 2 * (nw - 1)
        self.nsteps = self.measperiod * (self.n_all_omega // 2)
        self._lib = sys._lib
        bonds, counts, onsite = unit_coupling_sets(sys, self.params)
        arr = (_abi.BondC * max(1, len(bonds)))()
        for k, b in enumerate(bonds):
            arr[k] = b
        nb = (C.c_int32 * len(counts))(*counts)
        on = np.ascontiguousarray(onsite, dtype=float).reshape(-1)
        obs = np.ascontiguousarray(measure.observables, dtype=float).reshape(-1)
        pairs = np.ascontiguousarray(np.array(measure.corr_pairs, dtype=np.int32) - 1).reshape(-1)
        self._keep = (obs, pairs, arr, nb, on)
        d = _abi.CorrDesc()
        d.nobs = measure.nobs
        d.obs = _abi.dptr(obs)
        d.ncorr = len(measure.corr_pairs)
        d.pairs = pairs.ctypes.data_as(C.POINTER(C.c_int32))
        d.n_all_omega = self.n_all_omega
        d.measperiod = self.measperiod
        d.dt = self.dt
        d.damping = 0.0
        d.tol = tol
        d.max_iters = max_iters
        d.calculate_errors = 0
        sys._sync_to_device()
        h = C.c_void_p()
        self._check(self._lib.sgb_adjoint_create(sys.handle, C.byref(d), len(self.params), arr, nb, _abi.dptr(on),
                                                 C.byref(h)), None)
        self._h = h

    def _check(self, rc, h="self"):
        if rc != _abi.SGB_OK:
            hh = self._h if h == "self" else h
            # before the handle exists the message is the library's process-wide one
            msg = self._lib.sgb_adjoint_last_error(hh) if hh else self._lib.sgb_last_error(None)
            raise _abi.SunnyGPUError(rc, (msg or b"").decode() or f"error {rc}")

    def close(self):
        if getattr(self, "_h", None):
            self._lib.sgb_adjoint_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def shape(self):
        na = self.sys.natoms
        return (len(self.measure.corr_pairs), na, na, *self.sys.dims, self.n_all_omega)

    def set_params(self, theta):
        """Set every parameter's coupling on the System (the couplings the trajectory uses)."""
        theta = np.asarray(theta, dtype=float)
        if theta.shape != (len(self.params),):
            raise ValueError("one value per parameter")
        for f, v in zip(self.params, theta):
            f(self.sys, float(v))
        self.sys._sync_to_device()

    def set_target(self, data):
        data = np.asarray(data, dtype=complex)
        if data.shape != self.shape:
            raise ValueError(f"target must have shape {self.shape}")
        flat = np.ravel(data, order="F")
        buf = np.ascontiguousarray(np.stack([flat.real, flat.imag], -1).reshape(-1))
        self._check(self._lib.sgb_adjoint_set_target(self._h, _abi.dptr(buf)))

    def _data(self, buf):
        z = buf[0::2] + 1j * buf[1::2]
        return z.reshape(self.shape, order="F")

    def loss(self, S0, return_data: bool = False):
        S0 = np.ascontiguousarray(S0, dtype=float).reshape(-1)
        L = C.c_double()
        buf = np.zeros(2 * int(np.prod(self.shape))) if return_data else None
        self.sys._sync_to_device()
        self._check(self._lib.sgb_adjoint_loss(self._h, _abi.dptr(S0), C.byref(L), _abi.dptr(buf)))
        self.sys._dev_newer = True
        return (L.value, self._data(buf)) if return_data else L.value

    def loss_and_grad(self, S0, checkpoint: int = 64, state_grad: bool = False):
        """Returns (loss, dL/dθ) or, with state_grad, (loss, dL/dθ, dL/dS0 [ns][3])."""
        S0 = np.ascontiguousarray(S0, dtype=float).reshape(-1)
        L = C.c_double()
        g = np.zeros(len(self.params))
        gs = np.zeros(S0.size) if state_grad else None
        self.sys._sync_to_device()
        self._check(self._lib.sgb_adjoint_loss_grad(self._h, _abi.dptr(S0), int(checkpoint), C.byref(L), _abi.dptr(g),
                                                    _abi.dptr(gs), None))
        self.sys._dev_newer = True
        if state_grad:
            return L.value, g, gs.reshape(-1, 3)
        return L.value, g
