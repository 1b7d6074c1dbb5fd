"""Crystals, bonds and bond propagation for the host side of the library.

Sunny derives equivalent bonds from a full space-group analysis (src/Symmetry/*, out of
scope here). This module provides the crystals that the hot-path workloads use and
propagates a coupling to its equivalent bonds either with an explicit list of symmetry
operations (when the crystal carries one) or, for isotropic couplings, by distance
shell. Coupling matrices transform as J -> R J R^T and reversed bonds carry J^T
(src/Symmetry/AllowedCouplings.jl:121-123, src/System/PairExchange.jl:228-236).
"""
from __future__ import annotations

import itertools
from dataclasses import dataclass, field

import numpy as np


def lattice_vectors(a, b, c, alpha, beta, gamma) -> np.ndarray:
    """Columns are the lattice vectors (src/Symmetry/LatticeUtils.jl:40-56)."""
    sg, cg = np.sin(np.radians(gamma)), np.cos(np.radians(gamma))
    cb, ca = np.cos(np.radians(beta)), np.cos(np.radians(alpha))
    v1 = [a, 0.0, 0.0]
    v2 = [b * cg, b * sg, 0.0]
    v3 = [c * cb, c / sg * (ca - cb * cg), c / sg * np.sqrt(sg**2 - ca**2 - cb**2 + 2 * ca * cb * cg)]
    return np.array([v1, v2, v3]).T


@dataclass(frozen=True)
class Bond:
    """Sunny's Bond(i, j, n) with 1-based atom indices (src/Symmetry/Bond.jl:1-12)."""
    i: int
    j: int
    n: tuple

    def __init__(self, i, j, n):
        object.__setattr__(self, "i", int(i))
        object.__setattr__(self, "j", int(j))
        object.__setattr__(self, "n", tuple(int(x) for x in n))

    def reverse(self) -> "Bond":
        return Bond(self.j, self.i, tuple(-x for x in self.n))


def bond_parity(b: Bond) -> bool:
    """True for the non-culled copy of a bond (src/System/PairExchange.jl:11-15)."""
    delta = (b.j - b.i, *b.n)
    assert delta != (0, 0, 0, 0)
    return delta > (0, 0, 0, 0)


@dataclass
class Crystal:
    latvecs: np.ndarray
    positions: list
    # optional space-group operations in fractional coordinates: (R (3x3), t (3))
    symops: list | None = None
    types: list | None = None
    _pos: np.ndarray = field(init=False, repr=False)

    def __post_init__(self):
        self.latvecs = np.asarray(self.latvecs, dtype=float)
        self._pos = np.array([np.asarray(p, dtype=float) for p in self.positions])

    @property
    def natoms(self) -> int:
        return len(self._pos)

    @property
    def recipvecs(self) -> np.ndarray:
        return 2 * np.pi * np.linalg.inv(self.latvecs).T

    def position(self, i: int) -> np.ndarray:
        return self._pos[i - 1]

    def displacement(self, b: Bond) -> np.ndarray:
        return self.latvecs @ (self._pos[b.j - 1] + np.array(b.n) - self._pos[b.i - 1])

    def distance(self, b: Bond) -> float:
        return float(np.linalg.norm(self.displacement(b)))

    def locate(self, r: np.ndarray, tol=1e-8):
        """Atom index (1-based) and cell offset of a fractional position."""
        for k, p in enumerate(self._pos):
            d = r - p
            n = np.round(d)
            if np.all(np.abs(d - n) < tol):
                return k + 1, tuple(int(x) for x in n)
        raise ValueError(f"position {r} is not an atom of the crystal")

    def bonds_at_distance(self, dist: float, tol=1e-8):
        """All non-culled bonds of length `dist`."""
        nmax = int(np.ceil(dist / min(np.linalg.norm(self.latvecs, axis=0)))) + 1
        out = []
        for i in range(1, self.natoms + 1):
            for j in range(1, self.natoms + 1):
                for n in itertools.product(range(-nmax, nmax + 1), repeat=3):
                    if i == j and n == (0, 0, 0):
                        continue
                    b = Bond(i, j, n)
                    if abs(self.distance(b) - dist) < tol and bond_parity(b):
                        out.append(b)
        return out

    def equivalent_bonds(self, b: Bond, J: np.ndarray, tol=1e-8):
        """(bond, coupling) for every non-culled bond equivalent to `b`."""
        J = np.asarray(J, dtype=float)
        if self.symops is None:
            if not np.allclose(J, J[0, 0] * np.eye(3), rtol=1e-12, atol=0):
                raise ValueError("anisotropic couplings need a crystal with symmetry operations")
            return [(bb, J.copy()) for bb in self.bonds_at_distance(self.distance(b), tol)]
        found: dict = {}
        Linv = np.linalg.inv(self.latvecs)
        for R, t in self.symops:
            R = np.asarray(R, dtype=float)
            t = np.asarray(t, dtype=float)
            ri = R @ self._pos[b.i - 1] + t
            rj = R @ (self._pos[b.j - 1] + np.array(b.n)) + t
            i2, ni = self.locate(ri, tol)
            j2, nj = self.locate(rj, tol)
            nb = Bond(i2, j2, tuple(np.array(nj) - np.array(ni)))
            Rc = self.latvecs @ R @ Linv
            Jp = Rc @ J @ Rc.T
            if not bond_parity(nb):
                nb, Jp = nb.reverse(), Jp.T
            if nb in found:
                if not np.allclose(found[nb], Jp, atol=1e-10):
                    raise ValueError(f"coupling {J} violates the crystal symmetry on bond {nb}")
            else:
                found[nb] = Jp
        return sorted(found.items(), key=lambda kv: (kv[0].i, kv[0].j, kv[0].n))


def _rotz(k: int, order: int) -> np.ndarray:
    th = 2 * np.pi * k / order
    return np.array([[np.cos(th), -np.sin(th), 0], [np.sin(th), np.cos(th), 0], [0, 0, 1.0]])


def cubic_crystal(a=1.0) -> Crystal:
    """Simple cubic, one atom (src/Symmetry/Crystal.jl:773-777)."""
    return Crystal(lattice_vectors(a, a, a, 90, 90, 90), [[0, 0, 0]])


def bcc_crystal(a=1.0) -> Crystal:
    return Crystal(lattice_vectors(a, a, a, 90, 90, 90), [[0, 0, 0], [0.5, 0.5, 0.5]])


def fcc_primitive_crystal() -> Crystal:
    """FCC with primitive lattice vectors, as used in test_correlation_sampling.jl:5-8."""
    latvecs = np.array([[1, 1, 0], [0, 1, 1], [1, 0, 1]], dtype=float).T / 2
    return Crystal(latvecs, [[0, 0, 0]])


def diamond_crystal(a=1.0) -> Crystal:
    """Diamond, 8 atoms per conventional cell (src/Symmetry/Crystal.jl:796-812)."""
    pos = np.array([[0, 0, 0], [2, 2, 0], [1, 1, 1], [3, 3, 1], [2, 0, 2], [0, 2, 2], [3, 1, 3], [1, 3, 3]]) / 4
    return Crystal(lattice_vectors(a, a, a, 90, 90, 90), [p for p in pos])


def pyrochlore_crystal(a=1.0) -> Crystal:
    """Pyrochlore, 16 atoms per conventional cubic cell: FCC translations of a corner-
    sharing tetrahedron (same site set as src/Symmetry/Crystal.jl:813-816; the atom
    ordering here is this module's own)."""
    fcc = np.array([[0, 0, 0], [0, 0.5, 0.5], [0.5, 0, 0.5], [0.5, 0.5, 0]])
    tet = np.array([[0, 0, 0], [0, 0.25, 0.25], [0.25, 0, 0.25], [0.25, 0.25, 0]])
    pos = [(f + t) % 1.0 for f in fcc for t in tet]
    return Crystal(lattice_vectors(a, a, a, 90, 90, 90), pos)


def triangular_crystal(a=1.0, c=10.0) -> Crystal:
    """Layered triangular lattice with the -3 point group (C3 about z and inversion)
    as explicit operations, enough to propagate an anisotropic J1."""
    latvecs = lattice_vectors(a, a, c, 90, 90, 120)
    Linv = np.linalg.inv(latvecs)
    ops = []
    for k in range(3):
        Rc = _rotz(k, 3)
        for s in (1.0, -1.0):
            R = np.round(Linv @ (s * Rc) @ latvecs)
            ops.append((R, np.zeros(3)))
    return Crystal(latvecs, [[0, 0, 0]], symops=ops)
