"""Spin and Stevens operators, RCS renormalisation, and coherent-state helpers (host side).

Stevens operators follow the polynomial definitions of Rudowicz, J. Phys. C 18, 1415
(1985), in the q = k..-k ordering that Sunny uses (src/Operators/Stevens.jl:12-86);
RCS factors are those of arXiv:2304.03874 (src/System/OnsiteCoupling.jl:46-55).
"""
from __future__ import annotations

import numpy as np


def spin_matrices_of_dim(N: int):
    """(Sx, Sy, Sz) in the eigenbasis of Sz, descending m (src/Operators/Spin.jl:1-14)."""
    s = (N - 1) / 2
    j = np.arange(1, N)
    off = np.sqrt(2 * (s + 1) * j - j * (j + 1)) / 2
    Sx = np.diag(off, 1) + np.diag(off, -1)
    Sy = np.diag(-1j * off, 1) + np.diag(1j * off, -1)
    Sz = np.diag(s - np.arange(N))
    return Sx.astype(complex), Sy.astype(complex), Sz.astype(complex)


def spin_matrices(s: float):
    N = int(round(2 * s + 1))
    if abs(N - (2 * s + 1)) > 1e-12:
        raise ValueError("Spin `s` must be half-integer.")
    return spin_matrices_of_dim(N)


def _stevens_polys(J, k: int):
    Jx, Jy, Jz = J
    N = Jx.shape[0]
    I = np.eye(N, dtype=complex)
    X = Jx @ Jx + Jy @ Jy + Jz @ Jz
    Jp = Jx + 1j * Jy
    Jm = Jx - 1j * Jy
    mp = np.linalg.matrix_power
    A = [0.5 * (mp(Jp, m) + mp(Jm, m)) for m in range(k, 0, -1)] + [I] + \
        [(mp(Jp, m) - mp(Jm, m)) / 2j for m in range(1, k + 1)]
    z = Jz
    if k == 0:
        B = [I]
    elif k == 1:
        B = [z, I]
    elif k == 2:
        B = [3 * mp(z, 2) - X, z, I]
    elif k == 3:
        B = [5 * mp(z, 3) - (3 * X - I) @ z, 5 * mp(z, 2) - X - I / 2, z, I]
    elif k == 4:
        B = [35 * mp(z, 4) - (30 * X - 25 * I) @ mp(z, 2) + (3 * X @ X - 6 * X),
             7 * mp(z, 3) - (3 * X + I) @ z, 7 * mp(z, 2) - (X + 5 * I), z, I]
    elif k == 5:
        B = [63 * mp(z, 5) - (70 * X - 105 * I) @ mp(z, 3) + (15 * X @ X - 50 * X + 12 * I) @ z,
             21 * mp(z, 4) - 14 * X @ mp(z, 2) + (X @ X - X + 1.5 * I),
             3 * mp(z, 3) - (X + 6 * I) @ z, 9 * mp(z, 2) - (X + 16.5 * I), z, I]
    elif k == 6:
        B = [231 * mp(z, 6) - (315 * X - 735 * I) @ mp(z, 4) + (105 * X @ X - 525 * X + 294 * I) @ mp(z, 2)
             - (5 * X @ X @ X - 40 * X @ X + 60 * X),
             33 * mp(z, 5) - (30 * X - 15 * I) @ mp(z, 3) + (5 * X @ X - 10 * X + 12 * I) @ z,
             33 * mp(z, 4) - (18 * X + 123 * I) @ mp(z, 2) + (X @ X + 10 * X + 102 * I),
             11 * mp(z, 3) - (3 * X + 59 * I) @ z, 11 * mp(z, 2) - (X + 38 * I), z, I]
    else:
        raise ValueError(f"Stevens operators for k > 6 are unsupported, received k={k}")
    B = list(reversed(B)) + B[1:]
    return [(a @ b + b @ a) / 2 for a, b in zip(A, B)]


def stevens_matrices_of_dim(k: int, N: int):
    """O[k, q] for q = k..-k as N x N matrices (zero if k >= N)."""
    if k >= N:
        return [np.zeros((N, N), dtype=complex) for _ in range(2 * k + 1)]
    return _stevens_polys(spin_matrices_of_dim(N), k)


def matrix_to_stevens_coefficients(A: np.ndarray):
    """Coefficients c[k] (k = 0..6, q descending) of a Hermitian matrix
    (src/Operators/Stevens.jl:144-159)."""
    N = A.shape[0]
    out = []
    for k in range(7):
        if k >= N:
            out.append(np.zeros(2 * k + 1))
            continue
        cs = []
        for O in stevens_matrices_of_dim(k, N):
            c = np.trace(O.conj().T @ A) / np.trace(O.conj().T @ O)
            assert abs(c.imag) < 1e-12
            cs.append(0.0 if abs(c) < 1e-12 else c.real)
        out.append(np.array(cs))
    return out


def rcs_factors(s: float) -> np.ndarray:
    """lambda_k, k = 0..6 (src/System/OnsiteCoupling.jl:46-55)."""
    return np.array([
        1.0,
        1.0,
        1 - (1 / 2) / s,
        1 - (3 / 2) / s + (1 / 2) / s**2,
        1 - 3 / s + (11 / 4) / s**2 - (3 / 4) / s**3,
        1 - 5 / s + (35 / 4) / s**2 - (25 / 4) / s**3 + (3 / 2) / s**4,
        1 - (15 / 2) / s + (85 / 4) / s**2 - (225 / 8) / s**3 + (137 / 8) / s**4 - (15 / 4) / s**5,
    ])


def stevens_expansion_for_dipole(A: np.ndarray, s: float, renormalize: bool = True) -> np.ndarray:
    """28 coefficients c0, c2[5], c4[9], c6[13] for :dipole mode (OnsiteCoupling.jl:16-19)."""
    c = matrix_to_stevens_coefficients(A)
    for k in (1, 3, 5):
        if np.any(c[k] != 0):
            raise ValueError("Single-ion anisotropy must be time-reversal invariant.")
    lam = rcs_factors(s) if renormalize else np.ones(7)
    return np.concatenate([lam[0] * c[0], lam[2] * c[2], lam[4] * c[4], lam[6] * c[6]])


def expected_spin(Z: np.ndarray) -> np.ndarray:
    """<Z|S|Z> for an array of kets (..., N) (src/Operators/Spin.jl:72-87)."""
    N = Z.shape[-1]
    Sx, Sy, Sz = spin_matrices_of_dim(N)
    return np.stack([np.einsum("...i,ij,...j->...", Z.conj(), S, Z).real for S in (Sx, Sy, Sz)], axis=-1)


def ket_from_dipole(d: np.ndarray, N: int) -> np.ndarray:
    """Ket with maximal projection on `d` (src/Operators/Spin.jl:112-116)."""
    S = spin_matrices_of_dim(N)
    H = d[0] * S[0] + d[1] * S[1] + d[2] * S[2]
    w, v = np.linalg.eigh(H)
    return v[:, np.argmax(w)]


def hermitian_basis(N: int) -> np.ndarray:
    """An orthonormal basis of the N x N Hermitian matrices under Tr(X^† Y): the identity
    over √N, then the generalized Gell-Mann matrices (symmetric, antisymmetric and diagonal
    generators), shape (N², N, N)."""
    out = [np.eye(N, dtype=complex) / np.sqrt(N)]
    for r in range(N):
        for c in range(r + 1, N):
            E = np.zeros((N, N), dtype=complex)
            E[r, c] = E[c, r] = 1 / np.sqrt(2)
            out.append(E)
            E = np.zeros((N, N), dtype=complex)
            E[r, c] = -1j / np.sqrt(2)
            E[c, r] = 1j / np.sqrt(2)
            out.append(E)
    for k in range(1, N):
        d = np.zeros(N)
        d[:k] = 1.0
        d[k] = -k
        out.append(np.diag(d / np.sqrt(k * (k + 1))).astype(complex))
    return np.array(out)


def tensor_decomposition(op, N1: int, N2: int, tol: float = 1e-12):
    """Σ_k A_k ⊗ B_k with Hermitian A_k (N1 x N1) and B_k (N2 x N2) equal to the Hermitian
    operator `op` on C^N1 ⊗ C^N2 (the form of Sunny's TensorDecomposition, Types.jl:23-30).
    Its coefficients in products of orthonormal Hermitian bases form a real matrix whose
    singular value decomposition gives the pairs (an operator Schmidt decomposition)."""
    op = np.asarray(op, dtype=complex)
    if op.shape != (N1 * N2, N1 * N2):
        raise ValueError("Invalid matrix size.")
    if not np.allclose(op, op.conj().T):
        raise ValueError("Operator is not Hermitian")
    T1, T2 = hermitian_basis(N1), hermitian_basis(N2)
    coef = np.array([[np.trace(np.kron(a, b) @ op).real for b in T2] for a in T1])
    U, sv, Vt = np.linalg.svd(coef)
    pairs = []
    for k in range(len(sv)):
        if sv[k] <= tol * max(sv[0], 1e-300):
            continue
        w = np.sqrt(sv[k])
        A = w * np.tensordot(U[:, k], T1, axes=1)
        B = w * np.tensordot(Vt[k], T2, axes=1)
        pairs.append(((A + A.conj().T) / 2, (B + B.conj().T) / 2))
    return pairs
