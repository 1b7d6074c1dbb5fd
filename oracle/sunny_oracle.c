/*
 * sunny_oracle.c -- TEST INFRASTRUCTURE ONLY (see sunny_oracle.h). FP64 CPU restatement
 * of Sunny.jl v0.9.2 (src/...) for parity checks. Each function cites the reference
 * lines it follows. It is deliberately plain and sequential: it mirrors the reference's
 * scatter loops over non-culled bonds and its per-sublattice site ordering.
 */
#include "sunny_oracle.h"
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex cplx;

/* Types.jl:40 scalar_biquad_metric */
static const double METRIC[5] = {0.5, 2.0, 1.0 / 6.0, 2.0, 0.5};

int64_t or_nsites(const or_sys* s) { return (int64_t)s->L[0] * s->L[1] * s->L[2] * s->na; }

static inline int64_t site_index(const or_sys* s, int c1, int c2, int c3, int a) {
    return c1 + (int64_t)s->L[0] * (c2 + (int64_t)s->L[1] * (c3 + (int64_t)s->L[2] * a));
}

/* System.jl:204-212 altmod1 / bonded_site, 0-based */
static inline int wrap(int x, int L) {
    if (0 <= x && x < L) return x;
    int r = x % L;
    return r < 0 ? r + L : r;
}

static inline void cross3(const double* a, const double* b, double* out) {
    out[0] = a[1] * b[2] - a[2] * b[1];
    out[1] = a[2] * b[0] - a[0] * b[2];
    out[2] = a[0] * b[1] - a[1] * b[0];
}

/* Onsite coupling of site i: its own (inhomogeneous systems) or its sublattice's. */
static const double* onsite_at(const or_sys* s, int64_t i) {
    const int64_t ncell = (int64_t)s->L[0] * s->L[1] * s->L[2];
    const int64_t per = s->mode == SGB_MODE_SUN ? 2 * (int64_t)s->N * s->N : 28;
    if (s->onsite_site) return s->onsite_site + per * i;
    if (s->onsite) return s->onsite + per * (i / ncell);
    return NULL;
}

/* The two sites of an inhomogeneous coupling: (cell, bond.i) and
 * bonded_site((cell, bond.i), bond) (System.jl:204-212). */
static void site_bond_ends(const or_sys* s, const sgb_site_bond* e, int64_t* i, int64_t* j) {
    const sgb_bond* b = &e->bond;
    *i = site_index(s, e->cell[0], e->cell[1], e->cell[2], b->i);
    *j = site_index(s, wrap(e->cell[0] + b->n[0], s->L[0]), wrap(e->cell[1] + b->n[1], s->L[1]),
                    wrap(e->cell[2] + b->n[2], s->L[2]), b->j);
}

/* System.jl:421-423 normalize_dipole: κ*normalize(s) */
static inline void normalize_dipole(const double* v, double kappa, double* out) {
    if (kappa == 0.0) { out[0] = out[1] = out[2] = 0.0; return; }
    double n = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    out[0] = kappa * (v[0] / n);
    out[1] = kappa * (v[1] / n);
    out[2] = kappa * (v[2] / n);
}

/* Spin.jl:48-57 quadrupole */
static void quadrupole(const double* S, double* Q) {
    double x = S[0], y = S[1], z = S[2];
    Q[0] = x * x - y * y;
    Q[1] = z * x;
    Q[2] = -x * x - y * y + 2 * z * z;
    Q[3] = z * y;
    Q[4] = 2 * y * x;
}
/* Spin.jl:60-69 grad_quadrupole: dQ[q][component] */
static void grad_quadrupole(const double* S, double dQ[5][3]) {
    double x = S[0], y = S[1], z = S[2];
    dQ[0][0] = 2 * x;  dQ[0][1] = -2 * y; dQ[0][2] = 0;
    dQ[1][0] = z;      dQ[1][1] = 0;      dQ[1][2] = x;
    dQ[2][0] = -2 * x; dQ[2][1] = -2 * y; dQ[2][2] = 4 * z;
    dQ[3][0] = 0;      dQ[3][1] = z;      dQ[3][2] = y;
    dQ[4][0] = 2 * y;  dQ[4][1] = 2 * x;  dQ[4][2] = 0;
}

/* ---- spin and Stevens quadrupole matrices of dimension N (Spin.jl:1-14, Stevens.jl:12-86) */
typedef struct {
    int N;
    cplx Sm[3][8 * 8];   /* spin matrices, col-major, N <= 8 */
    cplx Q[5][8 * 8];    /* Stevens O[2,q], q = 2..-2 */
} or_ops;

static void mat_mul(int N, const cplx* A, const cplx* B, cplx* C) {
    for (int c = 0; c < N; c++)
        for (int r = 0; r < N; r++) {
            cplx acc = 0;
            for (int k = 0; k < N; k++) acc += A[r + N * k] * B[k + N * c];
            C[r + N * c] = acc;
        }
}

static void build_ops(int N, or_ops* ops) {
    memset(ops, 0, sizeof(*ops));
    ops->N = N;
    double s = (N - 1) / 2.0;
    for (int j = 1; j <= N - 1; j++) {
        double off = sqrt(2 * (s + 1) * j - (double)j * (j + 1)) / 2;
        /* Sx: superdiag and subdiag = off; Sy: superdiag -i off, subdiag +i off */
        int r = j - 1, c = j;       /* (r, c) = (j, j+1) in 1-based */
        ops->Sm[0][r + N * c] = off;
        ops->Sm[0][c + N * r] = off;
        ops->Sm[1][r + N * c] = -I * off;
        ops->Sm[1][c + N * r] = I * off;
    }
    for (int k = 0; k < N; k++) ops->Sm[2][k + N * k] = s - k;
    if (N <= 2) return; /* stevens_matrices_of_dim(2; N) is zero for k >= N */
    cplx Jp[64], Jm[64], Jp2[64], Jm2[64], Jz2[64], A[64], AJ[64], JA[64];
    for (int i = 0; i < N * N; i++) {
        Jp[i] = ops->Sm[0][i] + I * ops->Sm[1][i];
        Jm[i] = ops->Sm[0][i] - I * ops->Sm[1][i];
    }
    mat_mul(N, Jp, Jp, Jp2);
    mat_mul(N, Jm, Jm, Jm2);
    mat_mul(N, ops->Sm[2], ops->Sm[2], Jz2);
    cplx X[64];
    {
        cplx t[64];
        memset(X, 0, sizeof(X));
        for (int a = 0; a < 3; a++) {
            mat_mul(N, ops->Sm[a], ops->Sm[a], t);
            for (int i = 0; i < N * N; i++) X[i] += t[i];
        }
    }
    /* q = 2: (1/2)(Jp^2 + Jm^2) * I */
    for (int i = 0; i < N * N; i++) ops->Q[0][i] = 0.5 * (Jp2[i] + Jm2[i]);
    /* q = 1: A = (1/2)(Jp + Jm), B = Jz, O = (AB + BA)/2 */
    for (int i = 0; i < N * N; i++) A[i] = 0.5 * (Jp[i] + Jm[i]);
    mat_mul(N, A, ops->Sm[2], AJ);
    mat_mul(N, ops->Sm[2], A, JA);
    for (int i = 0; i < N * N; i++) ops->Q[1][i] = 0.5 * (AJ[i] + JA[i]);
    /* q = 0: 3Jz^2 - X */
    for (int i = 0; i < N * N; i++) ops->Q[2][i] = 3 * Jz2[i] - X[i];
    /* q = -1: A = (1/2i)(Jp - Jm), B = Jz */
    for (int i = 0; i < N * N; i++) A[i] = (Jp[i] - Jm[i]) / (2.0 * I);
    mat_mul(N, A, ops->Sm[2], AJ);
    mat_mul(N, ops->Sm[2], A, JA);
    for (int i = 0; i < N * N; i++) ops->Q[3][i] = 0.5 * (AJ[i] + JA[i]);
    /* q = -2: (1/2i)(Jp^2 - Jm^2) */
    for (int i = 0; i < N * N; i++) ops->Q[4][i] = (Jp2[i] - Jm2[i]) / (2.0 * I);
}

static inline cplx zget(const double* Z, int64_t site, int N, int k) {
    return Z[2 * (site * N + k)] + I * Z[2 * (site * N + k) + 1];
}
static inline void zset(double* Z, int64_t site, int N, int k, cplx v) {
    Z[2 * (site * N + k)] = creal(v);
    Z[2 * (site * N + k) + 1] = cimag(v);
}

/* Spin.jl:72-87 expected_spin */
void or_expected_spin(int N, const double* Zs, double* S3) {
    double s = (N - 1) / 2.0;
    cplx c = 0;
    double nz = 0;
    for (int j = 1; j <= N - 1; j++) {
        double off = sqrt(2 * (s + 1) * j - (double)j * (j + 1)) / 2;
        cplx zl = Zs[2 * (j - 1)] + I * Zs[2 * (j - 1) + 1];
        cplx zh = Zs[2 * j] + I * Zs[2 * j + 1];
        c += conj(zl) * (off * zh);
    }
    for (int k = 0; k < N; k++) {
        cplx z = Zs[2 * k] + I * Zs[2 * k + 1];
        nz += creal(conj(z) * ((s - k) * z));
    }
    S3[0] = 2 * creal(c);
    S3[1] = 2 * cimag(c);
    S3[2] = nz;
}

/* Spin.jl:90-104 expected_quadrupole */
static void expected_quadrupole(const or_ops* ops, const cplx* z, double* Q) {
    int N = ops->N;
    for (int a = 0; a < 5; a++) {
        cplx acc = 0;
        for (int c = 0; c < N; c++)
            for (int r = 0; r < N; r++) acc += conj(z[r]) * ops->Q[a][r + N * c] * z[c];
        Q[a] = creal(acc);
    }
}

/* <Z|M|Z> and M Z for an N x N complex matrix M, column-major (re, im). */
static double expect_op(int N, const double* Mx, const cplx* z) {
    cplx acc = 0;
    for (int c = 0; c < N; c++)
        for (int r = 0; r < N; r++) acc += conj(z[r]) * (Mx[2 * (r + N * c)] + I * Mx[2 * (r + N * c) + 1]) * z[c];
    return creal(acc);
}
static void apply_op(int N, const double* Mx, const cplx* z, cplx* out) {
    for (int r = 0; r < N; r++) {
        cplx acc = 0;
        for (int c = 0; c < N; c++) acc += (Mx[2 * (r + N * c)] + I * Mx[2 * (r + N * c) + 1]) * z[c];
        out[r] = acc;
    }
}

/* ---- OnsiteCoupling.jl:316-425 energy_and_gradient_for_classical_anisotropy --------- */
static int stevens_kmax(const double* c) {
    int k2 = 0, k4 = 0, k6 = 0;
    for (int i = 0; i < 5; i++) k2 |= c[1 + i] != 0.0;
    for (int i = 0; i < 9; i++) k4 |= c[6 + i] != 0.0;
    for (int i = 0; i < 13; i++) k6 |= c[15 + i] != 0.0;
    return k6 ? 6 : k4 ? 4 : k2 ? 2 : 0;
}

double or_classical_anisotropy(const double* cc, const double* S, double* grad3) {
    const double* c2 = cc + 1;  /* 5  */
    const double* c4 = cc + 6;  /* 9  */
    const double* c6 = cc + 15; /* 13 */
    int kmax = stevens_kmax(cc);
    double E = cc[0], dE_dz = 0.0;
    cplx dE_dJp = 0.0;
    if (kmax >= 2) {
        double X = S[0] * S[0] + S[1] * S[1] + S[2] * S[2];
        cplx Jp1 = S[0] + I * S[1];
        double Jz1 = S[2];
        cplx Jp2 = Jp1 * Jp1;
        double Jz2 = Jz1 * Jz1;
        double A[3] = {3 * Jz2 - X, Jz1, 1};
        double dA[2] = {6 * Jz1, 1};
        E += (c2[0] * creal(Jp2) + c2[4] * cimag(Jp2)) * A[2] +
             (c2[1] * creal(Jp1) + c2[3] * cimag(Jp1)) * A[1] + c2[2] * A[0];
        dE_dz += (c2[1] * creal(Jp1) + c2[3] * cimag(Jp1)) * dA[1] + c2[2] * dA[0];
        dE_dJp += (2.0 / 2) * (c2[0] * Jp1 - I * c2[4] * Jp1) * A[2] +
                  (1.0 / 2) * (c2[1] - I * c2[3]) * A[1];
        if (kmax >= 4) {
            double X2 = X * X;
            cplx Jp3 = Jp2 * Jp1, Jp4 = Jp2 * Jp2;
            double Jz3 = Jz2 * Jz1, Jz4 = Jz2 * Jz2;
            double B[5] = {35 * Jz4 - (30 * X) * Jz2 + (3 * X2), 7 * Jz3 - (3 * X) * Jz1,
                           7 * Jz2 - (X), Jz1, 1};
            double dB[4] = {140 * Jz3 - (60 * X) * Jz1, 21 * Jz2 - 3 * X, 14 * Jz1, 1};
            E += (c4[0] * creal(Jp4) + c4[8] * cimag(Jp4)) * B[4] +
                 (c4[1] * creal(Jp3) + c4[7] * cimag(Jp3)) * B[3] +
                 (c4[2] * creal(Jp2) + c4[6] * cimag(Jp2)) * B[2] +
                 (c4[3] * creal(Jp1) + c4[5] * cimag(Jp1)) * B[1] + c4[4] * B[0];
            dE_dz += (c4[1] * creal(Jp3) + c4[7] * cimag(Jp3)) * dB[3] +
                     (c4[2] * creal(Jp2) + c4[6] * cimag(Jp2)) * dB[2] +
                     (c4[3] * creal(Jp1) + c4[5] * cimag(Jp1)) * dB[1] + c4[4] * dB[0];
            dE_dJp += (4.0 / 2) * (c4[0] * Jp3 - I * c4[8] * Jp3) * B[4] +
                      (3.0 / 2) * (c4[1] * Jp2 - I * c4[7] * Jp2) * B[3] +
                      (2.0 / 2) * (c4[2] * Jp1 - I * c4[6] * Jp1) * B[2] +
                      (1.0 / 2) * (c4[3] - I * c4[5]) * B[1];
            if (kmax >= 6) {
                double X3 = X2 * X;
                cplx Jp5 = Jp4 * Jp1, Jp6 = Jp3 * Jp3;
                double Jz5 = Jz4 * Jz1, Jz6 = Jz3 * Jz3;
                double C[7] = {231 * Jz6 - (315 * X) * Jz4 + (105 * X2) * Jz2 - (5 * X3),
                               33 * Jz5 - (30 * X) * Jz3 + (5 * X2) * Jz1,
                               33 * Jz4 - (18 * X) * Jz2 + (X2),
                               11 * Jz3 - (3 * X) * Jz1,
                               11 * Jz2 - (X),
                               Jz1,
                               1};
                double dC[6] = {1386 * Jz5 - (1260 * X) * Jz3 + (210 * X2) * Jz1,
                                165 * Jz4 - (90 * X) * Jz2 + 5 * X2,
                                132 * Jz3 - (36 * X) * Jz1,
                                33 * Jz2 - 3 * X,
                                22 * Jz1,
                                1};
                E += (c6[0] * creal(Jp6) + c6[12] * cimag(Jp6)) * C[6] +
                     (c6[1] * creal(Jp5) + c6[11] * cimag(Jp5)) * C[5] +
                     (c6[2] * creal(Jp4) + c6[10] * cimag(Jp4)) * C[4] +
                     (c6[3] * creal(Jp3) + c6[9] * cimag(Jp3)) * C[3] +
                     (c6[4] * creal(Jp2) + c6[8] * cimag(Jp2)) * C[2] +
                     (c6[5] * creal(Jp1) + c6[7] * cimag(Jp1)) * C[1] + c6[6] * C[0];
                dE_dz += (c6[1] * creal(Jp5) + c6[11] * cimag(Jp5)) * dC[5] +
                         (c6[2] * creal(Jp4) + c6[10] * cimag(Jp4)) * dC[4] +
                         (c6[3] * creal(Jp3) + c6[9] * cimag(Jp3)) * dC[3] +
                         (c6[4] * creal(Jp2) + c6[8] * cimag(Jp2)) * dC[2] +
                         (c6[5] * creal(Jp1) + c6[7] * cimag(Jp1)) * dC[1] + c6[6] * dC[0];
                dE_dJp += (6.0 / 2) * (c6[0] * Jp5 - I * c6[12] * Jp5) * C[6] +
                          (5.0 / 2) * (c6[1] * Jp4 - I * c6[11] * Jp4) * C[5] +
                          (4.0 / 2) * (c6[2] * Jp3 - I * c6[10] * Jp3) * C[4] +
                          (3.0 / 2) * (c6[3] * Jp2 - I * c6[9] * Jp2) * C[3] +
                          (2.0 / 2) * (c6[4] * Jp1 - I * c6[8] * Jp1) * C[2] +
                          (1.0 / 2) * (c6[5] - I * c6[7]) * C[1];
            }
        }
    }
    grad3[0] = +2 * creal(dE_dJp);
    grad3[1] = -2 * cimag(dE_dJp);
    grad3[2] = dE_dz;
    return E;
}

/* ---- Interactions.jl:516-592 set_energy_grad_dipoles! ------------------------------ */
/* One non-culled coupling pc between sites i and j = bonded_site(i, pc.bond), scattered
 * into both ends (Interactions.jl:554-591). */
static void pair_grad_dipoles(const sgb_bond* pc, int64_t i, int64_t j, const double* S, double* grad, int dipole_mode) {
    const double* J = pc->bilin;
    const double* Si = S + 3 * i;
    const double* Sj = S + 3 * j;
    for (int r = 0; r < 3; r++) {
        grad[3 * i + r] += J[r + 0] * Sj[0] + J[r + 3] * Sj[1] + J[r + 6] * Sj[2];
    }
    for (int r = 0; r < 3; r++) {
        grad[3 * j + r] += J[0 + 3 * r] * Si[0] + J[1 + 3 * r] * Si[1] + J[2 + 3 * r] * Si[2];
    }
    if (dipole_mode && pc->biquad_kind != 0) {
        double Qi[5], Qj[5], dQi[5][3], dQj[5][3];
        quadrupole(Si, Qi);
        quadrupole(Sj, Qj);
        grad_quadrupole(Si, dQi);
        grad_quadrupole(Sj, dQj);
        double vi[5], vj[5];
        if (pc->biquad_kind == 1) {
            double Jb = pc->biquad[0];
            for (int q = 0; q < 5; q++) { vi[q] = Jb * (Qj[q] * METRIC[q]); vj[q] = Jb * (Qi[q] * METRIC[q]); }
        } else {
            const double* B = pc->biquad;
            for (int q = 0; q < 5; q++) {
                double acc_i = 0, acc_j = 0;
                for (int p = 0; p < 5; p++) {
                    acc_i += B[q + 5 * p] * Qj[p];   /* (J Qj)_q */
                    acc_j += Qi[p] * B[p + 5 * q];   /* (Qi' J)_q */
                }
                vi[q] = acc_i; vj[q] = acc_j;
            }
        }
        for (int r = 0; r < 3; r++) {
            double ai = 0, aj = 0;
            for (int q = 0; q < 5; q++) { ai += vi[q] * dQi[q][r]; aj += vj[q] * dQj[q][r]; }
            grad[3 * i + r] += ai;
            grad[3 * j + r] += aj;
        }
    }
}

void or_grad_dipoles(const or_sys* s, const double* S, double* grad) {
    int64_t ns = or_nsites(s);
    int L1 = s->L[0], L2 = s->L[1], L3 = s->L[2];
    memset(grad, 0, sizeof(double) * 3 * ns);
    /* Zeeman: ∇E += g' * B (Interactions.jl:520-523) */
    if (s->field) {
        for (int64_t i = 0; i < ns; i++) {
            const double* g = s->g + 9 * i;
            const double* B = s->field + 3 * i;
            for (int r = 0; r < 3; r++)
                grad[3 * i + r] += g[0 + 3 * r] * B[0] + g[1 + 3 * r] * B[1] + g[2 + 3 * r] * B[2];
        }
    }
    int dipole_mode = (s->mode != SGB_MODE_SUN);
    if (s->site_bonds || s->onsite_site) {
        /* inhomogeneous: per site, its onsite term then its own non-culled couplings
         * (Interactions.jl:535-540 with sites = (site,)) */
        if (dipole_mode)
            for (int64_t i = 0; i < ns; i++) {
                const double* c = onsite_at(s, i);
                if (!c) continue;
                double g3[3];
                or_classical_anisotropy(c, S + 3 * i, g3);
                grad[3 * i] += g3[0]; grad[3 * i + 1] += g3[1]; grad[3 * i + 2] += g3[2];
            }
        if (s->site_bonds) {
            for (int64_t e = 0; e < s->nsite_bonds; e++) {
                int64_t i, j;
                site_bond_ends(s, &s->site_bonds[e], &i, &j);
                pair_grad_dipoles(&s->site_bonds[e].bond, i, j, S, grad, dipole_mode);
            }
            return;
        }
    }
    for (int a = 0; a < s->na; a++) {
        /* onsite (dipole modes only), Interactions.jl:546-552 */
        if (dipole_mode && s->onsite && !s->onsite_site) {
            for (int c3 = 0; c3 < L3; c3++)
                for (int c2 = 0; c2 < L2; c2++)
                    for (int c1 = 0; c1 < L1; c1++) {
                        int64_t i = site_index(s, c1, c2, c3, a);
                        double g3[3];
                        or_classical_anisotropy(s->onsite + 28 * a, S + 3 * i, g3);
                        grad[3 * i] += g3[0]; grad[3 * i + 1] += g3[1]; grad[3 * i + 2] += g3[2];
                    }
        }
        /* pairs (Interactions.jl:554-591), non-culled bonds of sublattice a in order */
        for (int b = 0; b < s->nbonds; b++) {
            const sgb_bond* pc = &s->bonds[b];
            if (pc->i != a) continue;
            for (int c3 = 0; c3 < L3; c3++)
                for (int c2 = 0; c2 < L2; c2++)
                    for (int c1 = 0; c1 < L1; c1++) {
                        int64_t i = site_index(s, c1, c2, c3, a);
                        int64_t j = site_index(s, wrap(c1 + pc->n[0], L1), wrap(c2 + pc->n[1], L2),
                                               wrap(c3 + pc->n[2], L3), pc->j);
                        pair_grad_dipoles(pc, i, j, S, grad, dipole_mode);
                    }
        }
    }
}

/* Spin.jl:132-148 mul_spin_matrices: (Λ + dE/dS·S) Z */
static void mul_spin_matrices(const or_ops* ops, const double* lam, const double* dEdS, const cplx* z, cplx* out) {
    int N = ops->N;
    for (int r = 0; r < N; r++) {
        cplx acc = 0;
        for (int c = 0; c < N; c++) {
            cplx h = lam ? (lam[2 * (r + N * c)] + I * lam[2 * (r + N * c) + 1]) : 0;
            for (int a = 0; a < 3; a++) h += dEdS[a] * ops->Sm[a][r + N * c];
            acc += h * z[c];
        }
        out[r] = acc;
    }
}
/* Spin.jl:151-167 mul_quadrupole_matrices */
static void mul_quadrupole_matrices(const or_ops* ops, const double* dEdQ, const cplx* z, cplx* out) {
    int N = ops->N;
    for (int r = 0; r < N; r++) {
        cplx acc = 0;
        for (int c = 0; c < N; c++) {
            cplx h = 0;
            for (int a = 0; a < 5; a++) h += dEdQ[a] * ops->Q[a][r + N * c];
            acc += h * z[c];
        }
        out[r] = acc;
    }
}

/* ---- Interactions.jl:596-669 set_energy_grad_coherents! ----------------------------- */
/* Biquadratic coupling pc between sites i and j in SU(N) mode (Interactions.jl:643-658). */
static void pair_grad_coherents(const or_ops* ops, const sgb_bond* pc, int64_t i, int64_t j, const double* Z, double* HZ) {
    const int N = ops->N;
    cplx zi[8], zj[8], oi[8], oj[8];
    for (int k = 0; k < N; k++) { zi[k] = zget(Z, i, N, k); zj[k] = zget(Z, j, N, k); }
    double Qi[5], Qj[5], dQi[5], dQj[5];
    expected_quadrupole(ops, zi, Qi);
    expected_quadrupole(ops, zj, Qj);
    if (pc->biquad_kind == 1) {
        for (int q = 0; q < 5; q++) { dQi[q] = pc->biquad[0] * (METRIC[q] * Qj[q]); dQj[q] = pc->biquad[0] * (METRIC[q] * Qi[q]); }
    } else {
        const double* B = pc->biquad;
        for (int q = 0; q < 5; q++) {
            double ai = 0, aj = 0;
            for (int p = 0; p < 5; p++) { ai += B[q + 5 * p] * Qj[p]; aj += B[p + 5 * q] * Qi[p]; }
            dQi[q] = ai; dQj[q] = aj;
        }
    }
    mul_quadrupole_matrices(ops, dQi, zi, oi);
    mul_quadrupole_matrices(ops, dQj, zj, oj);
    for (int k = 0; k < N; k++) {
        zset(HZ, i, N, k, zget(HZ, i, N, k) + oi[k]);
        zset(HZ, j, N, k, zget(HZ, j, N, k) + oj[k]);
    }
}

void or_grad_coherents(const or_sys* s, const double* Z, double* HZ) {
    int N = s->N;
    int64_t ns = or_nsites(s);
    int L1 = s->L[0], L2 = s->L[1], L3 = s->L[2];
    or_ops ops;
    build_ops(N, &ops);
    double* dip = malloc(sizeof(double) * 3 * ns);
    double* dEdS = malloc(sizeof(double) * 3 * ns);
    for (int64_t i = 0; i < ns; i++) or_expected_spin(N, Z + 2 * N * i, dip + 3 * i);
    or_grad_dipoles(s, dip, dEdS); /* SU(N) mode: Zeeman + bilinear only */
    memset(HZ, 0, sizeof(double) * 2 * N * ns);
    /* (Λ + dE/dS·S) Z per site (Interactions.jl:605-630) */
    for (int64_t i = 0; i < ns; i++) {
        cplx z[8], out[8];
        for (int k = 0; k < N; k++) z[k] = zget(Z, i, N, k);
        mul_spin_matrices(&ops, onsite_at(s, i), dEdS + 3 * i, z, out);
        for (int k = 0; k < N; k++) zset(HZ, i, N, k, zget(HZ, i, N, k) + out[k]);
    }
    if (s->site_bonds) {
        for (int64_t e = 0; e < s->nsite_bonds; e++) {
            const sgb_bond* pc = &s->site_bonds[e].bond;
            if (pc->biquad_kind == 0) continue;
            int64_t i, j;
            site_bond_ends(s, &s->site_bonds[e], &i, &j);
            pair_grad_coherents(&ops, pc, i, j, Z, HZ);
        }
    } else {
        for (int a = 0; a < s->na; a++)
            for (int b = 0; b < s->nbonds; b++) {
                const sgb_bond* pc = &s->bonds[b];
                if (pc->i != a || pc->biquad_kind == 0) continue;
                for (int c3 = 0; c3 < L3; c3++)
                    for (int c2 = 0; c2 < L2; c2++)
                        for (int c1 = 0; c1 < L1; c1++) {
                            int64_t i = site_index(s, c1, c2, c3, a);
                            int64_t j = site_index(s, wrap(c1 + pc->n[0], L1), wrap(c2 + pc->n[1], L2),
                                                   wrap(c3 + pc->n[2], L3), pc->j);
                            pair_grad_coherents(&ops, pc, i, j, Z, HZ);
                        }
            }
        /* general couplings (Interactions.jl:660-666): HZ_i += <B>_j A Z_i, HZ_j += <A>_i B Z_j */
        for (int t = 0; t < s->ngen; t++) {
            const sgb_bond* pc = &s->bonds[s->gen_bond[t]];
            const double* A = s->gen_A + (size_t)2 * N * N * t;
            const double* B = s->gen_B + (size_t)2 * N * N * t;
            for (int c3 = 0; c3 < L3; c3++)
                for (int c2 = 0; c2 < L2; c2++)
                    for (int c1 = 0; c1 < L1; c1++) {
                        int64_t i = site_index(s, c1, c2, c3, pc->i);
                        int64_t j = site_index(s, wrap(c1 + pc->n[0], L1), wrap(c2 + pc->n[1], L2),
                                               wrap(c3 + pc->n[2], L3), pc->j);
                        cplx zi[8], zj[8], ai[8], bj[8];
                        for (int k = 0; k < N; k++) { zi[k] = zget(Z, i, N, k); zj[k] = zget(Z, j, N, k); }
                        const double Ab = expect_op(N, A, zi), Bb = expect_op(N, B, zj);
                        apply_op(N, A, zi, ai);
                        apply_op(N, B, zj, bj);
                        for (int k = 0; k < N; k++) {
                            zset(HZ, i, N, k, zget(HZ, i, N, k) + ai[k] * Bb);
                            zset(HZ, j, N, k, zget(HZ, j, N, k) + bj[k] * Ab);
                        }
                    }
        }
    }
    free(dip);
    free(dEdS);
}

/* ---- Interactions.jl:401-508 energy ------------------------------------------------- */
/* Energy of one non-culled coupling between sites i and j (Interactions.jl:466-505). */
static double pair_energy(const or_sys* s, const or_ops* ops, const sgb_bond* pc, int64_t i, int64_t j, const double* S,
                          const double* Z, int sun) {
    const int N = s->N;
    const double* J = pc->bilin;
    const double* Si = S + 3 * i;
    const double* Sj = S + 3 * j;
    double Ea = 0;
    if (sun) Ea += pc->scalar * s->kappa[i] * s->kappa[j];
    else Ea += pc->scalar;
    double JS[3];
    for (int r = 0; r < 3; r++) JS[r] = J[r] * Sj[0] + J[r + 3] * Sj[1] + J[r + 6] * Sj[2];
    Ea += Si[0] * JS[0] + Si[1] * JS[1] + Si[2] * JS[2];
    if (pc->biquad_kind != 0) {
        double Qi[5], Qj[5];
        if (!sun) { quadrupole(Si, Qi); quadrupole(Sj, Qj); }
        else {
            cplx zi[8], zj[8];
            for (int k = 0; k < N; k++) { zi[k] = zget(Z, i, N, k); zj[k] = zget(Z, j, N, k); }
            expected_quadrupole(ops, zi, Qi);
            expected_quadrupole(ops, zj, Qj);
        }
        if (pc->biquad_kind == 1) {
            double acc = 0;
            for (int q = 0; q < 5; q++) acc += Qi[q] * (METRIC[q] * Qj[q]);
            Ea += pc->biquad[0] * acc;
        } else {
            double acc = 0;
            for (int q = 0; q < 5; q++)
                for (int p = 0; p < 5; p++) acc += Qi[q] * pc->biquad[q + 5 * p] * Qj[p];
            Ea += acc;
        }
    }
    return Ea;
}

/* Onsite energy of site i (Interactions.jl:449-462). */
static double onsite_energy(const or_sys* s, int64_t i, const double* S, const double* Z, int sun) {
    const double* c = onsite_at(s, i);
    if (!c) return 0;
    if (!sun) {
        double g3[3];
        return or_classical_anisotropy(c, S + 3 * i, g3);
    }
    const int N = s->N;
    cplx acc = 0;
    for (int cc = 0; cc < N; cc++)
        for (int r = 0; r < N; r++) acc += conj(zget(Z, i, N, r)) * (c[2 * (r + N * cc)] + I * c[2 * (r + N * cc) + 1]) * zget(Z, i, N, cc);
    return creal(acc);
}

double or_energy(const or_sys* s, const double* S, const double* Z) {
    int64_t ns = or_nsites(s);
    int L1 = s->L[0], L2 = s->L[1], L3 = s->L[2];
    int N = s->N;
    int sun = (s->mode == SGB_MODE_SUN);
    or_ops ops;
    if (sun) build_ops(N, &ops);
    double E = 0.0;
    if (s->field) {
        for (int64_t i = 0; i < ns; i++) {
            const double* g = s->g + 9 * i;
            const double* B = s->field + 3 * i;
            const double* Si = S + 3 * i;
            double gS[3];
            for (int r = 0; r < 3; r++) gS[r] = g[r] * Si[0] + g[r + 3] * Si[1] + g[r + 6] * Si[2];
            E += B[0] * gS[0] + B[1] * gS[1] + B[2] * gS[2];
        }
    }
    if (s->site_bonds) {
        /* inhomogeneous: per site, Interactions.jl:433-440 */
        for (int64_t i = 0; i < ns; i++) E += onsite_energy(s, i, S, Z, sun);
        for (int64_t e = 0; e < s->nsite_bonds; e++) {
            int64_t i, j;
            site_bond_ends(s, &s->site_bonds[e], &i, &j);
            E += pair_energy(s, &ops, &s->site_bonds[e].bond, i, j, S, Z, sun);
        }
        return E;
    }
    for (int a = 0; a < s->na; a++) {
        double Ea = 0.0;
        for (int c3 = 0; c3 < L3; c3++)
            for (int c2 = 0; c2 < L2; c2++)
                for (int c1 = 0; c1 < L1; c1++) Ea += onsite_energy(s, site_index(s, c1, c2, c3, a), S, Z, sun);
        for (int b = 0; b < s->nbonds; b++) {
            const sgb_bond* pc = &s->bonds[b];
            if (pc->i != a) continue;
            for (int c3 = 0; c3 < L3; c3++)
                for (int c2 = 0; c2 < L2; c2++)
                    for (int c1 = 0; c1 < L1; c1++) {
                        int64_t i = site_index(s, c1, c2, c3, a);
                        int64_t j = site_index(s, wrap(c1 + pc->n[0], L1), wrap(c2 + pc->n[1], L2),
                                               wrap(c3 + pc->n[2], L3), pc->j);
                        Ea += pair_energy(s, &ops, pc, i, j, S, Z, sun);
                    }
        }
        E += Ea;
    }
    /* general couplings (Interactions.jl:495-503): Σ_k <A_k>_i <B_k>_j */
    for (int t = 0; sun && t < s->ngen; t++) {
        const sgb_bond* pc = &s->bonds[s->gen_bond[t]];
        const double* A = s->gen_A + (size_t)2 * N * N * t;
        const double* B = s->gen_B + (size_t)2 * N * N * t;
        for (int c3 = 0; c3 < L3; c3++)
            for (int c2 = 0; c2 < L2; c2++)
                for (int c1 = 0; c1 < L1; c1++) {
                    int64_t i = site_index(s, c1, c2, c3, pc->i);
                    int64_t j = site_index(s, wrap(c1 + pc->n[0], L1), wrap(c2 + pc->n[1], L2), wrap(c3 + pc->n[2], L3),
                                           pc->j);
                    cplx zi[8], zj[8];
                    for (int k = 0; k < N; k++) { zi[k] = zget(Z, i, N, k); zj[k] = zget(Z, j, N, k); }
                    E += expect_op(N, A, zi) * expect_op(N, B, zj);
                }
    }
    return E;
}

/* ---- ewald_energy_delta (Ewald.jl:210-241): ΔS·∇E(site) + ½ Δμ·A[0,i,i]·Δμ, with
 * ∇E(site) = Σ_j g_siteᵀ A[cell_j - cell_site, i, j] g_j S_j over every site j ---------- */
static double ewald_delta(const or_sys* s, const double* S, int64_t site, const double* dS) {
    const int L1 = s->L[0], L2 = s->L[1], L3 = s->L[2], na = s->na;
    const int64_t ncell = (int64_t)L1 * L2 * L3, ns = or_nsites(s);
    const int ai = (int)(site / ncell);
    const int64_t ci = site % ncell;
    const int x1 = (int)(ci % L1), y1 = (int)((ci / L1) % L2), z1 = (int)(ci / ((int64_t)L1 * L2));
    const double* gi = s->g + 9 * site;
    double f[3] = {0, 0, 0};
    for (int64_t j = 0; j < ns; j++) {
        const int aj = (int)(j / ncell);
        const int64_t cj = j % ncell;
        const int x2 = (int)(cj % L1), y2 = (int)((cj / L1) % L2), z2 = (int)(cj / ((int64_t)L1 * L2));
        const int64_t off = wrap(x2 - x1, L1) + (int64_t)L1 * (wrap(y2 - y1, L2) + (int64_t)L2 * wrap(z2 - z1, L3));
        const double* A = s->ewA + ((off * na + ai) * na + aj) * 9;
        const double* gj = s->g + 9 * j;
        double mu[3], Am[3];
        for (int r = 0; r < 3; r++) mu[r] = gj[r] * S[3 * j] + gj[r + 3] * S[3 * j + 1] + gj[r + 6] * S[3 * j + 2];
        for (int r = 0; r < 3; r++) Am[r] = A[r] * mu[0] + A[r + 3] * mu[1] + A[r + 6] * mu[2];
        for (int r = 0; r < 3; r++) f[r] += gi[3 * r] * Am[0] + gi[3 * r + 1] * Am[1] + gi[3 * r + 2] * Am[2];
    }
    double dmu[3], Ad[3];
    for (int r = 0; r < 3; r++) dmu[r] = -(gi[r] * dS[0] + gi[r + 3] * dS[1] + gi[r + 6] * dS[2]);
    const double* A0 = s->ewA + ((int64_t)ai * na + ai) * 9;
    for (int r = 0; r < 3; r++) Ad[r] = A0[r] * dmu[0] + A0[r + 3] * dmu[1] + A0[r + 6] * dmu[2];
    return dS[0] * f[0] + dS[1] * f[1] + dS[2] * f[2] + 0.5 * (dmu[0] * Ad[0] + dmu[1] * Ad[1] + dmu[2] * Ad[2]);
}

/* ---- local_energy_change (Interactions.jl:311-373), dipole modes ------------------ */
static double biquad_pair(const sgb_bond* pc, const double* Qa, const double* Qb) {
    /* Qa' B Qb (kind 2) or biquad * sum_q Qa_q metric_q Qb_q (kind 1) */
    double acc = 0;
    if (pc->biquad_kind == 1) {
        for (int q = 0; q < 5; q++) acc += Qa[q] * (METRIC[q] * Qb[q]);
        return pc->biquad[0] * acc;
    }
    for (int q = 0; q < 5; q++)
        for (int p = 0; p < 5; p++) acc += Qa[q] * pc->biquad[q + 5 * p] * Qb[p];
    return acc;
}

static double local_energy_change_pairs(const or_sys* s, const double* S, int64_t site, const double* Snew);

double or_local_energy_change(const or_sys* s, const double* S, int64_t site, const double* Snew) {
    double dE = local_energy_change_pairs(s, S, site, Snew);
    if (s->ewA && !isnan(dE)) {
        const double dS[3] = {Snew[0] - S[3 * site], Snew[1] - S[3 * site + 1], Snew[2] - S[3 * site + 2]};
        dE += ewald_delta(s, S, site, dS);
    }
    return dE;
}

static double local_energy_change_pairs(const or_sys* s, const double* S, int64_t site, const double* Snew) {
    int L1 = s->L[0], L2 = s->L[1], L3 = s->L[2];
    int64_t ncell = (int64_t)L1 * L2 * L3;
    int a = (int)(site / ncell);
    int64_t cell = site % ncell;
    int c1 = (int)(cell % L1), c2 = (int)((cell / L1) % L2), c3 = (int)(cell / ((int64_t)L1 * L2));
    const double* S0 = S + 3 * site;
    double dS[3] = {Snew[0] - S0[0], Snew[1] - S0[1], Snew[2] - S0[2]};
    double dE = 0.0;
    if (s->field) {
        const double* g = s->g + 9 * site;
        const double* B = s->field + 3 * site;
        for (int r = 0; r < 3; r++) dE += B[r] * (g[r] * dS[0] + g[r + 3] * dS[1] + g[r + 6] * dS[2]);
    }
    const double* c28 = onsite_at(s, site);
    if (c28) {
        double g3[3];
        dE += or_classical_anisotropy(c28, Snew, g3) - or_classical_anisotropy(c28, S0, g3);
    }
    double Qn[5], Qo[5], dQ[5];
    quadrupole(Snew, Qn);
    quadrupole(S0, Qo);
    for (int q = 0; q < 5; q++) dQ[q] = Qn[q] - Qo[q];
    if (s->site_bonds) {
        /* inhomogeneous: the site's own list holds its non-culled couplings and the
         * reversed copies of its neighbours' (Interactions.jl:344-372) */
        for (int64_t e = 0; e < s->nsite_bonds; e++) {
            const sgb_bond* pc = &s->site_bonds[e].bond;
            const double* J = pc->bilin;
            int64_t i, j;
            site_bond_ends(s, &s->site_bonds[e], &i, &j);
            if (i == site && j == site) return NAN;
            if (i == site) {
                const double* Sj = S + 3 * j;
                for (int r = 0; r < 3; r++) dE += dS[r] * (J[r] * Sj[0] + J[r + 3] * Sj[1] + J[r + 6] * Sj[2]);
                if (pc->biquad_kind != 0) { double Qj[5]; quadrupole(Sj, Qj); dE += biquad_pair(pc, dQ, Qj); }
            } else if (j == site) {
                const double* Sk = S + 3 * i;
                for (int r = 0; r < 3; r++) dE += Sk[r] * (J[r] * dS[0] + J[r + 3] * dS[1] + J[r + 6] * dS[2]);
                if (pc->biquad_kind != 0) { double Qk[5]; quadrupole(Sk, Qk); dE += biquad_pair(pc, Qk, dQ); }
            }
        }
        return dE;
    }
    for (int b = 0; b < s->nbonds; b++) {
        const sgb_bond* pc = &s->bonds[b];
        const double* J = pc->bilin;
        if (pc->i == a) {   /* site is the first end: partner at c + n */
            int64_t j = site_index(s, wrap(c1 + pc->n[0], L1), wrap(c2 + pc->n[1], L2), wrap(c3 + pc->n[2], L3), pc->j);
            if (j == site) return NAN;
            const double* Sj = S + 3 * j;
            for (int r = 0; r < 3; r++) dE += dS[r] * (J[r] * Sj[0] + J[r + 3] * Sj[1] + J[r + 6] * Sj[2]);
            if (pc->biquad_kind != 0) { double Qj[5]; quadrupole(Sj, Qj); dE += biquad_pair(pc, dQ, Qj); }
        }
        if (pc->j == a) {   /* site is the second end: partner at c - n */
            int64_t k = site_index(s, wrap(c1 - pc->n[0], L1), wrap(c2 - pc->n[1], L2), wrap(c3 - pc->n[2], L3), pc->i);
            if (k == site) return NAN;
            const double* Sk = S + 3 * k;
            for (int r = 0; r < 3; r++) dE += Sk[r] * (J[r] * dS[0] + J[r + 3] * dS[1] + J[r + 6] * dS[2]);
            if (pc->biquad_kind != 0) { double Qk[5]; quadrupole(Sk, Qk); dE += biquad_pair(pc, Qk, dQ); }
        }
    }
    return dE;
}

/* SU(N) mode: Z [ns][N][2] and S [ns][3] (expected dipoles); the ket at `site` becomes
 * Znew [N][2]. Neighbours enter through expected dipoles and quadrupoles. */
static double onsite_e(int N, const double* lam, const cplx* z) {
    cplx acc = 0;
    for (int c = 0; c < N; c++)
        for (int r = 0; r < N; r++) acc += conj(z[r]) * (lam[2 * (r + N * c)] + I * lam[2 * (r + N * c) + 1]) * z[c];
    return creal(acc);
}

static double local_energy_change_sun_pairs(const or_sys* s, const double* S, const double* Z, int64_t site, const double* Znew);

double or_local_energy_change_sun(const or_sys* s, const double* S, const double* Z, int64_t site, const double* Znew) {
    double dE = local_energy_change_sun_pairs(s, S, Z, site, Znew);
    if (s->ewA && !isnan(dE)) {
        double sn[3];
        or_expected_spin(s->N, Znew, sn);
        const double dS[3] = {sn[0] - S[3 * site], sn[1] - S[3 * site + 1], sn[2] - S[3 * site + 2]};
        dE += ewald_delta(s, S, site, dS);
    }
    return dE;
}

static double local_energy_change_sun_pairs(const or_sys* s, const double* S, const double* Z, int64_t site, const double* Znew) {
    const int N = s->N, L1 = s->L[0], L2 = s->L[1], L3 = s->L[2];
    or_ops ops;
    build_ops(N, &ops);
    int64_t ncell = (int64_t)L1 * L2 * L3;
    int a = (int)(site / ncell);
    int64_t cell = site % ncell;
    int c1 = (int)(cell % L1), c2 = (int)((cell / L1) % L2), c3 = (int)(cell / ((int64_t)L1 * L2));
    cplx z0[8], zn[8];
    for (int k = 0; k < N; k++) { z0[k] = zget(Z, site, N, k); zn[k] = Znew[2 * k] + I * Znew[2 * k + 1]; }
    double s0[3], sn[3], q0[5], qn[5], dS[3], dQ[5];
    or_expected_spin(N, Z + 2 * (size_t)N * site, s0);
    or_expected_spin(N, Znew, sn);
    expected_quadrupole(&ops, z0, q0);
    expected_quadrupole(&ops, zn, qn);
    for (int r = 0; r < 3; r++) dS[r] = sn[r] - s0[r];
    for (int q = 0; q < 5; q++) dQ[q] = qn[q] - q0[q];
    double dE = 0;
    if (s->field) {
        const double* g = s->g + 9 * site;
        const double* B = s->field + 3 * site;
        for (int r = 0; r < 3; r++) dE += B[r] * (g[r] * dS[0] + g[r + 3] * dS[1] + g[r + 6] * dS[2]);
    }
    const double* lam = onsite_at(s, site);
    if (lam) dE += onsite_e(N, lam, zn) - onsite_e(N, lam, z0);
    if (s->site_bonds) {
        for (int64_t e = 0; e < s->nsite_bonds; e++) {
            const sgb_bond* pc = &s->site_bonds[e].bond;
            const double* J = pc->bilin;
            int64_t i, j;
            site_bond_ends(s, &s->site_bonds[e], &i, &j);
            if (i == site && j == site) return NAN;
            if (i != site && j != site) continue;
            const int end = i == site ? 0 : 1;
            const int64_t o = end == 0 ? j : i;
            const double* So = S + 3 * o;
            if (end == 0) for (int r = 0; r < 3; r++) dE += dS[r] * (J[r] * So[0] + J[r + 3] * So[1] + J[r + 6] * So[2]);
            else for (int r = 0; r < 3; r++) dE += So[r] * (J[r] * dS[0] + J[r + 3] * dS[1] + J[r + 6] * dS[2]);
            if (pc->biquad_kind != 0) {
                cplx zo[8];
                double Qo[5];
                for (int k = 0; k < N; k++) zo[k] = zget(Z, o, N, k);
                expected_quadrupole(&ops, zo, Qo);
                dE += end == 0 ? biquad_pair(pc, dQ, Qo) : biquad_pair(pc, Qo, dQ);
            }
        }
        return dE;
    }
    for (int b = 0; b < s->nbonds; b++) {
        const sgb_bond* pc = &s->bonds[b];
        const double* J = pc->bilin;
        for (int end = 0; end < 2; end++) {
            if ((end == 0 ? pc->i : pc->j) != a) continue;
            int sg_ = end == 0 ? 1 : -1;
            int64_t j = site_index(s, wrap(c1 + sg_ * pc->n[0], L1), wrap(c2 + sg_ * pc->n[1], L2), wrap(c3 + sg_ * pc->n[2], L3),
                                   end == 0 ? pc->j : pc->i);
            if (j == site) return NAN;
            const double* Sj = S + 3 * j;
            if (end == 0) for (int r = 0; r < 3; r++) dE += dS[r] * (J[r] * Sj[0] + J[r + 3] * Sj[1] + J[r + 6] * Sj[2]);
            else for (int r = 0; r < 3; r++) dE += Sj[r] * (J[r] * dS[0] + J[r + 3] * dS[1] + J[r + 6] * dS[2]);
            if (pc->biquad_kind != 0) {
                cplx zj[8];
                double Qj[5];
                for (int k = 0; k < N; k++) zj[k] = zget(Z, j, N, k);
                expected_quadrupole(&ops, zj, Qj);
                dE += end == 0 ? biquad_pair(pc, dQ, Qj) : biquad_pair(pc, Qj, dQ);
            }
        }
    }
    /* general couplings: Δ<A>_site <B>_j where the site is the first end, <A>_k Δ<B>_site
     * where it is the second (Interactions.jl:364-370) */
    for (int t = 0; t < s->ngen; t++) {
        const sgb_bond* pc = &s->bonds[s->gen_bond[t]];
        const double* A = s->gen_A + (size_t)2 * N * N * t;
        const double* B = s->gen_B + (size_t)2 * N * N * t;
        for (int end = 0; end < 2; end++) {
            if ((end == 0 ? pc->i : pc->j) != a) continue;
            int sg_ = end == 0 ? 1 : -1;
            int64_t o = site_index(s, wrap(c1 + sg_ * pc->n[0], L1), wrap(c2 + sg_ * pc->n[1], L2), wrap(c3 + sg_ * pc->n[2], L3),
                                   end == 0 ? pc->j : pc->i);
            if (o == site) return NAN;
            cplx zo[8];
            for (int k = 0; k < N; k++) zo[k] = zget(Z, o, N, k);
            if (end == 0) dE += (expect_op(N, A, zn) - expect_op(N, A, z0)) * expect_op(N, B, zo);
            else dE += expect_op(N, A, zo) * (expect_op(N, B, zn) - expect_op(N, B, z0));
        }
    }
    return dE;
}

void or_local_sweeps_sun(const or_sys* s, double* S, double* Z, double kT, int nsweeps, double frac, const int* perm,
                         int nkind, const int* kind, const double* cum, const double* mag, const double* rand,
                         double* dE, double* dS3) {
    const int N = s->N, per = 2 * N + 3;
    int64_t ns = or_nsites(s);
    double aE = 0, aS[3] = {0, 0, 0};
    for (int k = 0; k < nsweeps; k++) {
        int partial = (k == nsweeps - 1) && frac < 1.0;
        for (int64_t idx = 0; idx < ns; idx++) {
            int64_t site = perm[idx];
            const double* r = rand + ((size_t)k * ns + site) * per;
            if (partial && !(r[2 * N + 2] < frac)) continue;
            int kd = kind[nkind - 1];
            double m = mag[nkind - 1];
            for (int i = 0; i < nkind - 1; i++)
                if (r[2 * N] < cum[i]) { kd = kind[i]; m = mag[i]; break; }
            if (kd == SGB_PROPOSE_DELTA && isinf(m)) kd = SGB_PROPOSE_UNIFORM;
            const double kap = s->kappa[site];
            double zn[16];
            const double* z0 = Z + 2 * (size_t)N * site;
            if (kd == SGB_PROPOSE_FLIP) {       /* flip_ket: reverse(parity .* conj(z)) */
                for (int q = 0; q < N; q++) {
                    int src = N - 1 - q;
                    double par = (src % 2) ? -1.0 : 1.0;
                    zn[2 * q] = par * z0[2 * src];
                    zn[2 * q + 1] = -par * z0[2 * src + 1];
                }
            } else {
                for (int q = 0; q < 2 * N; q++) zn[q] = kd == SGB_PROPOSE_UNIFORM ? r[q] : z0[q] + m * sqrt(kap) * r[q];
                double n2 = 0;
                for (int q = 0; q < 2 * N; q++) n2 += zn[q] * zn[q];
                double d = sqrt(n2 / kap);   /* normalize_ket */
                for (int q = 0; q < 2 * N; q++) zn[q] = kap == 0 ? 0 : zn[q] / d;
            }
            double e = or_local_energy_change_sun(s, S, Z, site, zn);
            int accept = kT == 0.0 ? (e <= 0.0) : (r[2 * N + 1] <= exp(-e / kT));
            if (accept) {
                double sn[3];
                or_expected_spin(N, zn, sn);
                aE += e;
                for (int c = 0; c < 3; c++) { aS[c] += sn[c] - S[3 * site + c]; S[3 * site + c] = sn[c]; }
                for (int q = 0; q < 2 * N; q++) Z[2 * (size_t)N * site + q] = zn[q];
            }
        }
    }
    if (dE) *dE = aE;
    if (dS3) { dS3[0] = aS[0]; dS3[1] = aS[1]; dS3[2] = aS[2]; }
}

void or_local_sweeps(const or_sys* s, double* S, double kT, int nsweeps, double frac, const int* perm,
                     int nkind, const int* kind, const double* cum, const double* mag, const double* rand,
                     double* dE, double* dS3) {
    int64_t ns = or_nsites(s);
    double aE = 0, aS[3] = {0, 0, 0};
    for (int k = 0; k < nsweeps; k++) {
        int partial = (k == nsweeps - 1) && frac < 1.0;
        for (int64_t idx = 0; idx < ns; idx++) {
            int64_t site = perm[idx];
            const double* r = rand + ((size_t)k * ns + site) * 6;
            if (partial && !(r[5] < frac)) continue;
            int kd = kind[nkind - 1];
            double m = mag[nkind - 1];
            for (int i = 0; i < nkind - 1; i++)
                if (r[3] < cum[i]) { kd = kind[i]; m = mag[i]; break; }
            if (kd == SGB_PROPOSE_DELTA && isinf(m)) kd = SGB_PROPOSE_UNIFORM;
            const double kap = s->kappa[site];
            const double* S0 = S + 3 * site;
            double Sn[3];
            if (kd == SGB_PROPOSE_FLIP) {
                Sn[0] = -S0[0]; Sn[1] = -S0[1]; Sn[2] = -S0[2];
            } else {
                double v[3];
                if (kd == SGB_PROPOSE_UNIFORM) { v[0] = r[0]; v[1] = r[1]; v[2] = r[2]; }   /* randspin */
                else for (int c = 0; c < 3; c++) v[c] = S0[c] + m * kap * r[c];             /* perturbed_spin */
                normalize_dipole(v, kap, Sn);
            }
            double e = or_local_energy_change(s, S, site, Sn);
            int accept = kT == 0.0 ? (e <= 0.0) : (r[4] <= exp(-e / kT));
            if (accept) {
                aE += e;
                for (int c = 0; c < 3; c++) { aS[c] += Sn[c] - S0[c]; S[3 * site + c] = Sn[c]; }
            }
        }
    }
    if (dE) *dE = aE;
    if (dS3) { dS3[0] = aS[0]; dS3[1] = aS[1]; dS3[2] = aS[2]; }
}

/* ---- Ewald.jl:40-146: real-space and reciprocal sums of the dipole kernel ---------- */
static const double OR_PI = 3.14159265358979323846;

static void mat3_mul_vec(const double* M, const double* v, double* out) {   /* M column-major */
    for (int r = 0; r < 3; r++) out[r] = M[r] * v[0] + M[r + 3] * v[1] + M[r + 6] * v[2];
}

void or_ewald_matrices(int L1, int L2, int L3, int na, const double* latvecs, const double* positions,
                       const double* demag, double mu0_muB2, double* out) {
    const int L[3] = {L1, L2, L3};
    double sup[9], rec[9];   /* supercell vectors and their reciprocals (columns) */
    for (int c = 0; c < 3; c++)
        for (int r = 0; r < 3; r++) sup[r + 3 * c] = latvecs[r + 3 * c] * L[c];
    const double* a = sup;
    double det = a[0] * (a[4] * a[8] - a[7] * a[5]) - a[3] * (a[1] * a[8] - a[7] * a[2]) + a[6] * (a[1] * a[5] - a[4] * a[2]);
    /* rec = 2π (sup^-1)^T: columns b_k with a_i·b_k = 2π δ_ik */
    double inv[9];
    inv[0] = (a[4] * a[8] - a[7] * a[5]) / det; inv[3] = (a[6] * a[5] - a[3] * a[8]) / det; inv[6] = (a[3] * a[7] - a[6] * a[4]) / det;
    inv[1] = (a[7] * a[2] - a[1] * a[8]) / det; inv[4] = (a[0] * a[8] - a[6] * a[2]) / det; inv[7] = (a[6] * a[1] - a[0] * a[7]) / det;
    inv[2] = (a[1] * a[5] - a[4] * a[2]) / det; inv[5] = (a[3] * a[2] - a[0] * a[5]) / det; inv[8] = (a[0] * a[4] - a[3] * a[1]) / det;
    for (int c = 0; c < 3; c++)
        for (int r = 0; r < 3; r++) rec[r + 3 * c] = 2 * OR_PI * inv[c + 3 * r];
    const double V = fabs(det), Lc = cbrt(V);
    const double sig = Lc / 3, sig2 = sig * sig, sig3 = sig2 * sig;
    const double rmax = 6 * sqrt(2.0) * sig, kmax = 6 * sqrt(2.0) / sig;
    int nmax[3], mmax[3];
    for (int k = 0; k < 3; k++) {
        const double* ak = sup + 3 * k;
        const double* bk = rec + 3 * k;
        double nb = sqrt(bk[0] * bk[0] + bk[1] * bk[1] + bk[2] * bk[2]);
        double na_ = sqrt(ak[0] * ak[0] + ak[1] * ak[1] + ak[2] * ak[2]);
        double ab = (ak[0] * bk[0] + ak[1] * bk[1] + ak[2] * bk[2]);
        nmax[k] = (int)lround(rmax / (ab / nb) + 1e-6) + 1;
        mmax[k] = (int)lround(kmax / (ab / na_) + 1e-6);
    }
    const int ncell = L1 * L2 * L3;
    for (int i = 0; i < na; i++)
        for (int j = 0; j < na; j++)
            for (int c3 = 0; c3 < L3; c3++)
                for (int c2 = 0; c2 < L2; c2++)
                    for (int c1 = 0; c1 < L1; c1++) {
                        double acc[9] = {0};
                        double fr[3] = {c1 + positions[3 * j] - positions[3 * i], c2 + positions[3 * j + 1] - positions[3 * i + 1],
                                        c3 + positions[3 * j + 2] - positions[3 * i + 2]};
                        double dr[3];
                        mat3_mul_vec(latvecs, fr, dr);
                        for (int n1 = -nmax[0]; n1 <= nmax[0]; n1++)
                            for (int n2 = -nmax[1]; n2 <= nmax[1]; n2++)
                                for (int n3 = -nmax[2]; n3 <= nmax[2]; n3++) {
                                    double nn[3] = {n1, n2, n3}, sh[3];
                                    mat3_mul_vec(sup, nn, sh);
                                    double rv[3] = {dr[0] + sh[0], dr[1] + sh[1], dr[2] + sh[2]};
                                    double r2 = rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2];
                                    if (!(r2 > 0 && r2 <= rmax * rmax)) continue;
                                    double r = sqrt(r2), r3 = r2 * r;
                                    double ec = erfc(r / (sqrt(2.0) * sig));
                                    double ga = sqrt(2 / OR_PI) * (r / sig) * exp(-r2 / (2 * sig2));
                                    double c_iso = (ec + ga) / r3 / (4 * OR_PI);
                                    double c_rr = 3 * (ec + (1 + r2 / (3 * sig2)) * ga) / r3 / (4 * OR_PI) / r2;
                                    for (int q = 0; q < 3; q++)
                                        for (int p = 0; p < 3; p++) acc[p + 3 * q] += (p == q ? c_iso : 0) - c_rr * rv[p] * rv[q];
                                }
                        for (int m1 = -mmax[0]; m1 <= mmax[0]; m1++)
                            for (int m2 = -mmax[1]; m2 <= mmax[1]; m2++)
                                for (int m3 = -mmax[2]; m3 <= mmax[2]; m3++) {
                                    double mm[3] = {m1, m2, m3}, k[3];
                                    mat3_mul_vec(rec, mm, k);
                                    double k2 = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
                                    if (k2 <= 1e-16) {
                                        for (int q = 0; q < 9; q++) acc[q] += demag[q] / V;   /* surface term */
                                    } else if (k2 <= kmax * kmax) {
                                        double w = cos(k[0] * dr[0] + k[1] * dr[1] + k[2] * dr[2]) * exp(-sig2 * k2 / 2) / k2 / V;
                                        for (int q = 0; q < 3; q++)
                                            for (int p = 0; p < 3; p++) acc[p + 3 * q] += w * k[p] * k[q];
                                    }
                                }
                        if (dr[0] == 0 && dr[1] == 0 && dr[2] == 0)
                            for (int q = 0; q < 3; q++) acc[q + 3 * q] -= 1.0 / (3 * pow(2 * OR_PI, 1.5) * sig3);
                        int cell = c1 + L1 * (c2 + L2 * c3);
                        double* o = out + (((size_t)cell * na + i) * na + j) * 9;
                        for (int q = 0; q < 9; q++) o[q] = acc[q] * mu0_muB2;
                    }
    (void)ncell;
}

/* ---- Integrators.jl:266-275 rhs_dipole! for one site ------------------------------- */
static inline void rhs_dipole(const double* S, const double* xi, const double* g, double dt, double lam, double* dS) {
    double v[3];
    if (lam == 0.0) {
        double dg[3] = {dt * g[0], dt * g[1], dt * g[2]};
        cross3(S, dg, v);
    } else {
        double sxg[3];
        cross3(S, g, sxg);
        double dl = dt * lam;
        double w[3] = {xi[0] + dt * g[0] - dl * sxg[0], xi[1] + dt * g[1] - dl * sxg[1], xi[2] + dt * g[2] - dl * sxg[2]};
        cross3(S, w, v);
    }
    dS[0] = -v[0]; dS[1] = -v[1]; dS[2] = -v[2];
}

/* Integrators.jl:313-332 */
void or_langevin_dipole(const or_sys* s, double* S, double dt, double damping, double kT, const double* noise) {
    int64_t ns = or_nsites(s);
    double* Sp = malloc(sizeof(double) * 3 * ns);
    double* dS1 = malloc(sizeof(double) * 3 * ns);
    double* dS2 = malloc(sizeof(double) * 3 * ns);
    double* xi = calloc(3 * ns, sizeof(double));
    double* gE = malloc(sizeof(double) * 3 * ns);
    /* fill_noise! (Integrators.jl:288-298) */
    if (!(damping == 0.0 || kT == 0.0) && noise) {
        double sc = sqrt(2 * dt * damping * kT);
        for (int64_t k = 0; k < 3 * ns; k++) xi[k] = noise[k] * sc;
    }
    or_grad_dipoles(s, S, gE);
    for (int64_t i = 0; i < ns; i++) {
        rhs_dipole(S + 3 * i, xi + 3 * i, gE + 3 * i, dt, damping, dS1 + 3 * i);
        double t[3] = {S[3 * i] + dS1[3 * i], S[3 * i + 1] + dS1[3 * i + 1], S[3 * i + 2] + dS1[3 * i + 2]};
        normalize_dipole(t, s->kappa[i], Sp + 3 * i);
    }
    or_grad_dipoles(s, Sp, gE);
    for (int64_t i = 0; i < ns; i++) {
        rhs_dipole(Sp + 3 * i, xi + 3 * i, gE + 3 * i, dt, damping, dS2 + 3 * i);
        double t[3];
        for (int r = 0; r < 3; r++) t[r] = S[3 * i + r] + (dS1[3 * i + r] + dS2[3 * i + r]) / 2;
        normalize_dipole(t, s->kappa[i], S + 3 * i);
    }
    free(Sp); free(dS1); free(dS2); free(xi); free(gE);
}

/* System.jl:416-418 normalize_ket: Z / sqrt(|Z|^2/κ) */
static inline void normalize_ket(int N, const cplx* z, double kappa, cplx* out) {
    if (kappa == 0.0) { for (int k = 0; k < N; k++) out[k] = 0; return; }
    double n2 = 0;
    for (int k = 0; k < N; k++) n2 += creal(conj(z[k]) * z[k]);
    double d = sqrt(n2 / kappa);
    for (int k = 0; k < N; k++) out[k] = z[k] / d;
}

/* Integrators.jl:277-286 rhs_sun! for one site; MathBasics.jl:62 proj */
static inline void rhs_sun(int N, const cplx* z, const cplx* zeta, const cplx* hz, double dt, double lam, cplx* dz) {
    if (lam == 0.0) {
        for (int k = 0; k < N; k++) dz[k] = -I * dt * hz[k];
        return;
    }
    cplx v[8];
    for (int k = 0; k < N; k++) v[k] = zeta[k] + dt * (I + lam) * hz[k];
    cplx nv = 0;
    double nn = 0;
    for (int k = 0; k < N; k++) { nv += conj(z[k]) * v[k]; nn += creal(conj(z[k]) * z[k]); }
    cplx f = nv / nn;
    for (int k = 0; k < N; k++) dz[k] = -(v[k] - z[k] * f);
}

/* Integrators.jl:335-357 */
void or_langevin_sun(const or_sys* s, double* Z, double* S, double dt, double damping, double kT, const double* noise) {
    int N = s->N;
    int64_t ns = or_nsites(s);
    size_t nz = (size_t)2 * N * ns;
    double* Zp = malloc(sizeof(double) * nz);
    double* dZ1 = malloc(sizeof(double) * nz);
    double* zeta = calloc(nz, sizeof(double));
    double* HZ = malloc(sizeof(double) * nz);
    if (!(damping == 0.0 || kT == 0.0) && noise) {
        double sc = sqrt(2 * dt * damping * kT);
        for (size_t k = 0; k < nz; k++) zeta[k] = noise[k] * sc;
    }
    or_grad_coherents(s, Z, HZ);
    for (int64_t i = 0; i < ns; i++) {
        cplx z[8], ze[8], hz[8], d[8], t[8], o[8];
        for (int k = 0; k < N; k++) { z[k] = zget(Z, i, N, k); ze[k] = zget(zeta, i, N, k); hz[k] = zget(HZ, i, N, k); }
        rhs_sun(N, z, ze, hz, dt, damping, d);
        for (int k = 0; k < N; k++) { zset(dZ1, i, N, k, d[k]); t[k] = z[k] + d[k]; }
        normalize_ket(N, t, s->kappa[i], o);
        for (int k = 0; k < N; k++) zset(Zp, i, N, k, o[k]);
    }
    or_grad_coherents(s, Zp, HZ);
    for (int64_t i = 0; i < ns; i++) {
        cplx z[8], zp[8], ze[8], hz[8], d[8], t[8], o[8];
        for (int k = 0; k < N; k++) { z[k] = zget(Z, i, N, k); zp[k] = zget(Zp, i, N, k); ze[k] = zget(zeta, i, N, k); hz[k] = zget(HZ, i, N, k); }
        rhs_sun(N, zp, ze, hz, dt, damping, d);
        for (int k = 0; k < N; k++) t[k] = z[k] + (zget(dZ1, i, N, k) + d[k]) / 2;
        normalize_ket(N, t, s->kappa[i], o);
        for (int k = 0; k < N; k++) zset(Z, i, N, k, o[k]);
        or_expected_spin(N, Z + 2 * N * i, S + 3 * i);
    }
    free(Zp); free(dZ1); free(zeta); free(HZ);
}

/* Integrators.jl:361-371 fast_isapprox */
static int fast_isapprox(const double* x, const double* y, int64_t n, double atol) {
    double acc = 0.0;
    for (int64_t i = 0; i < n; i++) {
        double d = x[i] - y[i];
        acc += d * d;
        if (acc > atol * atol) return 0;
    }
    return !isnan(acc);
}

/* Integrators.jl:379-413 */
int or_midpoint_dipole(const or_sys* s, double* S, double dt, double damping, double tol, int max_iters, int64_t* iters) {
    int64_t ns = or_nsites(s);
    double atol = tol * sqrt((double)ns);
    double* Sh = malloc(sizeof(double) * 3 * ns);
    double* Sp = malloc(sizeof(double) * 3 * ns);
    double* Spp = malloc(sizeof(double) * 3 * ns);
    double* gE = malloc(sizeof(double) * 3 * ns);
    double xi0[3] = {0, 0, 0};
    memcpy(Sp, S, sizeof(double) * 3 * ns);
    memcpy(Spp, S, sizeof(double) * 3 * ns);
    int status = SGB_ERR_NOCONVERGE;
    for (int it = 0; it < max_iters; it++) {
        if (iters) (*iters)++;
        for (int64_t i = 0; i < ns; i++) {
            double t[3];
            for (int r = 0; r < 3; r++) t[r] = (S[3 * i + r] + Sp[3 * i + r]) / 2;
            normalize_dipole(t, s->kappa[i], Sh + 3 * i);
        }
        or_grad_dipoles(s, Sh, gE);
        for (int64_t i = 0; i < ns; i++) {
            double dS[3];
            rhs_dipole(Sh + 3 * i, xi0, gE + 3 * i, dt, damping, dS);
            for (int r = 0; r < 3; r++) Spp[3 * i + r] = S[3 * i + r] + dS[r];
        }
        if (fast_isapprox(Sp, Spp, 3 * ns, atol)) {
            for (int64_t i = 0; i < ns; i++) normalize_dipole(Spp + 3 * i, s->kappa[i], S + 3 * i);
            status = SGB_OK;
            break;
        }
        double* t = Sp; Sp = Spp; Spp = t;
    }
    free(Sh); free(Sp); free(Spp); free(gE);
    return status;
}

/* Integrators.jl:422-452 */
int or_midpoint_sun(const or_sys* s, double* Z, double* S, double dt, double damping, double tol, int max_iters, int64_t* iters) {
    int N = s->N;
    int64_t ns = or_nsites(s);
    size_t nz = (size_t)2 * N * ns;
    double atol = tol * sqrt((double)ns);
    double* Zb = malloc(sizeof(double) * nz);
    double* Zp = malloc(sizeof(double) * nz);
    double* Zpp = malloc(sizeof(double) * nz);
    double* HZ = malloc(sizeof(double) * nz);
    memcpy(Zp, Z, sizeof(double) * nz);
    memcpy(Zpp, Z, sizeof(double) * nz);
    int status = SGB_ERR_NOCONVERGE;
    cplx zero[8] = {0};
    for (int it = 0; it < max_iters; it++) {
        if (iters) (*iters)++;
        for (size_t k = 0; k < nz; k++) Zb[k] = (Z[k] + Zp[k]) / 2;
        or_grad_coherents(s, Zb, HZ);
        for (int64_t i = 0; i < ns; i++) {
            cplx zb[8], hz[8], d[8];
            for (int k = 0; k < N; k++) { zb[k] = zget(Zb, i, N, k); hz[k] = zget(HZ, i, N, k); }
            rhs_sun(N, zb, zero, hz, dt, damping, d);
            for (int k = 0; k < N; k++) zset(Zpp, i, N, k, zget(Z, i, N, k) + d[k]);
        }
        if (fast_isapprox(Zp, Zpp, (int64_t)nz, atol)) {
            for (int64_t i = 0; i < ns; i++) {
                cplx t[8], o[8];
                for (int k = 0; k < N; k++) t[k] = zget(Zpp, i, N, k);
                normalize_ket(N, t, s->kappa[i], o);
                for (int k = 0; k < N; k++) zset(Z, i, N, k, o[k]);
                or_expected_spin(N, Z + 2 * N * i, S + 3 * i);
            }
            status = SGB_OK;
            break;
        }
        double* t = Zp; Zp = Zpp; Zpp = t;
    }
    free(Zb); free(Zp); free(Zpp); free(HZ);
    return status;
}

void or_langevin_steps(const or_sys* s, double* S, double* Z, double dt, double damping, double kT, int nsteps, const double* noise) {
    int64_t ns = or_nsites(s);
    int64_t per = (s->mode == SGB_MODE_SUN) ? 2 * s->N * ns : 3 * ns;
    for (int k = 0; k < nsteps; k++) {
        const double* nz = noise ? noise + (size_t)k * per : NULL;
        if (s->mode == SGB_MODE_SUN) or_langevin_sun(s, Z, S, dt, damping, kT, nz);
        else or_langevin_dipole(s, S, dt, damping, kT, nz);
    }
}

int or_midpoint_steps(const or_sys* s, double* S, double* Z, double dt, double damping, double tol, int max_iters, int nsteps, int64_t* iters) {
    for (int k = 0; k < nsteps; k++) {
        int st = (s->mode == SGB_MODE_SUN) ? or_midpoint_sun(s, Z, S, dt, damping, tol, max_iters, iters)
                                           : or_midpoint_dipole(s, S, dt, damping, tol, max_iters, iters);
        if (st != SGB_OK) return st;
    }
    return SGB_OK;
}

/* CorrelationSampling.jl:1-19 observable_values! */
void or_observables(const or_sys* s, const double* S, const double* Z, int nobs, const double* obs, double* out) {
    int64_t ns = or_nsites(s);
    int N = s->N;
    for (int o = 0; o < nobs; o++) {
        for (int64_t i = 0; i < ns; i++) {
            if (s->mode != SGB_MODE_SUN) {
                const double* op = obs + 3 * ((size_t)o * ns + i);
                out[(size_t)o * ns + i] = op[0] * S[3 * i] + op[1] * S[3 * i + 1] + op[2] * S[3 * i + 2];
            } else {
                const double* A = obs + 2 * (size_t)N * N * ((size_t)o * ns + i);
                cplx acc = 0;
                for (int c = 0; c < N; c++)
                    for (int r = 0; r < N; r++)
                        acc += conj(zget(Z, i, N, r)) * (A[2 * (r + N * c)] + I * A[2 * (r + N * c) + 1]) * zget(Z, i, N, c);
                out[(size_t)o * ns + i] = creal(acc);
            }
        }
    }
}

/* ---- timed CPU baseline over replicas ----------------------------------------------- */
static inline uint64_t splitmix64(uint64_t* x) {
    uint64_t z = (*x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static inline double gauss(uint64_t* st) {
    double u1 = ((splitmix64(st) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    double u2 = ((splitmix64(st) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    return sqrt(-2 * log(u1)) * cos(6.283185307179586 * u2);
}

int or_langevin_replicas(const or_sys* s, int nrep, double* S, const double* kT, double dt, double damping, int nsteps, uint64_t seed) {
    int64_t ns = or_nsites(s);
    int threads = 1;
#ifdef _OPENMP
    threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int r = 0; r < nrep; r++) {
        double* noise = malloc(sizeof(double) * 3 * ns);
        uint64_t st = seed * 0x100000001B3ull + (uint64_t)r;
        for (int k = 0; k < nsteps; k++) {
            for (int64_t q = 0; q < 3 * ns; q++) noise[q] = gauss(&st);
            or_langevin_dipole(s, S + (size_t)r * 3 * ns, dt, damping, kT[r], noise);
        }
        free(noise);
    }
    return threads;
}
