// sgb_device.cuh -- device functions shared by the dipole, SU(N) and replica-batch
// kernels: coupling-table staging, the gather-form dipole gradient, the classical
// Stevens anisotropy and the Landau-Lifshitz right-hand side.
//
// Reference algorithms (Sunny.jl v0.9.2):
//   gradient      src/System/Interactions.jl:516-592
//   anisotropy    src/System/OnsiteCoupling.jl:316-425
//   quadrupoles   src/Operators/Spin.jl:48-69
//   rhs_dipole!   src/Integrators.jl:266-275
//   normalization src/System/System.jl:416-423
#pragma once
#include "sgb_internal.h"

namespace sgbdev {

template <class R>
struct Tab {
    const R* stev;
    const int* kmax;
    const int* boff;
    const DBond<R>* bonds;
    const R* bq;
};

template <class R>
__device__ inline Tab<R> stage_tables(const Model<R>& M, unsigned char* smem) {
    const uint4* src = reinterpret_cast<const uint4*>(M.tables);
    uint4* dst = reinterpret_cast<uint4*>(smem);
    int n16 = M.tables_bytes / 16;
    for (int i = threadIdx.x; i < n16; i += blockDim.x) dst[i] = src[i];
    __syncthreads();
    Tab<R> t;
    t.stev = reinterpret_cast<const R*>(smem + M.off_stev);
    t.kmax = reinterpret_cast<const int*>(smem + M.off_kmax);
    t.boff = reinterpret_cast<const int*>(smem + M.off_boff);
    t.bonds = reinterpret_cast<const DBond<R>*>(smem + M.off_bonds);
    t.bq = reinterpret_cast<const R*>(smem + M.off_bq);
    return t;
}

// Classical Stevens anisotropy, OnsiteCoupling.jl:316-425. Coefficients c (28) hold
// c0, c2[5], c4[9], c6[13] in descending q. Adds the gradient into g and returns E.
template <class R>
__device__ inline R aniso_k(const R* c, int k, const R* A, const R* dA, const R* pr, const R* pi,
                            R& E, R& dz, R& jr, R& ji) {
    // m = 0
    E += c[k] * A[0];
    dz += c[k] * dA[0];
#pragma unroll
    for (int m = 1; m <= 6; m++) {
        if (m > k) break;
        R ca = c[k - m], cb = c[k + m];
        R t = ca * pr[m] + cb * pi[m];
        E += t * A[m];
        if (m < k) dz += t * dA[m];
        // (m/2)(ca - i cb) Jp^(m-1) A[m]
        R h = (R)(0.5 * m) * A[m];
        jr += h * (ca * pr[m - 1] + cb * pi[m - 1]);
        ji += h * (ca * pi[m - 1] - cb * pr[m - 1]);
    }
    return E;
}

template <class R>
__device__ inline R classical_aniso(const R* c, int kmax, R x, R y, R z, R& gx, R& gy, R& gz) {
    R E = c[0];
    if (kmax == 0) return E;
    R X = x * x + y * y + z * z;
    R pr[7], pi[7];
    pr[0] = 1; pi[0] = 0;
#pragma unroll
    for (int m = 1; m <= 6; m++) {
        pr[m] = pr[m - 1] * x - pi[m - 1] * y;
        pi[m] = pr[m - 1] * y + pi[m - 1] * x;
    }
    R z2 = z * z, z3 = z2 * z, z4 = z2 * z2, z5 = z4 * z, z6 = z3 * z3;
    R X2 = X * X, X3 = X2 * X;
    R dz = 0, jr = 0, ji = 0;
    {
        R A[3] = {3 * z2 - X, z, 1};
        R dA[3] = {6 * z, 1, 0};
        aniso_k<R>(c + 1, 2, A, dA, pr, pi, E, dz, jr, ji);
    }
    if (kmax >= 4) {
        R A[5] = {35 * z4 - (30 * X) * z2 + 3 * X2, 7 * z3 - (3 * X) * z, 7 * z2 - X, z, 1};
        R dA[5] = {140 * z3 - (60 * X) * z, 21 * z2 - 3 * X, 14 * z, 1, 0};
        aniso_k<R>(c + 6, 4, A, dA, pr, pi, E, dz, jr, ji);
    }
    if (kmax >= 6) {
        R A[7] = {231 * z6 - (315 * X) * z4 + (105 * X2) * z2 - 5 * X3,
                  33 * z5 - (30 * X) * z3 + (5 * X2) * z,
                  33 * z4 - (18 * X) * z2 + X2,
                  11 * z3 - (3 * X) * z,
                  11 * z2 - X,
                  z,
                  1};
        R dA[7] = {1386 * z5 - (1260 * X) * z3 + (210 * X2) * z,
                   165 * z4 - (90 * X) * z2 + 5 * X2,
                   132 * z3 - (36 * X) * z,
                   33 * z2 - 3 * X,
                   22 * z,
                   1,
                   0};
        aniso_k<R>(c + 15, 6, A, dA, pr, pi, E, dz, jr, ji);
    }
    gx += 2 * jr;
    gy += -2 * ji;
    gz += dz;
    return E;
}

// Stevens quadrupoles and their gradient (src/Operators/Spin.jl:48-69).
template <class R>
__device__ inline void quad5(R x, R y, R z, R* Q) {
    Q[0] = x * x - y * y;
    Q[1] = z * x;
    Q[2] = -x * x - y * y + 2 * z * z;
    Q[3] = z * y;
    Q[4] = 2 * y * x;
}
template <class R>
__device__ inline void add_quad_grad(R x, R y, R z, const R* v, R& gx, R& gy, R& gz) {
    // sum_q v_q * grad Q_q
    gx += v[0] * (2 * x) + v[1] * z + v[2] * (-2 * x) + v[4] * (2 * y);
    gy += v[0] * (-2 * y) + v[2] * (-2 * y) + v[3] * z + v[4] * (2 * x);
    gz += v[1] * x + v[2] * (4 * z) + v[3] * y;
}

struct SiteIdx { int c1, c2, c3, a; };
__device__ __forceinline__ SiteIdx decompose(int s, int L1, int L2, int L3) {
    SiteIdx r;
    r.c1 = s % L1; s /= L1;
    r.c2 = s % L2; s /= L2;
    r.c3 = s % L3; r.a = s / L3;
    return r;
}

// dE/dS at one site in gather form. X/Y/Zc are the SoA spins seen by neighbours (already
// offset to the replica's first site); (L1, L2, L3) are the replica's dims. ANYWRAP
// selects the wrap for raw bond offsets |n| <= L (replica batches) instead of offsets
// pre-reduced into [0, L) (single systems). h/kap are per-site (single system) or per
// sublattice (batch).
template <class R, bool ANYWRAP>
__device__ inline void grad_site_L(const Model<R>& M, const Tab<R>& T, const SiteIdx& ix, int L1, int L2, int L3,
                                   R hx, R hy, R hz, R sx, R sy, R sz, const R* X, const R* Y, const R* Zc,
                                   R& gx, R& gy, R& gz) {
    gx = hx; gy = hy; gz = hz;
    const int a = ix.a;
    if (M.dipole_mode) {
        int km = T.kmax[a];
        if (km > 0) classical_aniso<R>(T.stev + 28 * a, km, sx, sy, sz, gx, gy, gz);
    }
    const int b0 = T.boff[a], b1 = T.boff[a + 1];
    // Gather in chunks: issue every neighbour load of a chunk before consuming any, so
    // that the L1/L2 latencies of up to 3*SGB_GATHER loads overlap.
    for (int b = b0; b < b1; b += SGB_GATHER) {
        R tx[SGB_GATHER], ty[SGB_GATHER], tz[SGB_GATHER];
#pragma unroll
        for (int k = 0; k < SGB_GATHER; k++) {
            if (b + k < b1) {
                const DBond<R>& B = T.bonds[b + k];
                int x1, x2, x3;
                if (ANYWRAP) {
                    x1 = sgb_wrap_any(ix.c1 + B.n[0], L1);
                    x2 = sgb_wrap_any(ix.c2 + B.n[1], L2);
                    x3 = sgb_wrap_any(ix.c3 + B.n[2], L3);
                } else {
                    x1 = sgb_wrap_pos(ix.c1 + B.n[0], L1);
                    x2 = sgb_wrap_pos(ix.c2 + B.n[1], L2);
                    x3 = sgb_wrap_pos(ix.c3 + B.n[2], L3);
                }
                int js = x1 + L1 * (x2 + L2 * (x3 + L3 * B.j));
                tx[k] = sgb_ld(X + js); ty[k] = sgb_ld(Y + js); tz[k] = sgb_ld(Zc + js);
            }
        }
#pragma unroll
        for (int k = 0; k < SGB_GATHER; k++) {
            if (b + k >= b1) break;
            const DBond<R>& B = T.bonds[b + k];
            if (B.jkind == 0) {
                R j = B.J[0];
                gx += j * tx[k]; gy += j * ty[k]; gz += j * tz[k];
            } else {
                gx += B.J[0] * tx[k] + B.J[3] * ty[k] + B.J[6] * tz[k];
                gy += B.J[1] * tx[k] + B.J[4] * ty[k] + B.J[7] * tz[k];
                gz += B.J[2] * tx[k] + B.J[5] * ty[k] + B.J[8] * tz[k];
            }
            if (M.dipole_mode && B.bqkind != 0) {
                R Qj[5], v[5];
                quad5<R>(tx[k], ty[k], tz[k], Qj);
                if (B.bqkind == 1) {
#pragma unroll
                    for (int q = 0; q < 5; q++) v[q] = B.bq * ((R)biquad_metric(q) * Qj[q]);
                } else {
                    const R* Bm = T.bq + 25 * B.bqidx;
#pragma unroll
                    for (int q = 0; q < 5; q++) {
                        R acc = 0;
#pragma unroll
                        for (int p = 0; p < 5; p++) acc += Bm[q + 5 * p] * Qj[p];
                        v[q] = acc;
                    }
                }
                add_quad_grad<R>(sx, sy, sz, v, gx, gy, gz);
            }
        }
    }
}

// Batch form: site coordinates given directly, bond offsets unpacked from DBond::pk (one
// shared-memory load per bond), raw offsets wrapped for |n| <= L. GEN = false is the fast
// path for isotropic bilinear couplings without biquadratic terms.
template <class R, bool GEN>
__device__ inline void grad_batch(const Model<R>& M, const Tab<R>& T, int c1, int c2, int c3, int a, int L1, int L2,
                                  int L3, R hx, R hy, R hz, R sx, R sy, R sz, const R* X, const R* Y, const R* Zc,
                                  R& gx, R& gy, R& gz) {
    gx = hx; gy = hy; gz = hz;
    {
        int km = T.kmax[a];
        if (km > 0) classical_aniso<R>(T.stev + 28 * a, km, sx, sy, sz, gx, gy, gz);
    }
    const int b0 = T.boff[a], b1 = T.boff[a + 1];
    constexpr int G = 6;
    for (int b = b0; b < b1; b += G) {
        R tx[G], ty[G], tz[G];
#pragma unroll
        for (int k = 0; k < G; k++) {
            if (b + k < b1) {
                const int pk = T.bonds[b + k].pk;
                int x1 = sgb_wrap_any(c1 + (int)(pk & 0xff) - 128, L1);
                int x2 = sgb_wrap_any(c2 + (int)((pk >> 8) & 0xff) - 128, L2);
                int x3 = sgb_wrap_any(c3 + (int)((pk >> 16) & 0xff) - 128, L3);
                int js = x1 + L1 * (x2 + L2 * (x3 + L3 * (int)((unsigned)pk >> 24)));
                tx[k] = sgb_ld(X + js); ty[k] = sgb_ld(Y + js); tz[k] = sgb_ld(Zc + js);
            }
        }
#pragma unroll
        for (int k = 0; k < G; k++) {
            if (b + k >= b1) break;
            const DBond<R>& B = T.bonds[b + k];
            if (!GEN) {
                R j = B.J[0];
                gx += j * tx[k]; gy += j * ty[k]; gz += j * tz[k];
                continue;
            }
            if (B.jkind == 0) {
                R j = B.J[0];
                gx += j * tx[k]; gy += j * ty[k]; gz += j * tz[k];
            } else {
                gx += B.J[0] * tx[k] + B.J[3] * ty[k] + B.J[6] * tz[k];
                gy += B.J[1] * tx[k] + B.J[4] * ty[k] + B.J[7] * tz[k];
                gz += B.J[2] * tx[k] + B.J[5] * ty[k] + B.J[8] * tz[k];
            }
            if (M.dipole_mode && B.bqkind != 0) {
                R Qj[5], v[5];
                quad5<R>(tx[k], ty[k], tz[k], Qj);
                if (B.bqkind == 1) {
#pragma unroll
                    for (int q = 0; q < 5; q++) v[q] = B.bq * ((R)biquad_metric(q) * Qj[q]);
                } else {
                    const R* Bm = T.bq + 25 * B.bqidx;
#pragma unroll
                    for (int q = 0; q < 5; q++) {
                        R acc = 0;
#pragma unroll
                        for (int p = 0; p < 5; p++) acc += Bm[q + 5 * p] * Qj[p];
                        v[q] = acc;
                    }
                }
                add_quad_grad<R>(sx, sy, sz, v, gx, gy, gz);
            }
        }
    }
}

// Table form: the neighbour of local site s along the k-th bond of its sublattice is
// nb[k * nsr + s] (precomputed with the periodic wrap), so a bond costs one coalesced
// index load instead of the wrap arithmetic. Used by the replica-batch kernels.
template <class R, bool GEN>
__device__ inline void grad_table(const Model<R>& M, const Tab<R>& T, int a, int s, const int* nb, int nsr,
                                  R hx, R hy, R hz, R sx, R sy, R sz, const R* X, const R* Y, const R* Zc,
                                  R& gx, R& gy, R& gz);

// Gradient of one site from a neighbour-index source: nbi(k) is the site index (within
// the replica) of the k-th bond of sublattice a, and nld(j, x, y, z) loads the spin of
// site j. Neighbour spins are fetched G bonds at a time so that their loads are in
// flight together.
template <class R, bool GEN, int G, class NBI, class NLD>
__device__ __forceinline__ void grad_nbi_ld(const Model<R>& M, const Tab<R>& T, int a, NBI nbi, NLD nld, R hx, R hy,
                                            R hz, R sx, R sy, R sz, R& gx, R& gy, R& gz) {
    gx = hx; gy = hy; gz = hz;
    {
        int km = T.kmax[a];
        if (km > 0) classical_aniso<R>(T.stev + 28 * a, km, sx, sy, sz, gx, gy, gz);
    }
    const int b0 = T.boff[a], b1 = T.boff[a + 1];
    for (int b = b0; b < b1; b += G) {
        int js[G];
#pragma unroll
        for (int k = 0; k < G; k++)
            if (b + k < b1) js[k] = nbi(b + k - b0);
        R tx[G], ty[G], tz[G];
#pragma unroll
        for (int k = 0; k < G; k++) {
            if (b + k < b1) nld(js[k], tx[k], ty[k], tz[k]);
        }
#pragma unroll
        for (int k = 0; k < G; k++) {
            if (b + k >= b1) break;
            const DBond<R>& B = T.bonds[b + k];
            if (!GEN) {
                R j = B.J[0];
                gx += j * tx[k]; gy += j * ty[k]; gz += j * tz[k];
                continue;
            }
            if (B.jkind == 0) {
                R j = B.J[0];
                gx += j * tx[k]; gy += j * ty[k]; gz += j * tz[k];
            } else {
                gx += B.J[0] * tx[k] + B.J[3] * ty[k] + B.J[6] * tz[k];
                gy += B.J[1] * tx[k] + B.J[4] * ty[k] + B.J[7] * tz[k];
                gz += B.J[2] * tx[k] + B.J[5] * ty[k] + B.J[8] * tz[k];
            }
            if (M.dipole_mode && B.bqkind != 0) {
                R Qj[5], v[5];
                quad5<R>(tx[k], ty[k], tz[k], Qj);
                if (B.bqkind == 1) {
#pragma unroll
                    for (int q = 0; q < 5; q++) v[q] = B.bq * ((R)biquad_metric(q) * Qj[q]);
                } else {
                    const R* Bm = T.bq + 25 * B.bqidx;
#pragma unroll
                    for (int q = 0; q < 5; q++) {
                        R acc = 0;
#pragma unroll
                        for (int p = 0; p < 5; p++) acc += Bm[q + 5 * p] * Qj[p];
                        v[q] = acc;
                    }
                }
                add_quad_grad<R>(sx, sy, sz, v, gx, gy, gz);
            }
        }
    }
}

// Spins in SoA form: X[j], Y[j], Zc[j].
template <class R, bool GEN, int G, class NBI>
__device__ __forceinline__ void grad_nbi(const Model<R>& M, const Tab<R>& T, int a, NBI nbi, R hx, R hy, R hz,
                                         R sx, R sy, R sz, const R* X, const R* Y, const R* Zc, R& gx, R& gy,
                                         R& gz) {
    grad_nbi_ld<R, GEN, G>(
        M, T, a, nbi,
        [X, Y, Zc](int j, R& x, R& y, R& z) {
            x = sgb_ld(X + j); y = sgb_ld(Y + j); z = sgb_ld(Zc + j);
        },
        hx, hy, hz, sx, sy, sz, gx, gy, gz);
}

template <class R, bool GEN>
__device__ inline void grad_table(const Model<R>& M, const Tab<R>& T, int a, int s, const int* nb, int nsr,
                                  R hx, R hy, R hz, R sx, R sy, R sz, const R* X, const R* Y, const R* Zc,
                                  R& gx, R& gy, R& gz) {
    const int* p = nb + s;
    grad_nbi<R, GEN, 6>(M, T, a, [p, nsr](int k) { return __ldg(p + (size_t)k * nsr); }, hx, hy, hz, sx, sy, sz,
                        X, Y, Zc, gx, gy, gz);
}

template <class R, class NLD>
__device__ inline void grad_inh(const Model<R>& M, const Tab<R>& T, int site, NLD nld, R sx, R sy, R sz, R& gx, R& gy,
                                R& gz);

// Single-system table form: per-site Zeeman field from M.h and the neighbour table M.nbr.
template <class R>
__device__ inline void grad_single(const Model<R>& M, const Tab<R>& T, int site, R sx, R sy, R sz, const R* X,
                                   const R* Y, const R* Zc, R& gx, R& gy, R& gz) {
    if (M.ioff || M.oidx) {
        grad_inh<R>(M, T, site, [X, Y, Zc](int j, R& x, R& y, R& z) {
            x = sgb_ld(X + j); y = sgb_ld(Y + j); z = sgb_ld(Zc + j);
        }, sx, sy, sz, gx, gy, gz);
        return;
    }
    R hx = 0, hy = 0, hz = 0;
    if (M.h) {
        hx = __ldg(M.h + site);
        hy = __ldg(M.h + M.ns + site);
        hz = __ldg(M.h + 2 * M.ns + site);
    }
    const int a = site / M.ncell;
    if (M.general) grad_table<R, true>(M, T, a, site, M.nbr, M.ns, hx, hy, hz, sx, sy, sz, X, Y, Zc, gx, gy, gz);
    else grad_table<R, false>(M, T, a, site, M.nbr, M.ns, hx, hy, hz, sx, sy, sz, X, Y, Zc, gx, gy, gz);
}

// Single-system form: per-site Zeeman field from M.h, offsets pre-reduced mod dims.
template <class R>
__device__ inline void grad_site(const Model<R>& M, const Tab<R>& T, int site, const SiteIdx& ix,
                                 R sx, R sy, R sz, const R* X, const R* Y, const R* Zc,
                                 R& gx, R& gy, R& gz) {
    R hx = 0, hy = 0, hz = 0;
    if (M.h) {
        hx = __ldg(M.h + site);
        hy = __ldg(M.h + M.ns + site);
        hz = __ldg(M.h + 2 * M.ns + site);
    }
    grad_site_L<R, false>(M, T, ix, M.L1, M.L2, M.L3, hx, hy, hz, sx, sy, sz, X, Y, Zc, gx, gy, gz);
}

// ---- inhomogeneous systems: per-site coupling rows ------------------------------------
// Visits the couplings of `site`: its own CSR entries when the system is inhomogeneous,
// else the rows of its sublattice with neighbours from the table M.nbr. f(B, bq, j) gets
// the coupling row, the base of its biquadratic matrices and the neighbour site.
template <class R, class F>
__device__ __forceinline__ void for_site_bonds(const Model<R>& M, const Tab<R>& T, int site, int a, F f) {
    if (M.ioff) {
        const int e1 = __ldg(M.ioff + site + 1);
        for (int e = __ldg(M.ioff + site); e < e1; e++) {
            const int2 en = __ldg(M.ient + e);
            f(M.ctab[en.y], M.cbq, en.x);
        }
    } else {
        const int b0 = T.boff[a], b1 = T.boff[a + 1];
        for (int b = b0; b < b1; b++) f(T.bonds[b], T.bq, __ldg(M.nbr + (size_t)(b - b0) * M.ns + site));
    }
}

// Stevens coefficients (and highest rank) of the onsite coupling at `site`.
template <class R>
__device__ __forceinline__ const R* stevens_at(const Model<R>& M, const Tab<R>& T, int site, int a, int& kmax) {
    if (M.oidx) {
        const int o = __ldg(M.oidx + site);
        kmax = __ldg(M.okmax + o);
        return M.otab + 28 * (size_t)o;
    }
    kmax = T.kmax[a];
    return T.stev + 28 * a;
}

// J·t (+ biquadratic dE/dS at s) of one coupling row on neighbour spin t.
template <class R>
__device__ __forceinline__ void bond_grad(const Model<R>& M, const DBond<R>& B, const R* bqtab, R sx, R sy, R sz, R tx,
                                          R ty, R tz, R& gx, R& gy, R& gz) {
    if (B.jkind == 0) {
        const R j = B.J[0];
        gx += j * tx; gy += j * ty; gz += j * tz;
    } else {
        gx += B.J[0] * tx + B.J[3] * ty + B.J[6] * tz;
        gy += B.J[1] * tx + B.J[4] * ty + B.J[7] * tz;
        gz += B.J[2] * tx + B.J[5] * ty + B.J[8] * tz;
    }
    if (M.dipole_mode && B.bqkind != 0) {
        R Qj[5], v[5];
        quad5<R>(tx, ty, tz, Qj);
        if (B.bqkind == 1) {
#pragma unroll
            for (int q = 0; q < 5; q++) v[q] = B.bq * ((R)biquad_metric(q) * Qj[q]);
        } else {
            const R* Bm = bqtab + 25 * B.bqidx;
#pragma unroll
            for (int q = 0; q < 5; q++) {
                R acc = 0;
#pragma unroll
                for (int p = 0; p < 5; p++) acc += Bm[q + 5 * p] * Qj[p];
                v[q] = acc;
            }
        }
        add_quad_grad<R>(sx, sy, sz, v, gx, gy, gz);
    }
}

// dE/dS at `site` of a system with per-site couplings (set_energy_grad_dipoles! with
// interactions_union[site], Interactions.jl:535-540); nld(j, x, y, z) loads spin j.
template <class R, class NLD>
__device__ inline void grad_inh(const Model<R>& M, const Tab<R>& T, int site, NLD nld, R sx, R sy, R sz, R& gx, R& gy,
                                R& gz) {
    gx = 0; gy = 0; gz = 0;
    if (M.h) {
        gx = __ldg(M.h + site);
        gy = __ldg(M.h + M.ns + site);
        gz = __ldg(M.h + 2 * M.ns + site);
    }
    const int a = site / M.ncell;
    if (M.dipole_mode) {
        int km;
        const R* c = stevens_at<R>(M, T, site, a, km);
        if (km > 0) classical_aniso<R>(c, km, sx, sy, sz, gx, gy, gz);
    }
    for_site_bonds<R>(M, T, site, a, [&](const DBond<R>& B, const R* bq, int j) {
        R tx, ty, tz;
        nld(j, tx, ty, tz);
        bond_grad<R>(M, B, bq, sx, sy, sz, tx, ty, tz, gx, gy, gz);
    });
}

// Integrators.jl:266-275 rhs_dipole!
template <class R>
__device__ __forceinline__ void rhs_dipole(R sx, R sy, R sz, R xx, R xy, R xz, R gx, R gy, R gz,
                                           R dt, R lam, R& dx, R& dy, R& dz) {
    R wx, wy, wz;
    if (lam == (R)0) {
        wx = dt * gx; wy = dt * gy; wz = dt * gz;
    } else {
        R cx = sy * gz - sz * gy, cy = sz * gx - sx * gz, cz = sx * gy - sy * gx;
        R dl = dt * lam;
        wx = xx + dt * gx - dl * cx;
        wy = xy + dt * gy - dl * cy;
        wz = xz + dt * gz - dl * cz;
    }
    dx = -(sy * wz - sz * wy);
    dy = -(sz * wx - sx * wz);
    dz = -(sx * wy - sy * wx);
}

// System.jl:421-423 normalize_dipole
template <class R>
__device__ __forceinline__ void normalize_dip(R& x, R& y, R& z, R kappa) {
    if (kappa == (R)0) { x = 0; y = 0; z = 0; return; }
    R f = kappa * sgb_rsqrt<R>(x * x + y * y + z * z);
    x *= f; y *= f; z *= f;
}

// LocalSampler with dipole-dipole interactions (ewald_energy_delta, Ewald.jl:210-241), with
// the field F = dE/dS of every site kept current: the change of the dipole-dipole energy
// when the (expected) dipole of `site` changes by d is d·F_site + ½ Δμ·A[0,i,i]·Δμ with
// Δμ = -g_site d. Writes g_site d (= -Δμ, the moved moment's change up to sign) to gd.
// E.Areal: [(a_i na + a_j) 9 + row + 3 col][cell offset of j's cell from i's].
__device__ __forceinline__ double ewald_site_delta(const EwaldDev& E, const double* F, int site, int ncell,
                                                   const double d[3], double gd[3]) {
    const double* gi = E.g + 9 * (size_t)site;
    const int ai = site / ncell;
    double dmu[3], ad[3];
    for (int r = 0; r < 3; r++) dmu[r] = -(gi[r] * d[0] + gi[r + 3] * d[1] + gi[r + 6] * d[2]);
    const size_t c0 = (size_t)((ai * E.na + ai) * 9) * ncell;
    for (int r = 0; r < 3; r++)
        ad[r] = E.Areal[c0 + (size_t)r * ncell] * dmu[0] + E.Areal[c0 + (size_t)(r + 3) * ncell] * dmu[1] +
                E.Areal[c0 + (size_t)(r + 6) * ncell] * dmu[2];
    const double* f = F + 3 * (size_t)site;
    for (int r = 0; r < 3; r++) gd[r] = -dmu[r];
    return d[0] * f[0] + d[1] * f[1] + d[2] * f[2] + 0.5 * (dmu[0] * ad[0] + dmu[1] * ad[1] + dmu[2] * ad[2]);
}

// After an accepted move at `site` with moment change gd = g_site ΔS, the threads of one
// block add F_j += g_jᵀ A[cell_site - cell_j, a_j, a_site] gd to every site j's field.
__device__ __forceinline__ void ewald_field_update(const EwaldDev& E, double* F, int site, int ns, int ncell,
                                                   const double gd[3]) {
    const int L1 = E.L[0], L2 = E.L[1], L3 = E.L[2], na = E.na;
    const int as = site / ncell, cs = site % ncell;
    const int xs = cs % L1, ys = (cs / L1) % L2, zs = cs / (L1 * L2);
    for (int j = threadIdx.x; j < ns; j += blockDim.x) {
        const int aj = j / ncell, cj = j % ncell;
        const int off = sgb_wrap_any(xs - cj % L1, L1) +
                        L1 * (sgb_wrap_any(ys - (cj / L1) % L2, L2) + L2 * sgb_wrap_any(zs - cj / (L1 * L2), L3));
        const size_t c0 = (size_t)((aj * na + as) * 9) * ncell + off;
        double am[3];
        for (int r = 0; r < 3; r++)
            am[r] = E.Areal[c0 + (size_t)r * ncell] * gd[0] + E.Areal[c0 + (size_t)(r + 3) * ncell] * gd[1] +
                    E.Areal[c0 + (size_t)(r + 6) * ncell] * gd[2];
        const double* gj = E.g + 9 * (size_t)j;
        for (int r = 0; r < 3; r++) F[3 * (size_t)j + r] += gj[3 * r] * am[0] + gj[3 * r + 1] * am[1] + gj[3 * r + 2] * am[2];
    }
}

}  // namespace sgbdev
