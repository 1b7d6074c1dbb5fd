// sgb_sun.cu -- SU(N) coherent-state kernels for sm_103a.
//
// Reference algorithms (Sunny.jl v0.9.2):
//   HZ = dE/dZbar     src/System/Interactions.jl:596-669
//   spin algebra      src/Operators/Spin.jl:72-167
//   energy            src/System/Interactions.jl:401-508
//   Langevin Heun     src/Integrators.jl:277-298, 335-357; proj MathBasics.jl:62
//   Schrodinger midpoint src/Integrators.jl:361-371, 422-452
//
// In SU(N) mode neighbours interact through expected dipoles (bilinear and Zeeman terms),
// expected Stevens quadrupoles (biquadratic terms) and, for general couplings
// (Σ_k A_k ⊗ B_k), expectations of arbitrary operators. Each thread therefore keeps its
// sites' coherent states Z in registers for the whole persistent launch and publishes
// <Z|S|Z> (3 reals), when biquadratic or general couplings exist <Z|O2q|Z> (5 reals), and
// with general couplings the packed density zz^† (N^2 reals) per site through
// L2-resident SoA buffers.
#include <cooperative_groups.h>

#include <algorithm>

#include "sgb_device.cuh"

namespace cg = cooperative_groups;

namespace {
using namespace sgbdev;

template <class R>
struct Cx { R re, im; };

template <class R> __device__ __forceinline__ Cx<R> cmul(Cx<R> a, Cx<R> b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }

// Spin-s matrix elements for N = 2s+1 (Spin.jl:1-14): off[j] couples levels j and j+1.
template <class R, int N>
struct SpinConst {
    R off[N > 1 ? N - 1 : 1];
    R sz[N];
    __device__ SpinConst() {
        const double s = (N - 1) / 2.0;
#pragma unroll
        for (int j = 1; j <= N - 1; j++) off[j - 1] = (R)(sqrt(2 * (s + 1) * j - (double)j * (j + 1)) / 2);
#pragma unroll
        for (int k = 0; k < N; k++) sz[k] = (R)(s - k);
    }
};

// <Z|S|Z> (Spin.jl:72-87)
template <class R, int N>
__device__ __forceinline__ void expected_spin(const SpinConst<R, N>& sc, const R* z, R& nx, R& ny, R& nz) {
    R cr = 0, ci = 0, zz = 0;
#pragma unroll
    for (int j = 0; j < N - 1; j++) {
        // conj(z_j) * off_j * z_{j+1}
        R ar = z[2 * j], ai = z[2 * j + 1], br = sc.off[j] * z[2 * j + 2], bi = sc.off[j] * z[2 * j + 3];
        cr += ar * br + ai * bi;
        ci += ar * bi - ai * br;
    }
#pragma unroll
    for (int k = 0; k < N; k++) zz += sc.sz[k] * (z[2 * k] * z[2 * k] + z[2 * k + 1] * z[2 * k + 1]);
    nx = 2 * cr; ny = 2 * ci; nz = zz;
}

// <Z|O2q|Z> (Spin.jl:90-104); qm: R[5][N*N][2] column-major
template <class R, int N>
__device__ __forceinline__ void expected_quad(const R* qm, const R* z, R* Q) {
#pragma unroll
    for (int a = 0; a < 5; a++) {
        R acc = 0;
        const R* O = qm + a * 2 * N * N;
#pragma unroll
        for (int c = 0; c < N; c++) {
            // (O z)_r summed against conj(z_r)
#pragma unroll
            for (int r = 0; r < N; r++) {
                R orr = O[2 * (r + N * c)], oi = O[2 * (r + N * c) + 1];
                R tr = orr * z[2 * c] - oi * z[2 * c + 1];
                R ti = orr * z[2 * c + 1] + oi * z[2 * c];
                acc += z[2 * r] * tr + z[2 * r + 1] * ti;
            }
        }
        Q[a] = acc;
    }
}

// HZ = (Λ + d.S) Z + sum_q v_q O2q Z  (Spin.jl:132-167)
template <class R, int N, bool BQ>
__device__ __forceinline__ void apply_H(const SpinConst<R, N>& sc, const R* lam, const R* qm, const R* d,
                                        const R* v, const R* z, R* hz) {
#pragma unroll
    for (int r = 0; r < N; r++) {
        R ar = 0, ai = 0;
#pragma unroll
        for (int c = 0; c < N; c++) {
            R hr = lam[2 * (r + N * c)], hi = lam[2 * (r + N * c) + 1];
            if (BQ) {
#pragma unroll
                for (int q = 0; q < 5; q++) {
                    hr += v[q] * qm[q * 2 * N * N + 2 * (r + N * c)];
                    hi += v[q] * qm[q * 2 * N * N + 2 * (r + N * c) + 1];
                }
            }
            ar += hr * z[2 * c] - hi * z[2 * c + 1];
            ai += hr * z[2 * c + 1] + hi * z[2 * c];
        }
        // dz * sz_r * z_r
        ar += d[2] * sc.sz[r] * z[2 * r];
        ai += d[2] * sc.sz[r] * z[2 * r + 1];
        if (r + 1 < N) {  // (dx - i dy) off_r z_{r+1}
            R o = sc.off[r];
            R pr = o * d[0], pi = -o * d[1];
            ar += pr * z[2 * r + 2] - pi * z[2 * r + 3];
            ai += pr * z[2 * r + 3] + pi * z[2 * r + 2];
        }
        if (r > 0) {  // (dx + i dy) off_{r-1} z_{r-1}
            R o = sc.off[r - 1];
            R pr = o * d[0], pi = o * d[1];
            ar += pr * z[2 * r - 2] - pi * z[2 * r - 1];
            ai += pr * z[2 * r - 1] + pi * z[2 * r - 2];
        }
        hz[2 * r] = ar;
        hz[2 * r + 1] = ai;
    }
}

// dE/dS (Zeeman + bilinear) from neighbours' dipoles, and the summed dE/dQ of the
// biquadratic couplings from neighbours' quadrupoles (Interactions.jl:596-669).
template <class R, bool BQ>
__device__ __forceinline__ void sun_field(const Model<R>& M, const Tab<R>& T, int site, const SiteIdx& ix,
                                          const R* D, const R* Qb, R* d, R* v) {
    const int ns = M.ns;
    d[0] = 0; d[1] = 0; d[2] = 0;
    if (M.h) { d[0] = __ldg(M.h + site); d[1] = __ldg(M.h + ns + site); d[2] = __ldg(M.h + 2 * ns + site); }
    if (BQ) {
#pragma unroll
        for (int q = 0; q < 5; q++) v[q] = 0;
    }
    const int b0 = T.boff[ix.a], b1 = T.boff[ix.a + 1];
    for (int b = b0; b < b1; b += SGB_GATHER) {
        R tx[SGB_GATHER], ty[SGB_GATHER], tz[SGB_GATHER];
        int jsv[SGB_GATHER];
#pragma unroll
        for (int k = 0; k < SGB_GATHER; k++) {
            if (b + k < b1) {
                const DBond<R>& B = T.bonds[b + k];
                int x1 = sgb_wrap_pos(ix.c1 + B.n[0], M.L1);
                int x2 = sgb_wrap_pos(ix.c2 + B.n[1], M.L2);
                int x3 = sgb_wrap_pos(ix.c3 + B.n[2], M.L3);
                int js = x1 + M.L1 * (x2 + M.L2 * (x3 + M.L3 * B.j));
                jsv[k] = js;
                tx[k] = sgb_ld(D + js); ty[k] = sgb_ld(D + ns + js); tz[k] = sgb_ld(D + 2 * ns + js);
            }
        }
#pragma unroll
        for (int k = 0; k < SGB_GATHER; k++) {
            if (b + k >= b1) break;
            const DBond<R>& B = T.bonds[b + k];
            if (B.jkind == 0) {
                R j = B.J[0];
                d[0] += j * tx[k]; d[1] += j * ty[k]; d[2] += j * tz[k];
            } else {
                d[0] += B.J[0] * tx[k] + B.J[3] * ty[k] + B.J[6] * tz[k];
                d[1] += B.J[1] * tx[k] + B.J[4] * ty[k] + B.J[7] * tz[k];
                d[2] += B.J[2] * tx[k] + B.J[5] * ty[k] + B.J[8] * tz[k];
            }
            if (BQ && B.bqkind != 0) {
                R Qj[5];
#pragma unroll
                for (int q = 0; q < 5; q++) Qj[q] = sgb_ld(Qb + (size_t)q * ns + jsv[k]);
                if (B.bqkind == 1) {
#pragma unroll
                    for (int q = 0; q < 5; q++) v[q] += B.bq * ((R)biquad_metric(q) * Qj[q]);
                } else {
                    const R* Bm = T.bq + 25 * B.bqidx;
#pragma unroll
                    for (int q = 0; q < 5; q++) {
                        R acc = 0;
#pragma unroll
                        for (int p = 0; p < 5; p++) acc += Bm[q + 5 * p] * Qj[p];
                        v[q] += acc;
                    }
                }
            }
        }
    }
}

// Integrators.jl:277-286 rhs_sun!, with proj (MathBasics.jl:62)
template <class R, int N>
__device__ __forceinline__ void rhs_sun(const R* z, const R* ze, const R* hz, R dt, R lam, R* dz) {
    if (lam == (R)0) {
#pragma unroll
        for (int k = 0; k < N; k++) { dz[2 * k] = dt * hz[2 * k + 1]; dz[2 * k + 1] = -dt * hz[2 * k]; }
        return;
    }
    R v[2 * N];
#pragma unroll
    for (int k = 0; k < N; k++) {
        // ζ + dt (i + λ) hz
        R hr = hz[2 * k], hi = hz[2 * k + 1];
        v[2 * k] = ze[2 * k] + dt * (lam * hr - hi);
        v[2 * k + 1] = ze[2 * k + 1] + dt * (hr + lam * hi);
    }
    R nr = 0, ni = 0, nn = 0;
#pragma unroll
    for (int k = 0; k < N; k++) {
        nr += z[2 * k] * v[2 * k] + z[2 * k + 1] * v[2 * k + 1];
        ni += z[2 * k] * v[2 * k + 1] - z[2 * k + 1] * v[2 * k];
        nn += z[2 * k] * z[2 * k] + z[2 * k + 1] * z[2 * k + 1];
    }
    R fr = nr / nn, fi = ni / nn;
#pragma unroll
    for (int k = 0; k < N; k++) {
        R pr = z[2 * k] * fr - z[2 * k + 1] * fi, pi = z[2 * k] * fi + z[2 * k + 1] * fr;
        dz[2 * k] = -(v[2 * k] - pr);
        dz[2 * k + 1] = -(v[2 * k + 1] - pi);
    }
}

// System.jl:416-418 normalize_ket: Z / sqrt(|Z|^2/κ)
template <class R, int N>
__device__ __forceinline__ void normalize_ket(R* z, R kappa) {
    if (kappa == (R)0) {
#pragma unroll
        for (int k = 0; k < 2 * N; k++) z[k] = 0;
        return;
    }
    R n2 = 0;
#pragma unroll
    for (int k = 0; k < N; k++) n2 += z[2 * k] * z[2 * k] + z[2 * k + 1] * z[2 * k + 1];
    if constexpr (sizeof(R) == 8) {
        R d = sqrt(n2 / kappa);
#pragma unroll
        for (int k = 0; k < 2 * N; k++) z[k] = z[k] / d;
    } else {
        R f = sqrtf(kappa) * rsqrtf(n2);
#pragma unroll
        for (int k = 0; k < 2 * N; k++) z[k] *= f;
    }
}

template <class R, int N>
struct SunTab {
    Tab<R> t;
    const R* lam;   // [na][N*N][2]
    const R* qm;    // [5][N*N][2]
};

template <class R, int N>
__device__ inline SunTab<R, N> stage_sun(const Model<R>& M, unsigned char* smem) {
    SunTab<R, N> s;
    s.t = stage_tables<R>(M, smem);
    s.lam = reinterpret_cast<const R*>(smem + M.off_lam);
    s.qm = reinterpret_cast<const R*>(smem + M.off_qmat);
    return s;
}

// Packed density of a ket, ρ = z z^†: |z_r|^2 for r < N, then for each r < c the real and
// imaginary parts of z_c conj(z_r). <M> = Σ_rc conj(z_r) M_rc z_c = a(M)·ρ with a(M) =
// (Re M_rr; 2 Re M_rc, -2 Im M_rc).
template <class R, int N>
__device__ __forceinline__ void sun_rho(const R* z, R* rho) {
#pragma unroll
    for (int r = 0; r < N; r++) rho[r] = z[2 * r] * z[2 * r] + z[2 * r + 1] * z[2 * r + 1];
    int k = N;
#pragma unroll
    for (int r = 0; r < N; r++)
#pragma unroll
        for (int c = r + 1; c < N; c++) {
            rho[k++] = z[2 * c] * z[2 * r] + z[2 * c + 1] * z[2 * r + 1];
            rho[k++] = z[2 * c + 1] * z[2 * r] - z[2 * c] * z[2 * r + 1];
        }
}

// Dipoles (and with BQ quadrupoles, and with rho the packed density ρ in rows 5..5+N^2) of
// ket z, for neighbours to read.
template <class R, int N, bool BQ>
__device__ __forceinline__ void publish(const SpinConst<R, N>& sc, const R* qm, const R* z, int ns, int site, R* D, R* Qb,
                                        bool rho = false) {
    R nx, ny, nz;
    expected_spin<R, N>(sc, z, nx, ny, nz);
    D[site] = nx; D[ns + site] = ny; D[2 * ns + site] = nz;
    if (BQ) {
        R q[5];
        expected_quad<R, N>(qm, z, q);
#pragma unroll
        for (int a = 0; a < 5; a++) Qb[(size_t)a * ns + site] = q[a];
        if (rho) {
            R p[N * N];
            sun_rho<R, N>(z, p);
#pragma unroll
            for (int a = 0; a < N * N; a++) Qb[(size_t)(5 + a) * ns + site] = p[a];
        }
    }
}

// General pair couplings (Interactions.jl:660-666): hz += Σ_bonds Σ_terms <B>_j (A z), with
// <B>_j from the neighbour's published density.
template <class R, int N>
__device__ __forceinline__ void general_HZ(const Model<R>& M, const Tab<R>& T, int site, int a, const R* Qb, const R* z,
                                           R* hz) {
    const int ns = M.ns, b0 = T.boff[a], b1 = T.boff[a + 1];
    for (int b = b0; b < b1; b++) {
        const DBond<R>& B = T.bonds[b];
        if (dbond_gcnt(B) == 0) continue;
        const int j = __ldg(M.nbr + (size_t)(b - b0) * ns + site);
        R rj[N * N];
#pragma unroll
        for (int k = 0; k < N * N; k++) rj[k] = sgb_ld(Qb + (size_t)(5 + k) * ns + j);
        for (int t = 0; t < dbond_gcnt(B); t++) {
            const R* row = M.gtab + (size_t)(dbond_gidx(B) + t) * 4 * N * N;
            const R* Am = row + N * N;
            const R* bv = row + 3 * N * N;
            R Bb = 0;
#pragma unroll
            for (int k = 0; k < N * N; k++) Bb += __ldg(bv + k) * rj[k];
#pragma unroll
            for (int r = 0; r < N; r++) {
                R ar = 0, ai = 0;
#pragma unroll
                for (int c = 0; c < N; c++) {
                    const R mr = __ldg(Am + 2 * (r + N * c)), mi = __ldg(Am + 2 * (r + N * c) + 1);
                    ar += mr * z[2 * c] - mi * z[2 * c + 1];
                    ai += mr * z[2 * c + 1] + mi * z[2 * c];
                }
                hz[2 * r] += Bb * ar;
                hz[2 * r + 1] += Bb * ai;
            }
        }
    }
}

// Λ of the onsite coupling at `site`: its own row (inhomogeneous systems) or its sublattice's.
template <class R, int N>
__device__ __forceinline__ const R* lam_at(const Model<R>& M, const SunTab<R, N>& S, int site, int a) {
    return M.oidx ? M.otab + (size_t)2 * N * N * __ldg(M.oidx + site) : S.lam + a * 2 * N * N;
}

// sun_field over the site's own coupling rows (inhomogeneous systems).
template <class R, bool BQ>
__device__ __forceinline__ void sun_field_inh(const Model<R>& M, const Tab<R>& T, int site, int a, const R* D,
                                              const R* Qb, R* d, R* v) {
    const int ns = M.ns;
    d[0] = 0; d[1] = 0; d[2] = 0;
    if (M.h) { d[0] = __ldg(M.h + site); d[1] = __ldg(M.h + ns + site); d[2] = __ldg(M.h + 2 * ns + site); }
    if (BQ) {
#pragma unroll
        for (int q = 0; q < 5; q++) v[q] = 0;
    }
    for_site_bonds<R>(M, T, site, a, [&](const DBond<R>& B, const R* bq, int js) {
        const R tx = sgb_ld(D + js), ty = sgb_ld(D + ns + js), tz = sgb_ld(D + 2 * ns + js);
        if (B.jkind == 0) {
            const R j = B.J[0];
            d[0] += j * tx; d[1] += j * ty; d[2] += j * tz;
        } else {
            d[0] += B.J[0] * tx + B.J[3] * ty + B.J[6] * tz;
            d[1] += B.J[1] * tx + B.J[4] * ty + B.J[7] * tz;
            d[2] += B.J[2] * tx + B.J[5] * ty + B.J[8] * tz;
        }
        if (BQ && B.bqkind != 0) {
            R Qj[5];
#pragma unroll
            for (int q = 0; q < 5; q++) Qj[q] = sgb_ld(Qb + (size_t)q * ns + js);
            if (B.bqkind == 1) {
#pragma unroll
                for (int q = 0; q < 5; q++) v[q] += B.bq * ((R)biquad_metric(q) * Qj[q]);
            } else {
                const R* Bm = bq + 25 * B.bqidx;
#pragma unroll
                for (int q = 0; q < 5; q++) {
                    R acc = 0;
#pragma unroll
                    for (int p = 0; p < 5; p++) acc += Bm[q + 5 * p] * Qj[p];
                    v[q] += acc;
                }
            }
        }
    });
}

template <class R, int N, bool BQ>
__device__ __forceinline__ void local_HZ(const Model<R>& M, const SunTab<R, N>& S, const SpinConst<R, N>& sc, int site,
                                         const R* D, const R* Qb, const R* z, R* hz) {
    SiteIdx ix = decompose(site, M.L1, M.L2, M.L3);
    R d[3], v[5];
    if (M.ioff) sun_field_inh<R, BQ>(M, S.t, site, ix.a, D, Qb, d, v);
    else sun_field<R, BQ>(M, S.t, site, ix, D, Qb, d, v);
    apply_H<R, N, BQ>(sc, lam_at<R, N>(M, S, site, ix.a), S.qm, d, v, z, hz);
    if (BQ && M.has_general) general_HZ<R, N>(M, S.t, site, ix.a, Qb, z, hz);
}

template <class R, int N, int SPT, bool INJECT, bool BQ>
__global__ void __launch_bounds__(sgb_maxblock(sizeof(R) == 8, true, SPT))
k_sun_heun(Model<R> M, R* Z, R* D, R* Qb, R* P, R* QP, Ctrl* ctrl, int nsteps, R dt, R lam, R nscale,
           uint64_t seed, uint64_t step0, const double* noise) {
    extern __shared__ __align__(16) unsigned char smem[];
    SunTab<R, N> S = stage_sun<R, N>(M, smem);
    SpinConst<R, N> sc;
    const int ns = M.ns;
    const int nthr = gridDim.x * blockDim.x;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    R z[SPT][2 * N], zp[SPT][2 * N], d1[SPT][2 * N], ze[SPT][2 * N];
#pragma unroll
    for (int k = 0; k < SPT; k++) {
        int site = tid + k * nthr;
        if (site >= ns) continue;
#pragma unroll
        for (int c = 0; c < 2 * N; c++) z[k][c] = Z[(size_t)c * ns + site];
    }
    for (int step = 0; step < nsteps; ++step) {
#pragma unroll
        for (int k = 0; k < SPT; k++) {
            int site = tid + k * nthr;
            if (site >= ns) continue;
            if (nscale == (R)0) {
#pragma unroll
                for (int c = 0; c < 2 * N; c++) ze[k][c] = 0;
            } else if (INJECT) {
                const double* nz = noise + ((size_t)step * ns + site) * 2 * N;
#pragma unroll
                for (int c = 0; c < 2 * N; c++) ze[k][c] = (R)nz[c] * nscale;
            } else {
                const R r2 = (R)0.70710678118654752440;
#pragma unroll
                for (int c = 0; c < 2 * N; c += 4) {
                    R g4[4];
                    sgb_normals4<R>(seed, 0u, step0 + step, (uint32_t)site, (uint32_t)(c / 4), g4);
#pragma unroll
                    for (int q = 0; q < 4; q++)
                        if (c + q < 2 * N) ze[k][c + q] = g4[q] * r2 * nscale;
                }
            }
            R hz[2 * N];
            local_HZ<R, N, BQ>(M, S, sc, site, D, Qb, z[k], hz);
            rhs_sun<R, N>(z[k], ze[k], hz, dt, lam, d1[k]);
#pragma unroll
            for (int c = 0; c < 2 * N; c++) zp[k][c] = z[k][c] + d1[k][c];
            normalize_ket<R, N>(zp[k], __ldg(M.kappa + site));
            publish<R, N, BQ>(sc, S.qm, zp[k], ns, site, P, QP, M.has_general);
        }
        if (!sgb_grid_barrier(ctrl, gridDim.x)) return;
#pragma unroll
        for (int k = 0; k < SPT; k++) {
            int site = tid + k * nthr;
            if (site >= ns) continue;
            R hz[2 * N], d2[2 * N];
            local_HZ<R, N, BQ>(M, S, sc, site, P, QP, zp[k], hz);
            rhs_sun<R, N>(zp[k], ze[k], hz, dt, lam, d2);
#pragma unroll
            for (int c = 0; c < 2 * N; c++) z[k][c] = z[k][c] + (d1[k][c] + d2[c]) / 2;
            normalize_ket<R, N>(z[k], __ldg(M.kappa + site));
            publish<R, N, BQ>(sc, S.qm, z[k], ns, site, D, Qb, M.has_general);
        }
        if (step + 1 < nsteps) {
            if (!sgb_grid_barrier(ctrl, gridDim.x)) return;
        }
    }
#pragma unroll
    for (int k = 0; k < SPT; k++) {
        int site = tid + k * nthr;
        if (site >= ns) continue;
#pragma unroll
        for (int c = 0; c < 2 * N; c++) Z[(size_t)c * ns + site] = z[k][c];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) ctrl->steps_done = nsteps;
}

template <class R, int N>
__device__ __forceinline__ void write_snapshot_sun(const Model<R>& M, const SnapArgs<R>& sn, int t, int site, const R* z) {
    const int ns = M.ns;
    const int cell = site % M.ncell, a = site / M.ncell;
    for (int o = 0; o < sn.nobs; o++) {
        const R* A = sn.ops + (size_t)o * 2 * N * N * ns;
        R acc = 0;
#pragma unroll
        for (int c = 0; c < N; c++)
#pragma unroll
            for (int r = 0; r < N; r++) {
                R ar = __ldg(A + (size_t)(2 * (r + N * c)) * ns + site);
                R ai = __ldg(A + (size_t)(2 * (r + N * c) + 1) * ns + site);
                R tr = ar * z[2 * c] - ai * z[2 * c + 1];
                R ti = ar * z[2 * c + 1] + ai * z[2 * c];
                acc += z[2 * r] * tr + z[2 * r + 1] * ti;
            }
        size_t idx = (((size_t)t * sn.nobs + o) * M.na + a) * M.ncell + cell;
        sn.buf[2 * idx] = acc * sn.scale;
        sn.buf[2 * idx + 1] = 0;
    }
}

// Schrodinger midpoint (Integrators.jl:422-452). H: 3 rotating [3][ns] dipole buffers of
// <Zbar|S|Zbar>; QH: 3 rotating [5][ns] quadrupole buffers.
template <class R, int N, int SPT, bool BQ>
__global__ void __launch_bounds__(sgb_maxblock(sizeof(R) == 8, true, SPT))
k_sun_midpoint(Model<R> M, R* Z, R* D, R* Qb, R* H, R* QH, Ctrl* ctrl, int nsteps, R dt, R lam,
               double atol2, int max_iters, SnapArgs<R> snap) {
    extern __shared__ __align__(16) unsigned char smem[];
    SunTab<R, N> S = stage_sun<R, N>(M, smem);
    SpinConst<R, N> sc;
    const int ns = M.ns;
    const int nthr = gridDim.x * blockDim.x;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const bool leader = (blockIdx.x == 0 && threadIdx.x == 0);
    R z[SPT][2 * N], zp[SPT][2 * N], zc[SPT][2 * N];
    int cur = 0;
#pragma unroll
    for (int k = 0; k < SPT; k++) {
        int site = tid + k * nthr;
        if (site >= ns) continue;
#pragma unroll
        for (int c = 0; c < 2 * N; c++) z[k][c] = Z[(size_t)c * ns + site];
        R zb[2 * N];
#pragma unroll
        for (int c = 0; c < 2 * N; c++) zb[c] = (z[k][c] + z[k][c]) / 2;
        publish<R, N, BQ>(sc, S.qm, zb, ns, site, H, QH, M.has_general);
        if (snap.enabled) write_snapshot_sun<R, N>(M, snap, snap.t0, site, z[k]);
    }
    if (leader) { ctrl->acc[0] = 0.0; ctrl->acc[1] = 0.0; ctrl->acc[2] = 0.0; }
    if (!sgb_grid_barrier(ctrl, gridDim.x)) return;
    long long itg = 0;
    int done = 0;
    for (int step = 0; step < nsteps; ++step) {
#pragma unroll
        for (int k = 0; k < SPT; k++)
#pragma unroll
            for (int c = 0; c < 2 * N; c++) zp[k][c] = z[k][c];
        bool conv = false;
        for (int it = 0; it < max_iters; ++it) {
            const int nxt = (cur + 1) % 3, nst = (cur + 2) % 3;
            const R* Hc = H + (size_t)cur * 3 * ns;
            const R* Qc = QH + (size_t)cur * M.qrows * ns;
            R acc = 0;   // per-site terms in R, block and grid sums in FP64
#pragma unroll
            for (int k = 0; k < SPT; k++) {
                int site = tid + k * nthr;
                if (site >= ns) continue;
                const R kap = __ldg(M.kappa + site);
                R zb[2 * N], hz[2 * N], dz[2 * N], zero[2 * N];
#pragma unroll
                for (int c = 0; c < 2 * N; c++) { zb[c] = (z[k][c] + zp[k][c]) / 2; zero[c] = 0; }
                local_HZ<R, N, BQ>(M, S, sc, site, Hc, Qc, zb, hz);
                rhs_sun<R, N>(zb, zero, hz, dt, lam, dz);
#pragma unroll
                for (int c = 0; c < 2 * N; c++) {
                    R q = z[k][c] + dz[c];
                    R e = zp[k][c] - q;
                    acc += e * e;
                    zp[k][c] = q;
                }
#pragma unroll
                for (int c = 0; c < 2 * N; c++) zb[c] = (z[k][c] + zp[k][c]) / 2;
                publish<R, N, BQ>(sc, S.qm, zb, ns, site, H + (size_t)nxt * 3 * ns, QH + (size_t)nxt * M.qrows * ns, M.has_general);
#pragma unroll
                for (int c = 0; c < 2 * N; c++) zc[k][c] = zp[k][c];
                normalize_ket<R, N>(zc[k], kap);
#pragma unroll
                for (int c = 0; c < 2 * N; c++) zb[c] = (zc[k][c] + zc[k][c]) / 2;
                publish<R, N, BQ>(sc, S.qm, zb, ns, site, H + (size_t)nst * 3 * ns, QH + (size_t)nst * M.qrows * ns, M.has_general);
            }
            double bsum = sgb_block_sum_r<R>(acc);
            const int slot = (int)(itg % 3);
            if (threadIdx.x == 0) atomicAdd(&ctrl->acc[slot], bsum);
            if (leader) { ctrl->acc[(slot + 1) % 3] = 0.0; ctrl->iters += 1; }
            if (!sgb_grid_barrier(ctrl, gridDim.x)) return;
            double tot = __ldcg(&ctrl->acc[slot]);
            itg++;
            if (tot <= atol2) {
                conv = true;
#pragma unroll
                for (int k = 0; k < SPT; k++)
#pragma unroll
                    for (int c = 0; c < 2 * N; c++) z[k][c] = zc[k][c];
                cur = nst;
                break;
            }
            cur = nxt;
        }
        if (!conv) {
            if (leader) sgb_set_status(ctrl, SGB_ERR_NOCONVERGE);
            break;
        }
        done = step + 1;
        if (snap.enabled && (done % snap.measperiod) == 0) {
#pragma unroll
            for (int k = 0; k < SPT; k++) {
                int site = tid + k * nthr;
                if (site < ns) write_snapshot_sun<R, N>(M, snap, snap.t0 + done / snap.measperiod, site, z[k]);
            }
        }
    }
#pragma unroll
    for (int k = 0; k < SPT; k++) {
        int site = tid + k * nthr;
        if (site >= ns) continue;
#pragma unroll
        for (int c = 0; c < 2 * N; c++) Z[(size_t)c * ns + site] = z[k][c];
        publish<R, N, BQ>(sc, S.qm, z[k], ns, site, D, Qb, M.has_general);
    }
    if (leader) ctrl->steps_done = done;
}

template <class R, int N>
__global__ void __launch_bounds__(SGB_BLOCK) k_sun_refresh(Model<R> M, const R* Z, R* D, R* Qb) {
    extern __shared__ __align__(16) unsigned char smem[];
    SunTab<R, N> S = stage_sun<R, N>(M, smem);
    SpinConst<R, N> sc;
    for (int site = blockIdx.x * blockDim.x + threadIdx.x; site < M.ns; site += gridDim.x * blockDim.x) {
        R z[2 * N];
#pragma unroll
        for (int c = 0; c < 2 * N; c++) z[c] = Z[(size_t)c * M.ns + site];
        if (M.has_biquad) publish<R, N, true>(sc, S.qm, z, M.ns, site, D, Qb, M.has_general);
        else publish<R, N, false>(sc, S.qm, z, M.ns, site, D, Qb);
    }
}

template <class R, int N>
__global__ void __launch_bounds__(SGB_BLOCK) k_sun_grad(Model<R> M, const R* Z, const R* D, const R* Qb, double* out) {
    extern __shared__ __align__(16) unsigned char smem[];
    SunTab<R, N> S = stage_sun<R, N>(M, smem);
    SpinConst<R, N> sc;
    for (int site = blockIdx.x * blockDim.x + threadIdx.x; site < M.ns; site += gridDim.x * blockDim.x) {
        R z[2 * N], hz[2 * N];
#pragma unroll
        for (int c = 0; c < 2 * N; c++) z[c] = Z[(size_t)c * M.ns + site];
        if (M.has_biquad) local_HZ<R, N, true>(M, S, sc, site, D, Qb, z, hz);
        else local_HZ<R, N, false>(M, S, sc, site, D, Qb, z, hz);
#pragma unroll
        for (int c = 0; c < 2 * N; c++) out[(size_t)site * 2 * N + c] = (double)hz[c];
    }
}

// FP64 energy (Interactions.jl:401-508), SU(N) mode: partials[block][4].
template <class R, int N>
__global__ void __launch_bounds__(SGB_BLOCK) k_sun_energy(Model<R> M, const R* Z, const R* D, const R* Qb, double* partials) {
    extern __shared__ __align__(16) unsigned char smem[];
    SunTab<R, N> S = stage_sun<R, N>(M, smem);
    const int ns = M.ns;
    double E = 0, mx = 0, my = 0, mz = 0;
    for (int site = blockIdx.x * blockDim.x + threadIdx.x; site < ns; site += gridDim.x * blockDim.x) {
        SiteIdx ix = decompose(site, M.L1, M.L2, M.L3);
        double sx = D[site], sy = D[ns + site], sz = D[2 * ns + site];
        mx += sx; my += sy; mz += sz;
        if (M.h) E += (double)M.h[site] * sx + (double)M.h[ns + site] * sy + (double)M.h[2 * ns + site] * sz;
        double z[2 * N];
#pragma unroll
        for (int c = 0; c < 2 * N; c++) z[c] = Z[(size_t)c * ns + site];
        const R* lam = lam_at<R, N>(M, S, site, ix.a);
        double eo = 0;
#pragma unroll
        for (int c = 0; c < N; c++)
#pragma unroll
            for (int r = 0; r < N; r++) {
                double ar = lam[2 * (r + N * c)], ai = lam[2 * (r + N * c) + 1];
                double tr = ar * z[2 * c] - ai * z[2 * c + 1], ti = ar * z[2 * c + 1] + ai * z[2 * c];
                eo += z[2 * r] * tr + z[2 * r + 1] * ti;
            }
        E += eo;
        double qi[5];
        if (M.has_biquad) {
            double qmd[5 * 2 * N * N];
            for (int q = 0; q < 5 * 2 * N * N; q++) qmd[q] = (double)S.qm[q];
            expected_quad<double, N>(qmd, z, qi);
        }
        const double ki = (double)M.kappa[site];
        auto bond_E = [&](const DBond<R>& B, const R* bqtab, int js) {
            double tx = D[js], ty = D[ns + js], tz = D[2 * ns + js];
            E += (double)B.scalar * ki * (double)M.kappa[js];
            if (B.jkind == 0) E += (double)B.J[0] * (sx * tx + sy * ty + sz * tz);
            else {
                double jx = (double)B.J[0] * tx + (double)B.J[3] * ty + (double)B.J[6] * tz;
                double jy = (double)B.J[1] * tx + (double)B.J[4] * ty + (double)B.J[7] * tz;
                double jz = (double)B.J[2] * tx + (double)B.J[5] * ty + (double)B.J[8] * tz;
                E += sx * jx + sy * jy + sz * jz;
            }
            if (M.has_biquad && B.bqkind != 0) {
                double zj[2 * N], qj[5], qmd[5 * 2 * N * N];
                for (int q = 0; q < 5 * 2 * N * N; q++) qmd[q] = (double)S.qm[q];
#pragma unroll
                for (int c = 0; c < 2 * N; c++) zj[c] = Z[(size_t)c * ns + js];
                expected_quad<double, N>(qmd, zj, qj);
                double acc = 0;
                if (B.bqkind == 1) {
                    for (int q = 0; q < 5; q++) acc += qi[q] * (biquad_metric(q) * qj[q]);
                    acc *= (double)B.bq;
                } else {
                    const R* Bm = bqtab + 25 * B.bqidx;
                    for (int q = 0; q < 5; q++)
                        for (int p = 0; p < 5; p++) acc += qi[q] * (double)Bm[q + 5 * p] * qj[p];
                }
                E += acc;
            }
            if (dbond_gcnt(B) > 0) {
                // general couplings (Interactions.jl:495-503): Σ_k <A_k>_i <B_k>_j
                double zj[2 * N], ri[N * N], rj[N * N];
#pragma unroll
                for (int c = 0; c < 2 * N; c++) zj[c] = Z[(size_t)c * ns + js];
                sun_rho<double, N>(z, ri);
                sun_rho<double, N>(zj, rj);
                for (int t = 0; t < dbond_gcnt(B); t++) {
                    const R* row = M.gtab + (size_t)(dbond_gidx(B) + t) * 4 * N * N;
                    double Ab = 0, Bb = 0;
                    for (int k = 0; k < N * N; k++) {
                        Ab += (double)row[k] * ri[k];
                        Bb += (double)row[3 * N * N + k] * rj[k];
                    }
                    E += Ab * Bb;
                }
            }
        };
        if (M.ioff) {
            for_site_bonds<R>(M, S.t, site, ix.a, [&](const DBond<R>& B, const R* bq, int js) {
                if (B.fwd) bond_E(B, bq, js);
            });
        } else {
            for (int b = S.t.boff[ix.a]; b < S.t.boff[ix.a + 1]; b++) {
                const DBond<R>& B = S.t.bonds[b];
                if (!B.fwd) continue;
                int x1 = sgb_wrap_pos(ix.c1 + B.n[0], M.L1);
                int x2 = sgb_wrap_pos(ix.c2 + B.n[1], M.L2);
                int x3 = sgb_wrap_pos(ix.c3 + B.n[2], M.L3);
                bond_E(B, S.t.bq, x1 + M.L1 * (x2 + M.L2 * (x3 + M.L3 * B.j)));
            }
        }
    }
    double e = sgb_block_sum(E);
    double a0 = sgb_block_sum(mx);
    double a1 = sgb_block_sum(my);
    double a2 = sgb_block_sum(mz);
    if (threadIdx.x == 0) {
        partials[4 * blockIdx.x + 0] = e;
        partials[4 * blockIdx.x + 1] = a0;
        partials[4 * blockIdx.x + 2] = a1;
        partials[4 * blockIdx.x + 3] = a2;
    }
}

template <class K>
int set_smem(K kernel, size_t smem) {
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return SGB_ERR_CUDA;
    return SGB_OK;
}

template <class K>
int coop(K kernel, const LaunchInfo& li, void** args, cudaStream_t st) {
    if (set_smem(kernel, li.smem) != SGB_OK) return SGB_ERR_CUDA;
    return cudaLaunchCooperativeKernel((const void*)kernel, dim3(li.grid), dim3(li.block), args, li.smem, st) == cudaSuccess
               ? SGB_OK : SGB_ERR_CUDA;
}

template <class R, int N>
int heun_n(const Model<R>& M, void** args, bool inject, const LaunchInfo& li, cudaStream_t st) {
    const bool bq = M.has_biquad != 0;
    if (li.spt == 1) {
        if (inject) return bq ? coop(k_sun_heun<R, N, 1, true, true>, li, args, st) : coop(k_sun_heun<R, N, 1, true, false>, li, args, st);
        return bq ? coop(k_sun_heun<R, N, 1, false, true>, li, args, st) : coop(k_sun_heun<R, N, 1, false, false>, li, args, st);
    }
    if (li.spt == 2) {
        if (inject) return bq ? coop(k_sun_heun<R, N, 2, true, true>, li, args, st) : coop(k_sun_heun<R, N, 2, true, false>, li, args, st);
        return bq ? coop(k_sun_heun<R, N, 2, false, true>, li, args, st) : coop(k_sun_heun<R, N, 2, false, false>, li, args, st);
    }
    return SGB_ERR_ARG;
}

template <class R, int N>
int mid_n(const Model<R>& M, void** args, const LaunchInfo& li, cudaStream_t st) {
    const bool bq = M.has_biquad != 0;
    if (li.spt == 1) return bq ? coop(k_sun_midpoint<R, N, 1, true>, li, args, st) : coop(k_sun_midpoint<R, N, 1, false>, li, args, st);
    if (li.spt == 2) return bq ? coop(k_sun_midpoint<R, N, 2, true>, li, args, st) : coop(k_sun_midpoint<R, N, 2, false>, li, args, st);
    return SGB_ERR_ARG;
}

template <class R, int N>
int occ_n(int spt, int block, size_t smem, int* bps) {
    int best = 1 << 30, a = 0;
    auto one = [&](auto k) -> int {
        if (set_smem(k, smem) != SGB_OK) return SGB_ERR_CUDA;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k, block, smem) != cudaSuccess) return SGB_ERR_CUDA;
        best = a < best ? a : best;
        return SGB_OK;
    };
    int rc = SGB_OK;
    if (spt == 1) {
        rc |= one(k_sun_heun<R, N, 1, true, true>); rc |= one(k_sun_heun<R, N, 1, false, true>);
        rc |= one(k_sun_heun<R, N, 1, true, false>); rc |= one(k_sun_heun<R, N, 1, false, false>);
        rc |= one(k_sun_midpoint<R, N, 1, true>); rc |= one(k_sun_midpoint<R, N, 1, false>);
    } else if (spt == 2) {
        rc |= one(k_sun_heun<R, N, 2, true, true>); rc |= one(k_sun_heun<R, N, 2, false, true>);
        rc |= one(k_sun_heun<R, N, 2, true, false>); rc |= one(k_sun_heun<R, N, 2, false, false>);
        rc |= one(k_sun_midpoint<R, N, 2, true>); rc |= one(k_sun_midpoint<R, N, 2, false>);
    } else return SGB_ERR_ARG;
    if (rc != SGB_OK) return SGB_ERR_CUDA;
    *bps = best;
    return SGB_OK;
}

template <class R, int N>
int grid1d(const Model<R>& M) {
    int grid = (M.ns + SGB_BLOCK - 1) / SGB_BLOCK;
    return grid > 4096 ? 4096 : grid;
}

// HZ += (f · S) Z for an external dipole field f = dE/dS per site (the dipole-dipole term
// of set_energy_grad_coherents!, Interactions.jl:596-669, which enters through dE/dS).
template <class R, int N>
__global__ void k_sun_add_dipole_field(const R* Z, const double* f, double* hz, int ns) {
    SpinConst<R, N> sc;
    for (int site = blockIdx.x * blockDim.x + threadIdx.x; site < ns; site += gridDim.x * blockDim.x) {
        const double dx = f[3 * (size_t)site], dy = f[3 * (size_t)site + 1], dz = f[3 * (size_t)site + 2];
        double z[2 * N];
#pragma unroll
        for (int c = 0; c < 2 * N; c++) z[c] = (double)Z[(size_t)c * ns + site];
#pragma unroll
        for (int r = 0; r < N; r++) {
            double ar = dz * (double)sc.sz[r] * z[2 * r], ai = dz * (double)sc.sz[r] * z[2 * r + 1];
            if (r + 1 < N) {   // (dx - i dy) off_r z_{r+1}
                const double o = (double)sc.off[r], pr = o * dx, pi = -o * dy;
                ar += pr * z[2 * r + 2] - pi * z[2 * r + 3];
                ai += pr * z[2 * r + 3] + pi * z[2 * r + 2];
            }
            if (r > 0) {       // (dx + i dy) off_{r-1} z_{r-1}
                const double o = (double)sc.off[r - 1], pr = o * dx, pi = o * dy;
                ar += pr * z[2 * r - 2] - pi * z[2 * r - 1];
                ai += pr * z[2 * r - 1] + pi * z[2 * r - 2];
            }
            hz[(size_t)site * 2 * N + 2 * r] += ar;
            hz[(size_t)site * 2 * N + 2 * r + 1] += ai;
        }
    }
}

template <class R, int N>
int add_field_n(const R* Z, const double* f, double* hz, int ns, cudaStream_t st) {
    int grid = (ns + SGB_BLOCK - 1) / SGB_BLOCK;
    if (grid > 4096) grid = 4096;
    k_sun_add_dipole_field<R, N><<<grid, SGB_BLOCK, 0, st>>>(Z, f, hz, ns);
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

// ---- stage kernels for SU(N) dynamics with dipole-dipole interactions --------------------
// Every HZ then needs a transform over the whole lattice, so each Heun stage and each
// midpoint iteration is its own launch (HZ from sun_launch_grad plus the dipole field).
// Kets SoA [2N][ns]; HZ AoS [ns][2N] in FP64. Same per-site arithmetic and noise stream as
// k_sun_heun / k_sun_midpoint.
template <class R, int N, bool INJECT>
__global__ void k_lr_sun_heun_a(const R* Z, const double* hz, R* ZP, R* D1, R* XI, const R* kappa, int ns, R dt, R lam,
                                R nscale, uint64_t seed, uint64_t step, const double* noise) {
    for (int site = blockIdx.x * blockDim.x + threadIdx.x; site < ns; site += gridDim.x * blockDim.x) {
        R z[2 * N], ze[2 * N], h[2 * N], d1[2 * N];
#pragma unroll
        for (int c = 0; c < 2 * N; c++) {
            z[c] = Z[(size_t)c * ns + site];
            h[c] = (R)hz[(size_t)site * 2 * N + c];
        }
        if (nscale == (R)0) {
#pragma unroll
            for (int c = 0; c < 2 * N; c++) ze[c] = 0;
        } else if (INJECT) {
#pragma unroll
            for (int c = 0; c < 2 * N; c++) ze[c] = (R)noise[(size_t)site * 2 * N + c] * nscale;
        } else {
            const R r2 = (R)0.70710678118654752440;
#pragma unroll
            for (int c = 0; c < 2 * N; c += 4) {
                R g4[4];
                sgb_normals4<R>(seed, 0u, step, (uint32_t)site, (uint32_t)(c / 4), g4);
#pragma unroll
                for (int q = 0; q < 4; q++)
                    if (c + q < 2 * N) ze[c + q] = g4[q] * r2 * nscale;
            }
        }
        rhs_sun<R, N>(z, ze, h, dt, lam, d1);
#pragma unroll
        for (int c = 0; c < 2 * N; c++) z[c] += d1[c];
        normalize_ket<R, N>(z, kappa[site]);
#pragma unroll
        for (int c = 0; c < 2 * N; c++) {
            ZP[(size_t)c * ns + site] = z[c];
            D1[(size_t)c * ns + site] = d1[c];
            XI[(size_t)c * ns + site] = ze[c];
        }
    }
}

template <class R, int N>
__global__ void k_lr_sun_heun_b(R* Z, const R* ZP, const double* hz, const R* D1, const R* XI, const R* kappa, int ns, R dt,
                                R lam) {
    for (int site = blockIdx.x * blockDim.x + threadIdx.x; site < ns; site += gridDim.x * blockDim.x) {
        R zp[2 * N], ze[2 * N], h[2 * N], d2[2 * N], z[2 * N];
#pragma unroll
        for (int c = 0; c < 2 * N; c++) {
            zp[c] = ZP[(size_t)c * ns + site];
            ze[c] = XI[(size_t)c * ns + site];
            h[c] = (R)hz[(size_t)site * 2 * N + c];
        }
        rhs_sun<R, N>(zp, ze, h, dt, lam, d2);
#pragma unroll
        for (int c = 0; c < 2 * N; c++) z[c] = Z[(size_t)c * ns + site] + (D1[(size_t)c * ns + site] + d2[c]) / 2;
        normalize_ket<R, N>(z, kappa[site]);
#pragma unroll
        for (int c = 0; c < 2 * N; c++) Z[(size_t)c * ns + site] = z[c];
    }
}

// Zbar = (Z + Z')/2 (Integrators.jl:431, not normalised)
template <class R, int N>
__global__ void k_lr_sun_mid_half(const R* Z, const R* Zp, R* Zb, int ns) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (size_t)2 * N * ns; i += (size_t)gridDim.x * blockDim.x)
        Zb[i] = (Z[i] + Zp[i]) / 2;
}

// Z'' = Z + rhs(Zbar); per-block partial sums of |Z' - Z''|^2 (fast_isapprox); Z' = Z''
template <class R, int N>
__global__ void k_lr_sun_mid_update(const R* Z, const R* Zb, const double* hz, R* Zp, int ns, R dt, R lam, double* part) {
    double acc = 0;
    for (int site = blockIdx.x * blockDim.x + threadIdx.x; site < ns; site += gridDim.x * blockDim.x) {
        R zb[2 * N], h[2 * N], zero[2 * N], dz[2 * N];
#pragma unroll
        for (int c = 0; c < 2 * N; c++) {
            zb[c] = Zb[(size_t)c * ns + site];
            h[c] = (R)hz[(size_t)site * 2 * N + c];
            zero[c] = 0;
        }
        rhs_sun<R, N>(zb, zero, h, dt, lam, dz);
#pragma unroll
        for (int c = 0; c < 2 * N; c++) {
            const R q = Z[(size_t)c * ns + site] + dz[c];
            const R e = Zp[(size_t)c * ns + site] - q;
            acc += (double)(e * e);
            Zp[(size_t)c * ns + site] = q;
        }
    }
    const double t = sgb_block_sum(acc);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

template <class R, int N>
__global__ void k_lr_sun_mid_accept(R* Z, const R* Zp, const R* kappa, int ns) {
    for (int site = blockIdx.x * blockDim.x + threadIdx.x; site < ns; site += gridDim.x * blockDim.x) {
        R z[2 * N];
#pragma unroll
        for (int c = 0; c < 2 * N; c++) z[c] = Zp[(size_t)c * ns + site];
        normalize_ket<R, N>(z, kappa[site]);
#pragma unroll
        for (int c = 0; c < 2 * N; c++) Z[(size_t)c * ns + site] = z[c];
    }
}

template <class R, int N>
__global__ void k_sun_snapshot(Model<R> M, const R* Z, SnapArgs<R> sn, int t) {
    for (int site = blockIdx.x * blockDim.x + threadIdx.x; site < M.ns; site += gridDim.x * blockDim.x) {
        R z[2 * N];
#pragma unroll
        for (int c = 0; c < 2 * N; c++) z[c] = Z[(size_t)c * M.ns + site];
        write_snapshot_sun<R, N>(M, sn, t, site, z);
    }
}

template <class R, int N>
int lr_sun_n(int stage, const Model<R>& M, R* Z, R* ZP, R* D1, R* XI, const double* hz, double dt, double lam, double nscale,
             uint64_t seed, uint64_t step, const double* noise, double* part, const SnapArgs<R>* sn, int t, cudaStream_t st) {
    const int ns = M.ns;
    const int grid = std::max(1, std::min(4096, (ns + SGB_BLOCK - 1) / SGB_BLOCK));
    switch (stage) {
        case 0:
            if (noise) k_lr_sun_heun_a<R, N, true><<<grid, SGB_BLOCK, 0, st>>>(Z, hz, ZP, D1, XI, M.kappa, ns, (R)dt, (R)lam, (R)nscale, seed, step, noise);
            else k_lr_sun_heun_a<R, N, false><<<grid, SGB_BLOCK, 0, st>>>(Z, hz, ZP, D1, XI, M.kappa, ns, (R)dt, (R)lam, (R)nscale, seed, step, noise);
            break;
        case 1: k_lr_sun_heun_b<R, N><<<grid, SGB_BLOCK, 0, st>>>(Z, ZP, hz, D1, XI, M.kappa, ns, (R)dt, (R)lam); break;
        case 2: k_lr_sun_mid_half<R, N><<<grid, SGB_BLOCK, 0, st>>>(Z, ZP, D1, ns); break;
        case 3: k_lr_sun_mid_update<R, N><<<EWALD_PART_BLOCKS, SGB_BLOCK, 0, st>>>(Z, D1, hz, ZP, ns, (R)dt, (R)lam, part); break;
        case 4: k_lr_sun_mid_accept<R, N><<<grid, SGB_BLOCK, 0, st>>>(Z, ZP, M.kappa, ns); break;
        case 5: k_sun_snapshot<R, N><<<grid, SGB_BLOCK, 0, st>>>(M, Z, *sn, t); break;
        default: return SGB_ERR_ARG;
    }
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

// ---- Langevin for small SU(N) lattices held by one thread-block cluster ---------------
// HZ of one site of sublattice a with the neighbours' expected dipoles (and quadrupoles)
// fetched through loaders of the neighbour reference nbi(k) of the site's k-th bond, bonds
// in table order (the same sums as sun_field).
template <class R, int N, bool BQ, class NBI, class LDD, class LDQ>
__device__ __forceinline__ void local_HZ_ld(const Model<R>& M, const SunTab<R, N>& S, const SpinConst<R, N>& sc, int site,
                                            int a, NBI nbi, LDD ldD, LDQ ldQ, const R* z, R* hz) {
    const int ns = M.ns;
    R d[3] = {0, 0, 0}, v[5] = {0, 0, 0, 0, 0};
    if (M.h) { d[0] = __ldg(M.h + site); d[1] = __ldg(M.h + ns + site); d[2] = __ldg(M.h + 2 * ns + site); }
    const int b0 = S.t.boff[a], b1 = S.t.boff[a + 1];
    for (int b = b0; b < b1; b++) {
        const DBond<R>& B = S.t.bonds[b];
        const int j = nbi(b - b0);
        R t[3];
        ldD(j, t);
        if (B.jkind == 0) {
            const R jj = B.J[0];
            d[0] += jj * t[0]; d[1] += jj * t[1]; d[2] += jj * t[2];
        } else {
            d[0] += B.J[0] * t[0] + B.J[3] * t[1] + B.J[6] * t[2];
            d[1] += B.J[1] * t[0] + B.J[4] * t[1] + B.J[7] * t[2];
            d[2] += B.J[2] * t[0] + B.J[5] * t[1] + B.J[8] * t[2];
        }
        if (BQ && B.bqkind != 0) {
            R Qj[5];
            ldQ(j, Qj);
            if (B.bqkind == 1) {
#pragma unroll
                for (int q = 0; q < 5; q++) v[q] += B.bq * ((R)biquad_metric(q) * Qj[q]);
            } else {
                const R* Bm = S.t.bq + 25 * B.bqidx;
#pragma unroll
                for (int q = 0; q < 5; q++) {
                    R acc = 0;
#pragma unroll
                    for (int p = 0; p < 5; p++) acc += Bm[q + 5 * p] * Qj[p];
                    v[q] += acc;
                }
            }
        }
    }
    apply_H<R, N, BQ>(sc, S.lam + a * 2 * N * N, S.qm, d, v, z, hz);
}

// CTA r of the cluster holds sites [r*nsl, (r+1)*nsl): their kets, predictor kets, first
// increments and noise, and the expected dipoles (quadrupoles) of the state and of the
// predictor that neighbours read. Stages end at the cluster barrier. Same per-site
// arithmetic and noise stream as k_sun_heun.
template <class R, int N, bool INJECT, bool BQ>
__global__ void __launch_bounds__(SGB_CLUSTER_BLOCK) k_sun_heun_cluster(Model<R> M, R* Z, R* D, R* Qb, int nsl, int nsteps,
                                                                       R dt, R lam, R nscale, uint64_t seed, uint64_t step0,
                                                                       const double* noise) {
    extern __shared__ __align__(16) unsigned char smem[];
    cg::cluster_group cl = cg::this_cluster();
    SunTab<R, N> S = stage_sun<R, N>(M, smem);
    SpinConst<R, N> sc;
    const int rank = (int)cl.block_rank();
    const int ns = M.ns;
    constexpr int K = 2 * N;
    R* lZ = reinterpret_cast<R*>(smem + ((M.tables_bytes + 15) / 16) * 16);   // [K][nsl]
    R* lZP = lZ + K * nsl;
    R* lD1 = lZP + K * nsl;
    R* lZE = lD1 + K * nsl;
    R* lD = lZE + K * nsl;     // [3][nsl]
    R* lDP = lD + 3 * nsl;
    R* lQ = lDP + 3 * nsl;     // [5][nsl] (BQ)
    R* lQP = lQ + 5 * nsl;
    // per owned site, staged once so that the steps do no index loads or divisions: for each
    // bond the neighbour's CTA and local index packed as rank << 11 | local (nsl <= 2048, at
    // most 16 CTAs), and the site's sublattice
    unsigned short* lN = reinterpret_cast<unsigned short*>(BQ ? lQP + 5 * nsl : lQ);   // [kb][nsl]
    unsigned char* lA = reinterpret_cast<unsigned char*>(lN + (size_t)M.kb * nsl);
    __shared__ const R* rD[SGB_CLUSTER_MAX];
    __shared__ const R* rDP[SGB_CLUSTER_MAX];
    __shared__ const R* rQ[SGB_CLUSTER_MAX];
    __shared__ const R* rQP[SGB_CLUSTER_MAX];
    if (threadIdx.x < cl.num_blocks()) {
        rD[threadIdx.x] = cl.map_shared_rank(lD, threadIdx.x);
        rDP[threadIdx.x] = cl.map_shared_rank(lDP, threadIdx.x);
        if (BQ) {
            rQ[threadIdx.x] = cl.map_shared_rank(lQ, threadIdx.x);
            rQP[threadIdx.x] = cl.map_shared_rank(lQP, threadIdx.x);
        }
    }
    const int s0 = rank * nsl, n = max(0, min(ns, s0 + nsl) - s0);
    // the noise of one step for this thread's sites, into lZE
    auto fill_noise = [&](int step) {
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const int site = s0 + i;
            R ze[K];
            if (nscale == (R)0) {
#pragma unroll
                for (int c = 0; c < K; c++) ze[c] = 0;
            } else if (INJECT) {
                const double* nz = noise + ((size_t)step * ns + site) * K;
#pragma unroll
                for (int c = 0; c < K; c++) ze[c] = (R)nz[c] * nscale;
            } else {
                const R r2 = (R)0.70710678118654752440;
#pragma unroll
                for (int c = 0; c < K; c += 4) {
                    R g4[4];
                    sgb_normals4<R>(seed, 0u, step0 + step, (uint32_t)site, (uint32_t)(c / 4), g4);
#pragma unroll
                    for (int q = 0; q < 4; q++)
                        if (c + q < K) ze[c + q] = g4[q] * r2 * nscale;
                }
            }
#pragma unroll
            for (int c = 0; c < K; c++) lZE[c * nsl + i] = ze[c];
        }
    };
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int site = s0 + i, a = site / M.ncell;
        lA[i] = (unsigned char)a;
        for (int b = 0; b < S.t.boff[a + 1] - S.t.boff[a]; b++) {
            const int j = __ldg(M.nbr + (size_t)b * ns + site), q = j / nsl;
            lN[(size_t)b * nsl + i] = (unsigned short)((q << 11) | (j - q * nsl));
        }
#pragma unroll
        for (int c = 0; c < K; c++) lZ[c * nsl + i] = Z[(size_t)c * ns + s0 + i];
#pragma unroll
        for (int c = 0; c < 3; c++) lD[c * nsl + i] = D[(size_t)c * ns + s0 + i];
        if (BQ) {
#pragma unroll
            for (int c = 0; c < 5; c++) lQ[c * nsl + i] = Qb[(size_t)c * ns + s0 + i];
        }
    }
    if (nsteps > 0) fill_noise(0);
    cl.sync();
    auto mkld = [&](const R* const* base, int ncomp) {
        return [base, ncomp, nsl](int v, R* out) {
            const R* b = base[v >> 11];
            const int l = v & 2047;
            for (int c = 0; c < ncomp; c++) out[c] = b[c * nsl + l];
        };
    };
    auto ldD = mkld(rD, 3);
    auto ldDP = mkld(rDP, 3);
    auto ldQ = mkld(rQ, 5);
    auto ldQP = mkld(rQP, 5);
    for (int step = 0; step < nsteps; ++step) {
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const int site = s0 + i;
            const unsigned short* ip = lN + i;
            auto nbi = [ip, nsl](int b) { return (int)ip[(size_t)b * nsl]; };
            R z[K], ze[K], hz[K], d1[K], zp[K];
#pragma unroll
            for (int c = 0; c < K; c++) { z[c] = lZ[c * nsl + i]; ze[c] = lZE[c * nsl + i]; }
            local_HZ_ld<R, N, BQ>(M, S, sc, site, lA[i], nbi, ldD, ldQ, z, hz);
            rhs_sun<R, N>(z, ze, hz, dt, lam, d1);
#pragma unroll
            for (int c = 0; c < K; c++) zp[c] = z[c] + d1[c];
            normalize_ket<R, N>(zp, __ldg(M.kappa + site));
#pragma unroll
            for (int c = 0; c < K; c++) { lZP[c * nsl + i] = zp[c]; lD1[c * nsl + i] = d1[c]; }
            R nx, ny, nz_;
            expected_spin<R, N>(sc, zp, nx, ny, nz_);
            lDP[i] = nx; lDP[nsl + i] = ny; lDP[2 * nsl + i] = nz_;
            if (BQ) {
                R q[5];
                expected_quad<R, N>(S.qm, zp, q);
#pragma unroll
                for (int c = 0; c < 5; c++) lQP[c * nsl + i] = q[c];
            }
        }
        cl.sync();
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const int site = s0 + i;
            const unsigned short* ip = lN + i;
            auto nbi = [ip, nsl](int b) { return (int)ip[(size_t)b * nsl]; };
            R zp[K], ze[K], hz[K], d2[K], z[K];
#pragma unroll
            for (int c = 0; c < K; c++) { zp[c] = lZP[c * nsl + i]; ze[c] = lZE[c * nsl + i]; }
            local_HZ_ld<R, N, BQ>(M, S, sc, site, lA[i], nbi, ldDP, ldQP, zp, hz);
            rhs_sun<R, N>(zp, ze, hz, dt, lam, d2);
#pragma unroll
            for (int c = 0; c < K; c++) z[c] = lZ[c * nsl + i] + (lD1[c * nsl + i] + d2[c]) / 2;
            normalize_ket<R, N>(z, __ldg(M.kappa + site));
#pragma unroll
            for (int c = 0; c < K; c++) lZ[c * nsl + i] = z[c];
            R nx, ny, nz_;
            expected_spin<R, N>(sc, z, nx, ny, nz_);
            lD[i] = nx; lD[nsl + i] = ny; lD[2 * nsl + i] = nz_;
            if (BQ) {
                R q[5];
                expected_quad<R, N>(S.qm, z, q);
#pragma unroll
                for (int c = 0; c < 5; c++) lQ[c * nsl + i] = q[c];
            }
        }
        // split cluster barrier: the next step's noise (own sites, read by this thread only)
        // is drawn between the arrival and the wait
        asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
        if (step + 1 < nsteps) fill_noise(step + 1);
        asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
#pragma unroll
        for (int c = 0; c < K; c++) Z[(size_t)c * ns + s0 + i] = lZ[c * nsl + i];
#pragma unroll
        for (int c = 0; c < 3; c++) D[(size_t)c * ns + s0 + i] = lD[c * nsl + i];
        if (BQ) {
#pragma unroll
            for (int c = 0; c < 5; c++) Qb[(size_t)c * ns + s0 + i] = lQ[c * nsl + i];
        }
    }
}

template <class R, int N>
int sun_heun_cluster_n(const Model<R>& M, R* Z, R* D, R* Q, int cs, int nsteps, double dt, double lam, double nscale,
                       uint64_t seed, uint64_t step0, const double* noise, cudaStream_t st) {
    const int nsl = (M.ns + cs - 1) / cs;
    const size_t smem = sun_cluster_smem<R>(M, nsl);
    const bool bq = M.has_biquad != 0;
    const void* k = noise ? (bq ? (const void*)k_sun_heun_cluster<R, N, true, true> : (const void*)k_sun_heun_cluster<R, N, true, false>)
                          : (bq ? (const void*)k_sun_heun_cluster<R, N, false, true> : (const void*)k_sun_heun_cluster<R, N, false, false>);
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return SGB_ERR_CUDA;
    if (cs > 8 && cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) return SGB_ERR_CUDA;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cs);
    cfg.blockDim = dim3(SGB_CLUSTER_BLOCK);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cs;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, k, &cfg) != cudaSuccess || clusters < 1) return SGB_ERR_ARG;
    Model<R> m = M;
    R rdt = (R)dt, rlam = (R)lam, rns = (R)nscale;
    int nsl_ = nsl, nst = nsteps;
    void* args[] = {&m, &Z, &D, &Q, &nsl_, &nst, &rdt, &rlam, &rns, &seed, &step0, &noise};
    return cudaLaunchKernelExC(&cfg, k, args) == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

// ---- LocalSampler in SU(N) mode (Samplers.jl:139-158, Interactions.jl:311-373) --------
// <z|Λ|z> of one ket (the onsite energy, Interactions.jl:331-332)
template <class R, int N>
__device__ __forceinline__ R onsite_energy(const R* lam, const R* z) {
    R acc = 0;
#pragma unroll
    for (int c = 0; c < N; c++)
#pragma unroll
        for (int r = 0; r < N; r++) {
            const R lr = lam[2 * (r + N * c)], li = lam[2 * (r + N * c) + 1];
            const R tr = lr * z[2 * c] - li * z[2 * c + 1], ti = lr * z[2 * c + 1] + li * z[2 * c];
            acc += z[2 * r] * tr + z[2 * r + 1] * ti;
        }
    return acc;
}

// local_energy_change for a coherent state: ket z0 (dipole s0, quadrupole q0) at `site`
// becomes zn (sn, qn); neighbours enter through their expected dipoles and quadrupoles.
template <class R, int N, bool BQ>
__device__ inline R sun_local_dE(const Model<R>& M, const SunTab<R, N>& S, int site, const R* D, const R* Qb,
                                 const R* z0, const R* s0, const R* q0, const R* zn, const R* sn, const R* qn) {
    const int ns = M.ns, a = site / M.ncell;
    const R dx = sn[0] - s0[0], dy = sn[1] - s0[1], dz = sn[2] - s0[2];
    R dE = 0;
    if (M.h) dE += M.h[site] * dx + M.h[ns + site] * dy + M.h[2 * ns + site] * dz;
    const R* lam = lam_at<R, N>(M, S, site, a);
    dE += onsite_energy<R, N>(lam, zn) - onsite_energy<R, N>(lam, z0);
    if (M.ioff) {
        // per-site couplings: every row of the site's own list (reversed copies carry J^T)
        for_site_bonds<R>(M, S.t, site, a, [&](const DBond<R>& B, const R* bq, int j) {
            const R tx = sgb_ld(D + j), ty = sgb_ld(D + ns + j), tz = sgb_ld(D + 2 * ns + j);
            if (B.jkind == 0) {
                dE += B.J[0] * (dx * tx + dy * ty + dz * tz);
            } else {
                dE += dx * (B.J[0] * tx + B.J[3] * ty + B.J[6] * tz) + dy * (B.J[1] * tx + B.J[4] * ty + B.J[7] * tz) +
                      dz * (B.J[2] * tx + B.J[5] * ty + B.J[8] * tz);
            }
            if (BQ && B.bqkind != 0) {
                R Qj[5];
#pragma unroll
                for (int q = 0; q < 5; q++) Qj[q] = sgb_ld(Qb + (size_t)q * ns + j);
                R acc = 0;
                if (B.bqkind == 1) {
#pragma unroll
                    for (int q = 0; q < 5; q++) acc += (qn[q] - q0[q]) * ((R)biquad_metric(q) * Qj[q]);
                    acc *= B.bq;
                } else {
                    const R* Bm = bq + 25 * B.bqidx;
#pragma unroll
                    for (int q = 0; q < 5; q++) {
                        R r = 0;
#pragma unroll
                        for (int p = 0; p < 5; p++) r += Bm[q + 5 * p] * Qj[p];
                        acc += (qn[q] - q0[q]) * r;
                    }
                }
                dE += acc;
            }
        });
        return dE;
    }
    // neighbour indices and dipoles are fetched 8 bonds at a time (loads in flight together)
    constexpr int GATHER = 8;
    const int b0 = S.t.boff[a], b1 = S.t.boff[a + 1];
    for (int bb = b0; bb < b1; bb += GATHER) {
        int js[GATHER];
        R txs[GATHER], tys[GATHER], tzs[GATHER];
#pragma unroll
        for (int g = 0; g < GATHER; g++)
            if (bb + g < b1) js[g] = __ldg(M.nbr + (size_t)(bb + g - b0) * ns + site);
#pragma unroll
        for (int g = 0; g < GATHER; g++)
            if (bb + g < b1) { txs[g] = sgb_ld(D + js[g]); tys[g] = sgb_ld(D + ns + js[g]); tzs[g] = sgb_ld(D + 2 * ns + js[g]); }
#pragma unroll
        for (int g = 0; g < GATHER; g++) {
            if (bb + g >= b1) break;
            const DBond<R>& B = S.t.bonds[bb + g];
            const int j = js[g];
            const R tx = txs[g], ty = tys[g], tz = tzs[g];
            if (B.jkind == 0) {
                dE += B.J[0] * (dx * tx + dy * ty + dz * tz);
            } else {
                dE += dx * (B.J[0] * tx + B.J[3] * ty + B.J[6] * tz) + dy * (B.J[1] * tx + B.J[4] * ty + B.J[7] * tz) +
                      dz * (B.J[2] * tx + B.J[5] * ty + B.J[8] * tz);
            }
            if (BQ && B.bqkind != 0) {
                R Qj[5];
#pragma unroll
                for (int q = 0; q < 5; q++) Qj[q] = sgb_ld(Qb + (size_t)q * ns + j);
                R acc = 0;
                if (B.bqkind == 1) {
#pragma unroll
                    for (int q = 0; q < 5; q++) acc += (qn[q] - q0[q]) * ((R)biquad_metric(q) * Qj[q]);
                    acc *= B.bq;
                } else {
                    const R* Bm = S.t.bq + 25 * B.bqidx;
#pragma unroll
                    for (int q = 0; q < 5; q++) {
                        R r = 0;
#pragma unroll
                        for (int p = 0; p < 5; p++) r += Bm[q + 5 * p] * Qj[p];
                        acc += (qn[q] - q0[q]) * r;
                    }
                }
                dE += acc;
            }
        }
    }
    if (BQ && M.has_general) {
        // general couplings: Δ<A>_site <B>_j over the rows of the site's sublattice (reversed
        // copies carry the swapped pair)
        R r0[N * N], rn[N * N];
        sun_rho<R, N>(z0, r0);
        sun_rho<R, N>(zn, rn);
        for (int b = b0; b < b1; b++) {
            const DBond<R>& B = S.t.bonds[b];
            if (dbond_gcnt(B) == 0) continue;
            const int j = __ldg(M.nbr + (size_t)(b - b0) * ns + site);
            for (int t = 0; t < dbond_gcnt(B); t++) {
                const R* row = M.gtab + (size_t)(dbond_gidx(B) + t) * 4 * N * N;
                R dA = 0, Bb = 0;
#pragma unroll
                for (int k = 0; k < N * N; k++) {
                    dA += __ldg(row + k) * (rn[k] - r0[k]);
                    Bb += __ldg(row + 3 * N * N + k) * sgb_ld(Qb + (size_t)(5 + k) * ns + j);
                }
                dE += dA * Bb;
            }
        }
    }
    return dE;
}

// Colour-class sweeps as the dipole LocalSampler. Proposals: randspin (normalize_ket of a
// complex normal vector, System.jl:448-452), flip_ket (Spin.jl:121-128), perturbed_spin
// (Z + magnitude·√κ·ξ, System.jl:461-468); complex normals have E|ξ_k|² = 1 (Julia's
// randn(ComplexF64)). Injected randoms: [sweep][ns][2N + 3].
// One LocalSampler proposal at `site` in SU(N) mode (Samplers.jl:108-156): the proposed
// ket zn (propose_uniform, propose_flip or propose_delta), its expected dipole sn and
// quadrupole qn, the old values z0, s0, q0, and the short-range energy change e; u1 is the
// acceptance uniform. Returns false when the partial last sweep skips the site.
template <class R, int N, bool BQ, bool INJECT>
__device__ __forceinline__ bool sun_mc_propose(const Model<R>& M, const SunTab<R, N>& S, const SpinConst<R, N>& sc,
                                               const R* Z, const R* D, const R* Qb, const McArgs& A, int k, uint64_t sweep,
                                               bool partial, int site, R* z0, R* zn, R* s0, R* sn, R* q0, R* qn, double& e,
                                               double& u1) {
    const int ns = M.ns;
    constexpr int PER = 2 * N + 3;
    double u[4];
    const double* rr = nullptr;
    if (INJECT) {
        rr = A.rnd + ((size_t)k * ns + site) * PER;
        u[0] = rr[2 * N]; u[1] = rr[2 * N + 1]; u[2] = rr[2 * N + 2];
    } else {
        sgb_mc_uniforms4(A.seed, sweep, (uint32_t)site, u);
    }
    if (partial && !(u[2] < A.frac)) return false;
    u1 = u[1];
    int kind = A.kind[A.nkind - 1];
    double mag = A.mag[A.nkind - 1];
    for (int i = 0; i < A.nkind - 1; i++)
        if (u[0] < A.cum[i]) { kind = A.kind[i]; mag = A.mag[i]; break; }
    if (kind == SGB_PROPOSE_DELTA && isinf(mag)) kind = SGB_PROPOSE_UNIFORM;
    const R kap = M.kappa[site];
#pragma unroll
    for (int q = 0; q < 2 * N; q++) z0[q] = Z[(size_t)q * ns + site];
    if (kind == SGB_PROPOSE_FLIP) {
#pragma unroll
        for (int q = 0; q < N; q++) {   // reverse(parity .* conj(z))
            const R par = ((N - 1 - q) % 2) ? (R)-1 : (R)1;
            zn[2 * q] = par * z0[2 * (N - 1 - q)];
            zn[2 * q + 1] = -par * z0[2 * (N - 1 - q) + 1];
        }
    } else {
        R g[12];
        if (INJECT) {
#pragma unroll
            for (int q = 0; q < 2 * N; q++) g[q] = (R)rr[q];
        } else {
#pragma unroll
            for (int blk = 0; blk < (2 * N + 3) / 4; blk++) sgb_normals4<R>(A.seed, SGB_MC_STREAM, sweep, (uint32_t)site, (uint32_t)blk, g + 4 * blk);
#pragma unroll
            for (int q = 0; q < 2 * N; q++) g[q] *= (R)0.70710678118654752;
        }
        if (kind == SGB_PROPOSE_UNIFORM) {
#pragma unroll
            for (int q = 0; q < 2 * N; q++) zn[q] = g[q];
        } else {
            const R m = (R)mag * sgb_sqrt<R>(kap);
#pragma unroll
            for (int q = 0; q < 2 * N; q++) zn[q] = z0[q] + m * g[q];
        }
        normalize_ket<R, N>(zn, kap);
    }
    s0[0] = D[site]; s0[1] = D[ns + site]; s0[2] = D[2 * ns + site];
    expected_spin<R, N>(sc, zn, sn[0], sn[1], sn[2]);
    if (BQ) {
#pragma unroll
        for (int q = 0; q < 5; q++) q0[q] = Qb[(size_t)q * ns + site];
        expected_quad<R, N>(S.qm, zn, qn);
    }
    e = (double)sun_local_dE<R, N, BQ>(M, S, site, D, Qb, z0, s0, q0, zn, sn, qn);
    return true;
}

// Writes an accepted SU(N) move: ket, expected dipole and, with biquadratic or general
// couplings, quadrupole and packed density.
template <class R, int N, bool BQ>
__device__ __forceinline__ void sun_mc_commit(const Model<R>& M, R* Z, R* D, R* Qb, int site, const R* zn, const R* sn,
                                              const R* qn) {
    const int ns = M.ns;
#pragma unroll
    for (int q = 0; q < 2 * N; q++) Z[(size_t)q * ns + site] = zn[q];
    D[site] = sn[0]; D[ns + site] = sn[1]; D[2 * ns + site] = sn[2];
    if (BQ) {
#pragma unroll
        for (int q = 0; q < 5; q++) Qb[(size_t)q * ns + site] = qn[q];
        if (M.has_general) {
            R p[N * N];
            sun_rho<R, N>(zn, p);
#pragma unroll
            for (int q = 0; q < N * N; q++) Qb[(size_t)(5 + q) * ns + site] = p[q];
        }
    }
}

template <class R, int N, bool BQ, bool INJECT>
__global__ void __launch_bounds__(SGB_BLOCK) k_sun_local_sweeps(Model<R> M, R* Z, R* D, R* Qb, Ctrl* ctrl, McArgs A,
                                                               double* partials) {
    extern __shared__ __align__(16) unsigned char smem[];
    SunTab<R, N> S = stage_sun<R, N>(M, smem);
    __syncthreads();
    SpinConst<R, N> sc;
    const int ns = M.ns;
    const int nthr = gridDim.x * blockDim.x;
    constexpr int PER = 2 * N + 3;
    double aE = 0, ax = 0, ay = 0, az = 0;
    bool ok = true;
    for (int k = 0; k < A.nsweeps && ok; k++) {
        const bool partial = (k == A.nsweeps - 1) && A.frac < 1.0;
        const uint64_t sweep = A.sweep0 + (uint64_t)k;
        for (int c = 0; c < A.ncol; c++) {
            for (int idx = A.coff[c] + blockIdx.x * blockDim.x + threadIdx.x; idx < A.coff[c + 1]; idx += nthr) {
                const int site = A.perm[idx];
                R z0[2 * N], zn[2 * N], s0[3], sn[3], q0[5], qn[5];
                double e, u1;
                if (!sun_mc_propose<R, N, BQ, INJECT>(M, S, sc, Z, D, Qb, A, k, sweep, partial, site, z0, zn, s0, sn, q0, qn, e, u1))
                    continue;
                if (A.kT == 0.0 ? (e <= 0.0) : (u1 <= exp(-e / A.kT))) {
                    sun_mc_commit<R, N, BQ>(M, Z, D, Qb, site, zn, sn, qn);
                    aE += e;
                    ax += (double)sn[0] - (double)s0[0];
                    ay += (double)sn[1] - (double)s0[1];
                    az += (double)sn[2] - (double)s0[2];
                }
            }
            if (!sgb_grid_barrier(ctrl, gridDim.x)) { ok = false; break; }
        }
    }
    const double e = sgb_block_sum(aE);
    const double s0 = sgb_block_sum(ax);
    const double s1 = sgb_block_sum(ay);
    const double s2 = sgb_block_sum(az);
    if (threadIdx.x == 0) {
        partials[4 * blockIdx.x + 0] = e;
        partials[4 * blockIdx.x + 1] = s0;
        partials[4 * blockIdx.x + 2] = s1;
        partials[4 * blockIdx.x + 3] = s2;
    }
}

// Sweeps of an SU(N) system with dipole-dipole interactions: one CTA proposes at the sites
// in the order of A.perm, one at a time (thread 0: the proposal, the short-range change and
// the Ewald change of the expected dipole, Ewald.jl:230-241), and after an accepted move all
// threads update every site's field F = dE/dS. Random numbers as k_sun_local_sweeps.
template <class R, int N, bool BQ, bool INJECT>
__global__ void __launch_bounds__(256) k_sun_local_sweeps_ewald(Model<R> M, R* Z, R* D, R* Qb, McArgs A, EwaldDev E,
                                                                double* F, double* partials) {
    extern __shared__ __align__(16) unsigned char smem[];
    SunTab<R, N> S = stage_sun<R, N>(M, smem);
    __shared__ int s_acc;
    __shared__ double s_d[3];
    __syncthreads();
    SpinConst<R, N> sc;
    const int ns = M.ns, ncell = M.ncell;
    double aE = 0, ax = 0, ay = 0, az = 0;
    for (int k = 0; k < A.nsweeps; k++) {
        const bool partial = (k == A.nsweeps - 1) && A.frac < 1.0;
        const uint64_t sweep = A.sweep0 + (uint64_t)k;
        for (int idx = 0; idx < ns; idx++) {
            const int site = A.perm[idx];
            if (threadIdx.x == 0) {
                int acc = 0;
                R z0[2 * N], zn[2 * N], s0[3], sn[3], q0[5], qn[5];
                double e, u1;
                if (sun_mc_propose<R, N, BQ, INJECT>(M, S, sc, Z, D, Qb, A, k, sweep, partial, site, z0, zn, s0, sn, q0, qn, e, u1)) {
                    const double d[3] = {(double)sn[0] - (double)s0[0], (double)sn[1] - (double)s0[1], (double)sn[2] - (double)s0[2]};
                    double gd[3];
                    e += ewald_site_delta(E, F, site, ncell, d, gd);
                    if (A.kT == 0.0 ? (e <= 0.0) : (u1 <= exp(-e / A.kT))) {
                        acc = 1;
                        sun_mc_commit<R, N, BQ>(M, Z, D, Qb, site, zn, sn, qn);
                        aE += e;
                        ax += d[0]; ay += d[1]; az += d[2];
                        s_d[0] = gd[0]; s_d[1] = gd[1]; s_d[2] = gd[2];
                    }
                }
                s_acc = acc;
            }
            __syncthreads();
            if (s_acc) {
                const double gd[3] = {s_d[0], s_d[1], s_d[2]};
                ewald_field_update(E, F, site, ns, ncell, gd);
            }
            __syncthreads();
        }
    }
    if (threadIdx.x == 0) {
        partials[0] = aE;
        partials[1] = ax;
        partials[2] = ay;
        partials[3] = az;
    }
}

template <class R, int N, bool BQ>
__global__ void k_sun_local_dE(Model<R> M, const R* Z, const R* D, const R* Qb, int site, SunKet zk, double* out) {
    extern __shared__ __align__(16) unsigned char smem[];
    SunTab<R, N> S = stage_sun<R, N>(M, smem);
    __syncthreads();
    if (threadIdx.x != 0) return;
    SpinConst<R, N> sc;
    const int ns = M.ns;
    R z0[2 * N], zn[2 * N], s0[3], sn[3], q0[5], qn[5];
#pragma unroll
    for (int q = 0; q < 2 * N; q++) { z0[q] = Z[(size_t)q * ns + site]; zn[q] = (R)zk.v[q]; }
    s0[0] = D[site]; s0[1] = D[ns + site]; s0[2] = D[2 * ns + site];
    expected_spin<R, N>(sc, zn, sn[0], sn[1], sn[2]);
    if (BQ) {
#pragma unroll
        for (int q = 0; q < 5; q++) q0[q] = Qb[(size_t)q * ns + site];
        expected_quad<R, N>(S.qm, zn, qn);
    }
    *out = (double)sun_local_dE<R, N, BQ>(M, S, site, D, Qb, z0, s0, q0, zn, sn, qn);
}

template <class R, int N>
int sun_sweeps_n(const Model<R>& M, R* Z, R* D, R* Q, Ctrl* ctrl, const McArgs& A, int grid, double* part,
                 cudaStream_t st) {
    Model<R> m = M;
    McArgs a = A;
    void* args[] = {&m, &Z, &D, &Q, &ctrl, &a, &part};
    const size_t smem = (size_t)M.tables_bytes;
    const bool bq = M.has_biquad != 0, inj = A.rnd != nullptr;
    const void* k = bq ? (inj ? (const void*)k_sun_local_sweeps<R, N, true, true> : (const void*)k_sun_local_sweeps<R, N, true, false>)
                       : (inj ? (const void*)k_sun_local_sweeps<R, N, false, true> : (const void*)k_sun_local_sweeps<R, N, false, false>);
    if (smem > 48 * 1024 && cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return SGB_ERR_CUDA;
    return cudaLaunchCooperativeKernel(k, dim3(grid), dim3(SGB_BLOCK), args, smem, st) == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

template <class R, int N>
int sun_sweeps_ewald_n(const Model<R>& M, R* Z, R* D, R* Q, const McArgs& A, const EwaldDev& E, double* F, double* part,
                       cudaStream_t st) {
    Model<R> m = M;
    McArgs a = A;
    EwaldDev e = E;
    void* args[] = {&m, &Z, &D, &Q, &a, &e, &F, &part};
    const size_t smem = (size_t)M.tables_bytes;
    const bool bq = M.has_biquad != 0, inj = A.rnd != nullptr;
    const void* k = bq ? (inj ? (const void*)k_sun_local_sweeps_ewald<R, N, true, true> : (const void*)k_sun_local_sweeps_ewald<R, N, true, false>)
                       : (inj ? (const void*)k_sun_local_sweeps_ewald<R, N, false, true> : (const void*)k_sun_local_sweeps_ewald<R, N, false, false>);
    if (smem > 48 * 1024 && cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return SGB_ERR_CUDA;
    return cudaLaunchKernel(k, dim3(1), dim3(256), args, smem, st) == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

template <class R, int N>
int sun_mc_occ_n(size_t smem, int* bps) {
    int best = 1 << 30, a = 0;
    const void* ks[4] = {(const void*)k_sun_local_sweeps<R, N, true, true>, (const void*)k_sun_local_sweeps<R, N, true, false>,
                         (const void*)k_sun_local_sweeps<R, N, false, true>, (const void*)k_sun_local_sweeps<R, N, false, false>};
    for (const void* k : ks) {
        if (smem > 48 * 1024 && cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
            return SGB_ERR_CUDA;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k, SGB_BLOCK, smem) != cudaSuccess) return SGB_ERR_CUDA;
        best = a < best ? a : best;
    }
    *bps = best;
    return SGB_OK;
}

template <class R, int N>
int sun_dE_n(const Model<R>& M, const R* Z, const R* D, const R* Q, int site, const SunKet& zk, double* out, cudaStream_t st) {
    const size_t smem = (size_t)M.tables_bytes;
    const void* k = M.has_biquad ? (const void*)k_sun_local_dE<R, N, true> : (const void*)k_sun_local_dE<R, N, false>;
    if (smem > 48 * 1024 && cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return SGB_ERR_CUDA;
    Model<R> m = M;
    SunKet z = zk;
    void* args[] = {&m, &Z, &D, &Q, &site, &z, &out};
    return cudaLaunchKernel(k, dim3(1), dim3(32), args, smem, st) == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

}  // namespace

#define SGB_SUN_DISPATCH(EXPR2, EXPR3, EXPR4, EXPR5) \
    switch (M.N) {                                  \
        case 2: return EXPR2;                       \
        case 3: return EXPR3;                       \
        case 4: return EXPR4;                       \
        case 5: return EXPR5;                       \
    }                                               \
    return SGB_ERR_ARG;

template <class R>
int sun_launch_heun(const Model<R>& M, R* Z, R* D, R* Q, R* P, R* QP, Ctrl* ctrl, int nsteps, double dt,
                    double lam, double noise_scale, uint64_t seed, uint64_t step0, const double* noise,
                    const LaunchInfo& li, cudaStream_t st) {
    Model<R> m = M;
    R rdt = (R)dt, rlam = (R)lam, rns = (R)noise_scale;
    void* args[] = {&m, &Z, &D, &Q, &P, &QP, &ctrl, &nsteps, &rdt, &rlam, &rns, &seed, &step0, &noise};
    bool inj = noise != nullptr;
    SGB_SUN_DISPATCH((heun_n<R, 2>(M, args, inj, li, st)), (heun_n<R, 3>(M, args, inj, li, st)),
                     (heun_n<R, 4>(M, args, inj, li, st)), (heun_n<R, 5>(M, args, inj, li, st)))
}

template <class R>
int sun_launch_midpoint(const Model<R>& M, R* Z, R* D, R* Q, R* H, R* QH, Ctrl* ctrl, int nsteps, double dt,
                        double lam, double atol2, int max_iters, const SnapArgs<R>& snap, const LaunchInfo& li,
                        cudaStream_t st) {
    Model<R> m = M;
    SnapArgs<R> sn = snap;
    R rdt = (R)dt, rlam = (R)lam;
    void* args[] = {&m, &Z, &D, &Q, &H, &QH, &ctrl, &nsteps, &rdt, &rlam, &atol2, &max_iters, &sn};
    SGB_SUN_DISPATCH((mid_n<R, 2>(M, args, li, st)), (mid_n<R, 3>(M, args, li, st)), (mid_n<R, 4>(M, args, li, st)),
                     (mid_n<R, 5>(M, args, li, st)))
}

template <class R>
int sun_max_blocks(int N, int spt, int block, size_t smem, int* bps) {
    switch (N) {
        case 2: return occ_n<R, 2>(spt, block, smem, bps);
        case 3: return occ_n<R, 3>(spt, block, smem, bps);
        case 4: return occ_n<R, 4>(spt, block, smem, bps);
        case 5: return occ_n<R, 5>(spt, block, smem, bps);
    }
    return SGB_ERR_ARG;
}

#define SGB_SIMPLE_LAUNCH(KER, ...)                                                               \
    do {                                                                                          \
        size_t smem = (size_t)M.tables_bytes;                                                     \
        if (set_smem(KER, smem) != SGB_OK) return SGB_ERR_CUDA;                                   \
        KER<<<grid1d<R, 2>(M), SGB_BLOCK, smem, st>>>(__VA_ARGS__);                               \
        return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;                         \
    } while (0)

template <class R, int N>
static int refresh_n(const Model<R>& M, const R* Z, R* D, R* Q, cudaStream_t st) { SGB_SIMPLE_LAUNCH((k_sun_refresh<R, N>), M, Z, D, Q); }
template <class R, int N>
static int grad_n(const Model<R>& M, const R* Z, const R* D, const R* Q, double* g, cudaStream_t st) { SGB_SIMPLE_LAUNCH((k_sun_grad<R, N>), M, Z, D, Q, g); }
template <class R, int N>
static int energy_n(const Model<R>& M, const R* Z, const R* D, const R* Q, double* p, int nb, cudaStream_t st) {
    size_t smem = (size_t)M.tables_bytes;
    if (set_smem(k_sun_energy<R, N>, smem) != SGB_OK) return SGB_ERR_CUDA;
    k_sun_energy<R, N><<<nb, SGB_BLOCK, smem, st>>>(M, Z, D, Q, p);
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

template <class R>
int sun_launch_refresh(const Model<R>& M, const R* Z, R* D, R* Q, cudaStream_t st) {
    SGB_SUN_DISPATCH((refresh_n<R, 2>(M, Z, D, Q, st)), (refresh_n<R, 3>(M, Z, D, Q, st)), (refresh_n<R, 4>(M, Z, D, Q, st)),
                     (refresh_n<R, 5>(M, Z, D, Q, st)))
}
template <class R>
int sun_launch_grad(const Model<R>& M, const R* Z, const R* D, const R* Q, double* grad, cudaStream_t st) {
    SGB_SUN_DISPATCH((grad_n<R, 2>(M, Z, D, Q, grad, st)), (grad_n<R, 3>(M, Z, D, Q, grad, st)),
                     (grad_n<R, 4>(M, Z, D, Q, grad, st)), (grad_n<R, 5>(M, Z, D, Q, grad, st)))
}
template <class R>
int sun_launch_energy(const Model<R>& M, const R* Z, const R* D, const R* Q, double* partials, int nblocks, cudaStream_t st) {
    SGB_SUN_DISPATCH((energy_n<R, 2>(M, Z, D, Q, partials, nblocks, st)), (energy_n<R, 3>(M, Z, D, Q, partials, nblocks, st)),
                     (energy_n<R, 4>(M, Z, D, Q, partials, nblocks, st)), (energy_n<R, 5>(M, Z, D, Q, partials, nblocks, st)))
}

template <class R>
int sun_launch_add_dipole_field(const Model<R>& M, const R* Z, const double* f, double* hz, cudaStream_t st) {
    SGB_SUN_DISPATCH((add_field_n<R, 2>(Z, f, hz, M.ns, st)), (add_field_n<R, 3>(Z, f, hz, M.ns, st)),
                     (add_field_n<R, 4>(Z, f, hz, M.ns, st)), (add_field_n<R, 5>(Z, f, hz, M.ns, st)))
}

template <class R>
int sun_launch_lr_stage(int stage, const Model<R>& M, R* Z, R* ZP, R* D1, R* XI, const double* hz, double dt, double lam,
                        double nscale, uint64_t seed, uint64_t step, const double* noise, double* part,
                        const SnapArgs<R>* sn, int t, cudaStream_t st) {
    SGB_SUN_DISPATCH((lr_sun_n<R, 2>(stage, M, Z, ZP, D1, XI, hz, dt, lam, nscale, seed, step, noise, part, sn, t, st)),
                     (lr_sun_n<R, 3>(stage, M, Z, ZP, D1, XI, hz, dt, lam, nscale, seed, step, noise, part, sn, t, st)),
                     (lr_sun_n<R, 4>(stage, M, Z, ZP, D1, XI, hz, dt, lam, nscale, seed, step, noise, part, sn, t, st)),
                     (lr_sun_n<R, 5>(stage, M, Z, ZP, D1, XI, hz, dt, lam, nscale, seed, step, noise, part, sn, t, st)))
}

template <class R>
size_t sun_cluster_smem(const Model<R>& M, int nsl) {
    return (size_t)((M.tables_bytes + 15) / 16) * 16 + (size_t)(8 * M.N + 6 + (M.has_biquad ? 10 : 0)) * nsl * sizeof(R) +
           (size_t)2 * M.kb * nsl + nsl;
}

template <class R>
int sun_launch_heun_cluster(const Model<R>& M, R* Z, R* D, R* Q, int cs, int nsteps, double dt, double lam, double nscale,
                            uint64_t seed, uint64_t step0, const double* noise, cudaStream_t st) {
    SGB_SUN_DISPATCH((sun_heun_cluster_n<R, 2>(M, Z, D, Q, cs, nsteps, dt, lam, nscale, seed, step0, noise, st)),
                     (sun_heun_cluster_n<R, 3>(M, Z, D, Q, cs, nsteps, dt, lam, nscale, seed, step0, noise, st)),
                     (sun_heun_cluster_n<R, 4>(M, Z, D, Q, cs, nsteps, dt, lam, nscale, seed, step0, noise, st)),
                     (sun_heun_cluster_n<R, 5>(M, Z, D, Q, cs, nsteps, dt, lam, nscale, seed, step0, noise, st)))
}

template <class R>
int sun_launch_local_sweeps(const Model<R>& M, R* Z, R* D, R* Q, Ctrl* ctrl, const McArgs& A, int grid, double* part,
                            cudaStream_t st) {
    SGB_SUN_DISPATCH((sun_sweeps_n<R, 2>(M, Z, D, Q, ctrl, A, grid, part, st)), (sun_sweeps_n<R, 3>(M, Z, D, Q, ctrl, A, grid, part, st)),
                     (sun_sweeps_n<R, 4>(M, Z, D, Q, ctrl, A, grid, part, st)), (sun_sweeps_n<R, 5>(M, Z, D, Q, ctrl, A, grid, part, st)))
}

template <class R>
int sun_launch_local_sweeps_ewald(const Model<R>& M, R* Z, R* D, R* Q, const McArgs& A, const EwaldDev& E, double* F,
                                  double* part, cudaStream_t st) {
    SGB_SUN_DISPATCH((sun_sweeps_ewald_n<R, 2>(M, Z, D, Q, A, E, F, part, st)), (sun_sweeps_ewald_n<R, 3>(M, Z, D, Q, A, E, F, part, st)),
                     (sun_sweeps_ewald_n<R, 4>(M, Z, D, Q, A, E, F, part, st)), (sun_sweeps_ewald_n<R, 5>(M, Z, D, Q, A, E, F, part, st)))
}

template <class R>
int sun_mc_max_blocks(const Model<R>& M, int* bps) {
    const size_t smem = (size_t)M.tables_bytes;
    SGB_SUN_DISPATCH((sun_mc_occ_n<R, 2>(smem, bps)), (sun_mc_occ_n<R, 3>(smem, bps)), (sun_mc_occ_n<R, 4>(smem, bps)),
                     (sun_mc_occ_n<R, 5>(smem, bps)))
}

template <class R>
int sun_launch_local_dE(const Model<R>& M, const R* Z, const R* D, const R* Q, int site, const SunKet& zk, double* out,
                        cudaStream_t st) {
    SGB_SUN_DISPATCH((sun_dE_n<R, 2>(M, Z, D, Q, site, zk, out, st)), (sun_dE_n<R, 3>(M, Z, D, Q, site, zk, out, st)),
                     (sun_dE_n<R, 4>(M, Z, D, Q, site, zk, out, st)), (sun_dE_n<R, 5>(M, Z, D, Q, site, zk, out, st)))
}

#define SGB_SUN_INST(R)                                                                                         \
    template int sun_launch_heun<R>(const Model<R>&, R*, R*, R*, R*, R*, Ctrl*, int, double, double, double,    \
                                    uint64_t, uint64_t, const double*, const LaunchInfo&, cudaStream_t);        \
    template int sun_launch_midpoint<R>(const Model<R>&, R*, R*, R*, R*, R*, Ctrl*, int, double, double, double, \
                                        int, const SnapArgs<R>&, const LaunchInfo&, cudaStream_t);              \
    template int sun_max_blocks<R>(int, int, int, size_t, int*);                                                     \
    template int sun_launch_refresh<R>(const Model<R>&, const R*, R*, R*, cudaStream_t);                        \
    template int sun_launch_grad<R>(const Model<R>&, const R*, const R*, const R*, double*, cudaStream_t);      \
    template int sun_launch_energy<R>(const Model<R>&, const R*, const R*, const R*, double*, int, cudaStream_t); \
    template int sun_launch_local_sweeps<R>(const Model<R>&, R*, R*, R*, Ctrl*, const McArgs&, int, double*, cudaStream_t); \
    template int sun_launch_local_sweeps_ewald<R>(const Model<R>&, R*, R*, R*, const McArgs&, const EwaldDev&, double*, \
                                                  double*, cudaStream_t); \
    template int sun_mc_max_blocks<R>(const Model<R>&, int*);                                                    \
    template size_t sun_cluster_smem<R>(const Model<R>&, int);                                                  \
    template int sun_launch_add_dipole_field<R>(const Model<R>&, const R*, const double*, double*, cudaStream_t); \
    template int sun_launch_lr_stage<R>(int, const Model<R>&, R*, R*, R*, R*, const double*, double, double, double, uint64_t, \
                                        uint64_t, const double*, double*, const SnapArgs<R>*, int, cudaStream_t); \
    template int sun_launch_heun_cluster<R>(const Model<R>&, R*, R*, R*, int, int, double, double, double, uint64_t, \
                                            uint64_t, const double*, cudaStream_t);                            \
    template int sun_launch_local_dE<R>(const Model<R>&, const R*, const R*, const R*, int, const SunKet&, double*, cudaStream_t);
// SGB_INST_PRECISION (32 or 64) builds this file once per precision, in parallel.
#if !defined(SGB_INST_PRECISION) || SGB_INST_PRECISION == 32
SGB_SUN_INST(float)
#endif
#if !defined(SGB_INST_PRECISION) || SGB_INST_PRECISION == 64
SGB_SUN_INST(double)
#endif
