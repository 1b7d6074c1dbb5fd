// sgb_dipole.cu -- dipole-mode kernels for sm_103a.
//
// Reference algorithms (Sunny.jl v0.9.2):
//   gradient      src/System/Interactions.jl:516-592, src/System/OnsiteCoupling.jl:316-425
//   energy        src/System/Interactions.jl:401-508
//   Langevin Heun src/Integrators.jl:266-275, 288-298, 313-332
//   midpoint      src/Integrators.jl:361-371, 379-413
//
// Design: every step kernel is persistent (cooperative launch, one CTA per slot of the
// SM budget). A thread owns SPT sites for the whole launch and keeps their spins, the
// Heun increment and the noise in registers; only the spins that neighbours need are
// exchanged through L2-resident SoA buffers, separated by a bounded grid barrier. The
// implicit midpoint iteration speculatively writes both the next iterate's midpoint
// spins and the next step's starting midpoint spins, so each fixed-point iteration costs
// exactly one barrier; the FP64 convergence sum rotates through three accumulators.
#include "sgb_internal.h"
#include <cooperative_groups.h>
#include <stdio.h>

#include "sgb_device.cuh"

namespace cg = cooperative_groups;

namespace {
using namespace sgbdev;

template <class R, int SPT, bool INJECT>
__global__ void __launch_bounds__(sgb_maxblock(sizeof(R) == 8, false, SPT))
k_dip_heun(Model<R> M, R* S, R* P, Ctrl* ctrl, int nsteps, R dt, R lam, R nscale, uint64_t seed,
           uint64_t step0, const double* noise) {
    extern __shared__ __align__(16) unsigned char smem[];
    Tab<R> T = stage_tables<R>(M, smem);
    const int ns = M.ns;
    const int nthr = gridDim.x * blockDim.x;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    R* Sx = S; R* Sy = S + ns; R* Sz = S + 2 * ns;
    R* Px = P; R* Py = P + ns; R* Pz = P + 2 * ns;
    R s[SPT][3], d1[SPT][3], xi[SPT][3];
#pragma unroll
    for (int k = 0; k < SPT; k++) {
        int site = tid + k * nthr;
        if (site < ns) { s[k][0] = Sx[site]; s[k][1] = Sy[site]; s[k][2] = Sz[site]; }
    }
    for (int step = 0; step < nsteps; ++step) {
#pragma unroll
        for (int k = 0; k < SPT; k++) {
            int site = tid + k * nthr;
            if (site >= ns) continue;
            if (nscale == (R)0) {
                xi[k][0] = xi[k][1] = xi[k][2] = 0;
            } else if (INJECT) {
                const double* nz = noise + ((size_t)step * ns + site) * 3;
                xi[k][0] = (R)nz[0] * nscale; xi[k][1] = (R)nz[1] * nscale; xi[k][2] = (R)nz[2] * nscale;
            } else {
                R g4[4];
                sgb_normals4<R>(seed, 0u, step0 + step, (uint32_t)site, 0u, g4);
                xi[k][0] = g4[0] * nscale; xi[k][1] = g4[1] * nscale; xi[k][2] = g4[2] * nscale;
            }
            R gx, gy, gz;
            grad_single<R>(M, T, site, s[k][0], s[k][1], s[k][2], Sx, Sy, Sz, gx, gy, gz);
            rhs_dipole<R>(s[k][0], s[k][1], s[k][2], xi[k][0], xi[k][1], xi[k][2], gx, gy, gz, dt, lam,
                          d1[k][0], d1[k][1], d1[k][2]);
            R px = s[k][0] + d1[k][0], py = s[k][1] + d1[k][1], pz = s[k][2] + d1[k][2];
            normalize_dip<R>(px, py, pz, __ldg(M.kappa + site));
            Px[site] = px; Py[site] = py; Pz[site] = pz;
        }
        if (!sgb_grid_barrier(ctrl, gridDim.x)) return;
#pragma unroll
        for (int k = 0; k < SPT; k++) {
            int site = tid + k * nthr;
            if (site >= ns) continue;
            R px = Px[site], py = Py[site], pz = Pz[site];
            R gx, gy, gz, e0, e1, e2;
            grad_single<R>(M, T, site, px, py, pz, Px, Py, Pz, gx, gy, gz);
            rhs_dipole<R>(px, py, pz, xi[k][0], xi[k][1], xi[k][2], gx, gy, gz, dt, lam, e0, e1, e2);
            R nx = s[k][0] + (d1[k][0] + e0) / 2, ny = s[k][1] + (d1[k][1] + e1) / 2,
              nz = s[k][2] + (d1[k][2] + e2) / 2;
            normalize_dip<R>(nx, ny, nz, __ldg(M.kappa + site));
            s[k][0] = nx; s[k][1] = ny; s[k][2] = nz;
            Sx[site] = nx; Sy[site] = ny; Sz[site] = nz;
        }
        if (step + 1 < nsteps) {
            if (!sgb_grid_barrier(ctrl, gridDim.x)) return;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) ctrl->steps_done = nsteps;
}

template <class R>
__device__ __forceinline__ void write_snapshot_dip(const Model<R>& M, const SnapArgs<R>& sn, int t, int site,
                                                   R sx, R sy, R sz) {
    const int ns = M.ns;
    const int cell = site % M.ncell, a = site / M.ncell;
    for (int o = 0; o < sn.nobs; o++) {
        const R* op = sn.ops + (size_t)o * 3 * ns;
        R v = __ldg(op + site) * sx + __ldg(op + ns + site) * sy + __ldg(op + 2 * ns + site) * sz;
        size_t idx = (((size_t)t * sn.nobs + o) * M.na + a) * M.ncell + cell;
        sn.buf[2 * idx] = v * sn.scale;
        sn.buf[2 * idx + 1] = 0;
    }
}

// Degree-k polynomial extrapolation of the next state from c = S_{n+1}, s = S_n and the
// history h1 = S_{n-1}, h2 = S_{n-2}, h3 = S_{n-3} (Newton backward differences).
template <class R>
__device__ __forceinline__ R extrap(int k, R c, R s, R h1, R h2, R h3) {
    switch (k) {
        case 1: return 2 * c - s;
        case 2: return 3 * (c - s) + h1;
        case 3: return 4 * (c + h1) - 6 * s - h2;
        case 4: return 5 * (c - h2) + 10 * (h1 - s) + h3;
    }
    return c;
}

// Spherical midpoint, Integrators.jl:379-413. H holds 3 rotating SoA buffers of
// midpoint spins S-hat (3*3*ns reals). With PRED, each step after the first starts its
// fixed-point iteration from the degree-`ord` extrapolation of the last states (kept in
// registers) instead of S' = S, and a step is accepted from its second iteration on.
template <class R, int SPT, bool PRED>
__global__ void __launch_bounds__(sgb_maxblock(sizeof(R) == 8, false, SPT))
k_dip_midpoint(Model<R> M, R* S, R* H, Ctrl* ctrl, int nsteps, R dt, R lam, double atol2,
               int max_iters, SnapArgs<R> snap, int ord) {
    extern __shared__ __align__(16) unsigned char smem[];
    Tab<R> T = stage_tables<R>(M, smem);
    const int ns = M.ns;
    const int nthr = gridDim.x * blockDim.x;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const bool leader = (blockIdx.x == 0 && threadIdx.x == 0);
    R s[SPT][3], sp[SPT][3], sc[SPT][3];
    constexpr int PH = PRED ? SPT : 1;
    R h1[PH][3], h2[PH][3], h3[PH][3], pn[PH][3];   // history and next first iterate (PRED)
    int cur = 0;
#pragma unroll
    for (int k = 0; k < SPT; k++) {
        int site = tid + k * nthr;
        if (site >= ns) continue;
        s[k][0] = S[site]; s[k][1] = S[ns + site]; s[k][2] = S[2 * ns + site];
        R hx = (s[k][0] + s[k][0]) / 2, hy = (s[k][1] + s[k][1]) / 2, hz = (s[k][2] + s[k][2]) / 2;
        normalize_dip<R>(hx, hy, hz, __ldg(M.kappa + site));
        R* Hc = H + (size_t)cur * 3 * ns;
        Hc[site] = hx; Hc[ns + site] = hy; Hc[2 * ns + site] = hz;
        if (snap.enabled) write_snapshot_dip<R>(M, snap, snap.t0, site, s[k][0], s[k][1], s[k][2]);
    }
    if (leader) { ctrl->acc[0] = 0.0; ctrl->acc[1] = 0.0; ctrl->acc[2] = 0.0; }
    if (!sgb_grid_barrier(ctrl, gridDim.x)) return;
    long long itg = 0;
    int done = 0;
    for (int step = 0; step < nsteps; ++step) {
        const int oe = PRED ? min(ord, step + 1) : 0;   // extrapolation order for the next step
#pragma unroll
        for (int k = 0; k < SPT; k++) {
            if (PRED && step > 0) { sp[k][0] = pn[k % PH][0]; sp[k][1] = pn[k % PH][1]; sp[k][2] = pn[k % PH][2]; }
            else { sp[k][0] = s[k][0]; sp[k][1] = s[k][1]; sp[k][2] = s[k][2]; }
        }
        bool conv = false;
        for (int it = 0; it < max_iters; ++it) {
            const int nxt = (cur + 1) % 3, nst = (cur + 2) % 3;
            const R* Hc = H + (size_t)cur * 3 * ns;
            R* Hn = H + (size_t)nxt * 3 * ns;
            R* Hs = H + (size_t)nst * 3 * ns;
            R acc = 0;   // per-site terms in R, block and grid sums in FP64
#pragma unroll
            for (int k = 0; k < SPT; k++) {
                int site = tid + k * nthr;
                if (site >= ns) continue;
                const R kap = __ldg(M.kappa + site);
                R hx = (s[k][0] + sp[k][0]) / 2, hy = (s[k][1] + sp[k][1]) / 2, hz = (s[k][2] + sp[k][2]) / 2;
                normalize_dip<R>(hx, hy, hz, kap);
                R gx, gy, gz, dx, dy, dz;
                grad_single<R>(M, T, site, hx, hy, hz, Hc, Hc + ns, Hc + 2 * ns, gx, gy, gz);
                rhs_dipole<R>(hx, hy, hz, (R)0, (R)0, (R)0, gx, gy, gz, dt, lam, dx, dy, dz);
                R qx = s[k][0] + dx, qy = s[k][1] + dy, qz = s[k][2] + dz;
                R ex = sp[k][0] - qx, ey = sp[k][1] - qy, ez = sp[k][2] - qz;
                acc += ex * ex + ey * ey + ez * ez;
                sp[k][0] = qx; sp[k][1] = qy; sp[k][2] = qz;
                // candidate midpoint for the next iteration
                R nx = (s[k][0] + qx) / 2, ny = (s[k][1] + qy) / 2, nz = (s[k][2] + qz) / 2;
                normalize_dip<R>(nx, ny, nz, kap);
                Hn[site] = nx; Hn[ns + site] = ny; Hn[2 * ns + site] = nz;
                // candidate new state and the next step's first midpoint
                if (!PRED || it > 0) {
                    R cx = qx, cy = qy, cz = qz;
                    normalize_dip<R>(cx, cy, cz, kap);
                    sc[k][0] = cx; sc[k][1] = cy; sc[k][2] = cz;
                    R px = cx, py = cy, pz = cz;
                    if (PRED) {
                        const int j = k % PH;
                        px = extrap<R>(oe, cx, s[k][0], h1[j][0], h2[j][0], h3[j][0]);
                        py = extrap<R>(oe, cy, s[k][1], h1[j][1], h2[j][1], h3[j][1]);
                        pz = extrap<R>(oe, cz, s[k][2], h1[j][2], h2[j][2], h3[j][2]);
                        pn[j][0] = px; pn[j][1] = py; pn[j][2] = pz;
                    }
                    R mx = (cx + px) / 2, my = (cy + py) / 2, mz = (cz + pz) / 2;
                    normalize_dip<R>(mx, my, mz, kap);
                    Hs[site] = mx; Hs[ns + site] = my; Hs[2 * ns + site] = mz;
                }
            }
            double bsum = sgb_block_sum_r<R>(acc);
            const int slot = (int)(itg % 3);
            if (threadIdx.x == 0) atomicAdd(&ctrl->acc[slot], bsum);
            if (leader) { ctrl->acc[(slot + 1) % 3] = 0.0; ctrl->iters += 1; }
            if (!sgb_grid_barrier(ctrl, gridDim.x)) return;
            double tot = __ldcg(&ctrl->acc[slot]);
            itg++;
            if (tot <= atol2 && (!PRED || it > 0)) {  // false for NaN, as fast_isapprox
                conv = true;
#pragma unroll
                for (int k = 0; k < SPT; k++) {
                    if (PRED) {
                        const int j = k % PH;
                        for (int q = 0; q < 3; q++) { h3[j][q] = h2[j][q]; h2[j][q] = h1[j][q]; h1[j][q] = s[k][q]; }
                    }
                    s[k][0] = sc[k][0]; s[k][1] = sc[k][1]; s[k][2] = sc[k][2];
                }
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
                if (site < ns) write_snapshot_dip<R>(M, snap, snap.t0 + done / snap.measperiod, site,
                                                     s[k][0], s[k][1], s[k][2]);
            }
        }
    }
#pragma unroll
    for (int k = 0; k < SPT; k++) {
        int site = tid + k * nthr;
        if (site < ns) { S[site] = s[k][0]; S[ns + site] = s[k][1]; S[2 * ns + site] = s[k][2]; }
    }
    if (leader) ctrl->steps_done = done;
}

template <class R>
__global__ void __launch_bounds__(SGB_BLOCK)
k_dip_grad(Model<R> M, const R* S, double* out) {
    extern __shared__ __align__(16) unsigned char smem[];
    Tab<R> T = stage_tables<R>(M, smem);
    const int ns = M.ns;
    const bool inh = M.ioff || M.oidx;
    for (int site = blockIdx.x * blockDim.x + threadIdx.x; site < ns; site += gridDim.x * blockDim.x) {
        R gx, gy, gz;
        if (inh) {
            grad_single<R>(M, T, site, S[site], S[ns + site], S[2 * ns + site], S, S + ns, S + 2 * ns, gx, gy, gz);
        } else {
            SiteIdx ix = decompose(site, M.L1, M.L2, M.L3);
            grad_site<R>(M, T, site, ix, S[site], S[ns + site], S[2 * ns + site], S, S + ns, S + 2 * ns, gx, gy, gz);
        }
        out[3 * site] = gx; out[3 * site + 1] = gy; out[3 * site + 2] = gz;
    }
}

// Energy of one non-culled coupling row between spins s (this site) and t (Interactions.jl:466-505).
template <class R>
__device__ __forceinline__ double pair_energy_dip(const Model<R>& M, const DBond<R>& B, const R* bqtab, double sx,
                                                  double sy, double sz, double tx, double ty, double tz) {
    double E = (double)B.scalar;
    if (B.jkind == 0) E += (double)B.J[0] * (sx * tx + sy * ty + sz * tz);
    else {
        double jx = (double)B.J[0] * tx + (double)B.J[3] * ty + (double)B.J[6] * tz;
        double jy = (double)B.J[1] * tx + (double)B.J[4] * ty + (double)B.J[7] * tz;
        double jz = (double)B.J[2] * tx + (double)B.J[5] * ty + (double)B.J[8] * tz;
        E += sx * jx + sy * jy + sz * jz;
    }
    if (M.dipole_mode && B.bqkind != 0) {
        double Qi[5], Qj[5];
        quad5<double>(sx, sy, sz, Qi);
        quad5<double>(tx, ty, tz, Qj);
        double acc = 0;
        if (B.bqkind == 1) {
            for (int q = 0; q < 5; q++) acc += Qi[q] * (biquad_metric(q) * Qj[q]);
            acc *= (double)B.bq;
        } else {
            const R* Bm = bqtab + 25 * B.bqidx;
            for (int q = 0; q < 5; q++)
                for (int p = 0; p < 5; p++) acc += Qi[q] * (double)Bm[q + 5 * p] * Qj[p];
        }
        E += acc;
    }
    return E;
}

// FP64 energy and magnetisation (Interactions.jl:401-508): partials[block][4].
template <class R>
__global__ void __launch_bounds__(SGB_BLOCK)
k_dip_energy(Model<R> M, const R* S, double* partials) {
    extern __shared__ __align__(16) unsigned char smem[];
    Tab<R> T = stage_tables<R>(M, smem);
    const int ns = M.ns;
    double E = 0, mx = 0, my = 0, mz = 0;
    for (int site = blockIdx.x * blockDim.x + threadIdx.x; site < ns; site += gridDim.x * blockDim.x) {
        SiteIdx ix = decompose(site, M.L1, M.L2, M.L3);
        double sx = S[site], sy = S[ns + site], sz = S[2 * ns + site];
        mx += sx; my += sy; mz += sz;
        if (M.h) E += (double)M.h[site] * sx + (double)M.h[ns + site] * sy + (double)M.h[2 * ns + site] * sz;
        const int a = ix.a;
        if (M.dipole_mode) {
            int km;
            const R* cr = stevens_at<R>(M, T, site, a, km);
            double c[28];
            for (int q = 0; q < 28; q++) c[q] = (double)cr[q];
            double gx = 0, gy = 0, gz = 0;
            E += classical_aniso<double>(c, km, sx, sy, sz, gx, gy, gz);
        }
        if (M.ioff) {
            // per-site couplings: the non-culled rows of this site's own list
            for_site_bonds<R>(M, T, site, a, [&](const DBond<R>& B, const R* bq, int js) {
                if (B.fwd) E += pair_energy_dip<R>(M, B, bq, sx, sy, sz, S[js], S[ns + js], S[2 * ns + js]);
            });
            continue;
        }
        for (int b = T.boff[a]; b < T.boff[a + 1]; b++) {
            const DBond<R>& B = T.bonds[b];
            if (!B.fwd) continue;
            int x1 = sgb_wrap_pos(ix.c1 + B.n[0], M.L1);
            int x2 = sgb_wrap_pos(ix.c2 + B.n[1], M.L2);
            int x3 = sgb_wrap_pos(ix.c3 + B.n[2], M.L3);
            int js = x1 + M.L1 * (x2 + M.L2 * (x3 + M.L3 * B.j));
            double tx = S[js], ty = S[ns + js], tz = S[2 * ns + js];
            E += (double)B.scalar;
            if (B.jkind == 0) E += (double)B.J[0] * (sx * tx + sy * ty + sz * tz);
            else {
                double jx = (double)B.J[0] * tx + (double)B.J[3] * ty + (double)B.J[6] * tz;
                double jy = (double)B.J[1] * tx + (double)B.J[4] * ty + (double)B.J[7] * tz;
                double jz = (double)B.J[2] * tx + (double)B.J[5] * ty + (double)B.J[8] * tz;
                E += sx * jx + sy * jy + sz * jz;
            }
            if (M.dipole_mode && B.bqkind != 0) {
                double Qi[5], Qj[5];
                quad5<double>(sx, sy, sz, Qi);
                quad5<double>(tx, ty, tz, Qj);
                double acc = 0;
                if (B.bqkind == 1) {
                    for (int q = 0; q < 5; q++) acc += Qi[q] * (biquad_metric(q) * Qj[q]);
                    acc *= (double)B.bq;
                } else {
                    const R* Bm = T.bq + 25 * B.bqidx;
                    for (int q = 0; q < 5; q++)
                        for (int p = 0; p < 5; p++) acc += Qi[q] * (double)Bm[q + 5 * p] * Qj[p];
                }
                E += acc;
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

// Sums partials[n][ncomp] in a fixed order (deterministic) into out[ncomp].
__global__ void k_reduce_partials(const double* partials, int n, int ncomp, double* out) {
    for (int c = 0; c < ncomp; c++) {
        double v = 0;
        for (int i = threadIdx.x; i < n; i += blockDim.x) v += partials[(size_t)i * ncomp + c];
        double t = sgb_block_sum(v);
        if (threadIdx.x == 0) out[c] = t;
        __syncthreads();
    }
}

template <class R>
__global__ void k_noise_export(int sun, int N, int ns, uint64_t seed, uint64_t step, double* out) {
    for (int site = blockIdx.x * blockDim.x + threadIdx.x; site < ns; site += gridDim.x * blockDim.x) {
        if (!sun) {
            R g4[4];
            sgb_normals4<R>(seed, 0u, step, (uint32_t)site, 0u, g4);
            out[3 * site] = (double)g4[0]; out[3 * site + 1] = (double)g4[1]; out[3 * site + 2] = (double)g4[2];
        } else {
            for (int k = 0; k < N; k += 2) {
                R g4[4];
                sgb_normals4<R>(seed, 0u, step, (uint32_t)site, (uint32_t)(k / 2), g4);
                const R r2 = (R)0.70710678118654752440;
                out[2 * ((size_t)site * N + k)] = (double)(g4[0] * r2);
                out[2 * ((size_t)site * N + k) + 1] = (double)(g4[1] * r2);
                if (k + 1 < N) {
                    out[2 * ((size_t)site * N + k + 1)] = (double)(g4[2] * r2);
                    out[2 * ((size_t)site * N + k + 1) + 1] = (double)(g4[3] * r2);
                }
            }
        }
    }
}

__global__ void k_fill(double* p, size_t n, double v) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) p[i] = v;
}

template <class K>
int set_smem_attr(K kernel, size_t smem) {
    if (smem > 48 * 1024) {
        if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
            return SGB_ERR_CUDA;
    }
    return SGB_OK;
}

// Small lattices: one thread-block cluster holds the whole state in distributed shared
// memory, CTA r owning sites [r*nsl, (r+1)*nsl) as [3][nsl] slices of S, the predictor
// P, the first increment and the noise. Neighbour spins are read from the owning CTA's
// shared memory, and the two Heun stages of a step are separated by the cluster's
// hardware barrier instead of a grid barrier through L2. Same per-site arithmetic and
// noise stream as k_dip_heun.
template <class R, bool INJECT, bool GEN>
__global__ void __launch_bounds__(SGB_CLUSTER_BLOCK) k_dip_heun_cluster(Model<R> M, R* S, int nsl, int nsteps, R dt, R lam,
                                                                       R nscale, uint64_t seed, uint64_t step0,
                                                                       const double* noise) {
    extern __shared__ __align__(16) unsigned char smem[];
    cg::cluster_group cl = cg::this_cluster();
    Tab<R> T = stage_tables<R>(M, smem);
    const int rank = (int)cl.block_rank();
    const int ns = M.ns;
    R* lS = reinterpret_cast<R*>(smem + ((M.tables_bytes + 15) / 16) * 16);   // [3][nsl]
    R* lP = lS + 3 * nsl;
    R* lD = lP + 3 * nsl;
    R* lX = lD + 3 * nsl;
    // per owned site, staged once so that the steps do no index loads or divisions: for each
    // bond the neighbour's CTA and local index packed as rank << 11 | local (nsl <= 2048, at
    // most 16 CTAs), and the site's sublattice
    unsigned short* lN = reinterpret_cast<unsigned short*>(lX + 3 * nsl);   // [kb][nsl]
    unsigned char* lA = reinterpret_cast<unsigned char*>(lN + (size_t)M.kb * nsl);
    __shared__ const R* rS[SGB_CLUSTER_MAX];
    __shared__ const R* rP[SGB_CLUSTER_MAX];
    if (threadIdx.x < cl.num_blocks()) {
        rS[threadIdx.x] = cl.map_shared_rank(lS, threadIdx.x);
        rP[threadIdx.x] = cl.map_shared_rank(lP, threadIdx.x);
    }
    const int s0 = rank * nsl, n = max(0, min(ns, s0 + nsl) - s0);
    // the noise of one step for this thread's sites, into lX
    auto fill_noise = [&](int step) {
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const int site = s0 + i;
            R x0 = 0, x1 = 0, x2 = 0;
            if (nscale != (R)0) {
                if (INJECT) {
                    const double* nz = noise + ((size_t)step * ns + site) * 3;
                    x0 = (R)nz[0] * nscale; x1 = (R)nz[1] * nscale; x2 = (R)nz[2] * nscale;
                } else {
                    R g4[4];
                    sgb_normals4<R>(seed, 0u, step0 + step, (uint32_t)site, 0u, g4);
                    x0 = g4[0] * nscale; x1 = g4[1] * nscale; x2 = g4[2] * nscale;
                }
            }
            lX[i] = x0; lX[nsl + i] = x1; lX[2 * nsl + i] = x2;
        }
    };
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int site = s0 + i, a = site / M.ncell;
        lS[i] = S[site]; lS[nsl + i] = S[ns + site]; lS[2 * nsl + i] = S[2 * ns + site];
        lA[i] = (unsigned char)a;
        for (int b = 0; b < T.boff[a + 1] - T.boff[a]; b++) {
            const int j = __ldg(M.nbr + (size_t)b * ns + site), q = j / nsl;
            lN[(size_t)b * nsl + i] = (unsigned short)((q << 11) | (j - q * nsl));
        }
    }
    if (nsteps > 0) fill_noise(0);
    cl.sync();
    auto ldS = [&](int v, R& x, R& y, R& z) {
        const R* b = rS[v >> 11];
        const int l = v & 2047;
        x = b[l]; y = b[nsl + l]; z = b[2 * nsl + l];
    };
    auto ldP = [&](int v, R& x, R& y, R& z) {
        const R* b = rP[v >> 11];
        const int l = v & 2047;
        x = b[l]; y = b[nsl + l]; z = b[2 * nsl + l];
    };
    for (int step = 0; step < nsteps; ++step) {
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const int site = s0 + i, a = lA[i];
            const R x0 = lX[i], x1 = lX[nsl + i], x2 = lX[2 * nsl + i];
            const R sx = lS[i], sy = lS[nsl + i], sz = lS[2 * nsl + i];
            R hx = 0, hy = 0, hz = 0;
            if (M.h) { hx = __ldg(M.h + site); hy = __ldg(M.h + ns + site); hz = __ldg(M.h + 2 * ns + site); }
            const unsigned short* ip = lN + i;
            R gx, gy, gz, d0, d1, d2;
            grad_nbi_ld<R, GEN, 6>(M, T, a, [ip, nsl](int b) { return (int)ip[(size_t)b * nsl]; }, ldS, hx, hy, hz, sx, sy,
                                   sz, gx, gy, gz);
            rhs_dipole<R>(sx, sy, sz, x0, x1, x2, gx, gy, gz, dt, lam, d0, d1, d2);
            R px = sx + d0, py = sy + d1, pz = sz + d2;
            normalize_dip<R>(px, py, pz, __ldg(M.kappa + site));
            lP[i] = px; lP[nsl + i] = py; lP[2 * nsl + i] = pz;
            lD[i] = d0; lD[nsl + i] = d1; lD[2 * nsl + i] = d2;
        }
        cl.sync();
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const int site = s0 + i, a = lA[i];
            const R px = lP[i], py = lP[nsl + i], pz = lP[2 * nsl + i];
            R hx = 0, hy = 0, hz = 0;
            if (M.h) { hx = __ldg(M.h + site); hy = __ldg(M.h + ns + site); hz = __ldg(M.h + 2 * ns + site); }
            const unsigned short* ip = lN + i;
            R gx, gy, gz, e0, e1, e2;
            grad_nbi_ld<R, GEN, 6>(M, T, a, [ip, nsl](int b) { return (int)ip[(size_t)b * nsl]; }, ldP, hx, hy, hz, px, py,
                                   pz, gx, gy, gz);
            rhs_dipole<R>(px, py, pz, lX[i], lX[nsl + i], lX[2 * nsl + i], gx, gy, gz, dt, lam, e0, e1, e2);
            R nx = lS[i] + (lD[i] + e0) / 2, ny = lS[nsl + i] + (lD[nsl + i] + e1) / 2, nz = lS[2 * nsl + i] + (lD[2 * nsl + i] + e2) / 2;
            normalize_dip<R>(nx, ny, nz, __ldg(M.kappa + site));
            lS[i] = nx; lS[nsl + i] = ny; lS[2 * nsl + i] = nz;
        }
        // split cluster barrier: the next step's noise (own sites, read by this thread only)
        // is drawn between the arrival and the wait
        asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
        if (step + 1 < nsteps) fill_noise(step + 1);
        asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        S[s0 + i] = lS[i]; S[ns + s0 + i] = lS[nsl + i]; S[2 * ns + s0 + i] = lS[2 * nsl + i];
    }
}

// One snapshot row t of every site's observables (the snapshot of the fused kernels).
template <class R>
__global__ void k_dip_snapshot(Model<R> M, const R* S, SnapArgs<R> sn, int t) {
    for (int site = blockIdx.x * blockDim.x + threadIdx.x; site < M.ns; site += gridDim.x * blockDim.x)
        write_snapshot_dip<R>(M, sn, t, site, S[site], S[M.ns + site], S[2 * M.ns + site]);
}

template <class K>
int coop_launch(K kernel, const LaunchInfo& li, void** args, cudaStream_t st) {
    if (set_smem_attr(kernel, li.smem) != SGB_OK) return SGB_ERR_CUDA;
    cudaError_t e = cudaLaunchCooperativeKernel((const void*)kernel, dim3(li.grid), dim3(li.block), args, li.smem, st);
    return e == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

}  // namespace

// ------------------------------------------------------------------------------------
// launchers
// ------------------------------------------------------------------------------------
template <class R>
int dip_launch_heun(const Model<R>& M, R* S, R* P, Ctrl* ctrl, int nsteps, double dt, double lam,
                    double noise_scale, uint64_t seed, uint64_t step0, const double* noise,
                    const LaunchInfo& li, cudaStream_t st) {
    Model<R> m = M;
    R rdt = (R)dt, rlam = (R)lam, rns = (R)noise_scale;
    void* args[] = {&m, &S, &P, &ctrl, &nsteps, &rdt, &rlam, &rns, &seed, &step0, &noise};
#define SGB_HEUN_CASE(SPTV)                                                                  \
    case SPTV:                                                                               \
        return noise ? coop_launch(k_dip_heun<R, SPTV, true>, li, args, st)                  \
                     : coop_launch(k_dip_heun<R, SPTV, false>, li, args, st);
    switch (li.spt) {
        SGB_HEUN_CASE(1)
        SGB_HEUN_CASE(2)
        SGB_HEUN_CASE(4)
        SGB_HEUN_CASE(8)
    }
#undef SGB_HEUN_CASE
    return SGB_ERR_ARG;
}

template <class R>
int dip_launch_snapshot(const Model<R>& M, const R* S, const SnapArgs<R>& sn, int t, cudaStream_t st) {
    int grid = (M.ns + SGB_BLOCK - 1) / SGB_BLOCK;
    if (grid > 4096) grid = 4096;
    k_dip_snapshot<R><<<grid, SGB_BLOCK, 0, st>>>(M, S, sn, t);
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

template <class R>
size_t dip_cluster_smem(const Model<R>& M, int nsl) {
    return (size_t)((M.tables_bytes + 15) / 16) * 16 + (size_t)12 * nsl * sizeof(R) + (size_t)2 * M.kb * nsl + nsl;
}

template <class R>
int dip_launch_heun_cluster(const Model<R>& M, R* S, int cs, int nsteps, double dt, double lam, double noise_scale,
                            uint64_t seed, uint64_t step0, const double* noise, cudaStream_t st) {
    const int nsl = (M.ns + cs - 1) / cs;
    const size_t smem = dip_cluster_smem<R>(M, nsl);
    const void* k = noise ? (M.general ? (const void*)k_dip_heun_cluster<R, true, true> : (const void*)k_dip_heun_cluster<R, true, false>)
                          : (M.general ? (const void*)k_dip_heun_cluster<R, false, true> : (const void*)k_dip_heun_cluster<R, false, false>);
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
    R rdt = (R)dt, rlam = (R)lam, rns = (R)noise_scale;
    int ns_ = nsl, nst = nsteps;
    void* args[] = {&m, &S, &ns_, &nst, &rdt, &rlam, &rns, &seed, &step0, &noise};
    return cudaLaunchKernelExC(&cfg, k, args) == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

template <class R>
int dip_launch_midpoint(const Model<R>& M, R* S, R* H, Ctrl* ctrl, int nsteps, double dt, double lam,
                        double atol2, int max_iters, const SnapArgs<R>& snap, const LaunchInfo& li,
                        cudaStream_t st, int order) {
    Model<R> m = M;
    SnapArgs<R> sn = snap;
    R rdt = (R)dt, rlam = (R)lam;
    int ord = order;
    void* args[] = {&m, &S, &H, &ctrl, &nsteps, &rdt, &rlam, &atol2, &max_iters, &sn, &ord};
    // extrapolated first iterates keep their history in registers: 1 or 2 sites per thread
    const bool pred = order > 0 && li.spt <= 2;
    switch (li.spt) {
        case 1: return pred ? coop_launch(k_dip_midpoint<R, 1, true>, li, args, st)
                            : coop_launch(k_dip_midpoint<R, 1, false>, li, args, st);
        case 2: return pred ? coop_launch(k_dip_midpoint<R, 2, true>, li, args, st)
                            : coop_launch(k_dip_midpoint<R, 2, false>, li, args, st);
        case 4: return coop_launch(k_dip_midpoint<R, 4, false>, li, args, st);
        case 8: return coop_launch(k_dip_midpoint<R, 8, false>, li, args, st);
    }
    return SGB_ERR_ARG;
}

template <class R>
int dip_max_blocks(int spt, int block, size_t smem, int* bps) {
    int best = 1 << 30, a = 0;
    auto one = [&](auto k) -> int {
        if (set_smem_attr(k, smem) != SGB_OK) return SGB_ERR_CUDA;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k, block, smem) != cudaSuccess) return SGB_ERR_CUDA;
        best = a < best ? a : best;
        return SGB_OK;
    };
    int rc = SGB_OK;
    switch (spt) {
        case 1: rc |= one(k_dip_heun<R, 1, false>); rc |= one(k_dip_heun<R, 1, true>); rc |= one(k_dip_midpoint<R, 1, false>);
                rc |= one(k_dip_midpoint<R, 1, true>); break;
        case 2: rc |= one(k_dip_heun<R, 2, false>); rc |= one(k_dip_heun<R, 2, true>); rc |= one(k_dip_midpoint<R, 2, false>);
                rc |= one(k_dip_midpoint<R, 2, true>); break;
        case 4: rc |= one(k_dip_heun<R, 4, false>); rc |= one(k_dip_heun<R, 4, true>); rc |= one(k_dip_midpoint<R, 4, false>); break;
        case 8: rc |= one(k_dip_heun<R, 8, false>); rc |= one(k_dip_heun<R, 8, true>); rc |= one(k_dip_midpoint<R, 8, false>); break;
        default: return SGB_ERR_ARG;
    }
    if (rc != SGB_OK) return SGB_ERR_CUDA;
    *bps = best;
    return SGB_OK;
}

template <class R>
int dip_launch_grad(const Model<R>& M, const R* S, double* grad, cudaStream_t st) {
    size_t smem = (size_t)M.tables_bytes;
    if (set_smem_attr(k_dip_grad<R>, smem) != SGB_OK) return SGB_ERR_CUDA;
    int grid = (M.ns + SGB_BLOCK - 1) / SGB_BLOCK;
    if (grid > 4096) grid = 4096;
    k_dip_grad<R><<<grid, SGB_BLOCK, smem, st>>>(M, S, grad);
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

template <class R>
int dip_launch_energy(const Model<R>& M, const R* S, double* partials, int nblocks, cudaStream_t st) {
    size_t smem = (size_t)M.tables_bytes;
    if (set_smem_attr(k_dip_energy<R>, smem) != SGB_OK) return SGB_ERR_CUDA;
    k_dip_energy<R><<<nblocks, SGB_BLOCK, smem, st>>>(M, S, partials);
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

// SGB_INST_PRECISION (32 or 64) builds this file once per precision, in parallel; the
// precision-independent launchers go with the FP64 copy.
#if !defined(SGB_INST_PRECISION) || SGB_INST_PRECISION == 64
int util_launch_reduce(const double* partials, int n, int ncomp, double* out, cudaStream_t st) {
    k_reduce_partials<<<1, SGB_BLOCK, 0, st>>>(partials, n, ncomp, out);
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

#endif

template <class R>
int util_launch_noise_export(int sun, int N, int ns, uint64_t seed, uint64_t step, double* out, cudaStream_t st) {
    int grid = (ns + SGB_BLOCK - 1) / SGB_BLOCK;
    if (grid > 4096) grid = 4096;
    k_noise_export<R><<<grid, SGB_BLOCK, 0, st>>>(sun, N, ns, seed, step, out);
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

#if !defined(SGB_INST_PRECISION) || SGB_INST_PRECISION == 64
int util_launch_fill(double* p, size_t n, double v, cudaStream_t st) {
    k_fill<<<1024, SGB_BLOCK, 0, st>>>(p, n, v);
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

// A grid barrier that expects one more CTA than the launch has, so it can only end by the
// handle's wait limit: every CTA records SGB_ERR_TIMEOUT (or sees the abort flag) and
// returns. Used to show callers that a bounded wait ends and the handle stays usable.
__global__ void k_wait_probe(Ctrl* ctrl) {
    sgb_grid_barrier(ctrl, gridDim.x + 1);
}

int util_launch_wait_probe(Ctrl* ctrl, int grid, cudaStream_t st) {
    k_wait_probe<<<grid, 32, 0, st>>>(ctrl);
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}
#endif

#define SGB_INST(R)                                                                                      \
    template int dip_launch_heun<R>(const Model<R>&, R*, R*, Ctrl*, int, double, double, double, uint64_t, \
                                    uint64_t, const double*, const LaunchInfo&, cudaStream_t);          \
    template int dip_launch_midpoint<R>(const Model<R>&, R*, R*, Ctrl*, int, double, double, double, int,  \
                                        const SnapArgs<R>&, const LaunchInfo&, cudaStream_t, int);      \
    template int dip_launch_grad<R>(const Model<R>&, const R*, double*, cudaStream_t);                    \
    template int dip_launch_energy<R>(const Model<R>&, const R*, double*, int, cudaStream_t);             \
    template int dip_max_blocks<R>(int, int, size_t, int*);                                                    \
    template int dip_launch_heun_cluster<R>(const Model<R>&, R*, int, int, double, double, double, uint64_t, uint64_t, \
                                            const double*, cudaStream_t);                                      \
    template size_t dip_cluster_smem<R>(const Model<R>&, int);                                                 \
    template int dip_launch_snapshot<R>(const Model<R>&, const R*, const SnapArgs<R>&, int, cudaStream_t);     \
    template int util_launch_noise_export<R>(int, int, int, uint64_t, uint64_t, double*, cudaStream_t);
#if !defined(SGB_INST_PRECISION) || SGB_INST_PRECISION == 32
SGB_INST(float)
#endif
#if !defined(SGB_INST_PRECISION) || SGB_INST_PRECISION == 64
SGB_INST(double)
#endif
