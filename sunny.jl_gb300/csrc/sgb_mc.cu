// sgb_mc.cu -- LocalSampler (single-spin Metropolis) for sm_103a, dipole modes.
//
// Reference algorithms (Sunny.jl v0.9.2):
//   step!(sys, ::LocalSampler)   src/MonteCarlo/Samplers.jl:139-158
//   proposals                    src/MonteCarlo/Samplers.jl:1-98, src/System/System.jl:440-460
//   local_energy_change          src/System/Interactions.jl:311-373
//
// Design: Sunny draws a random site per proposal and updates sequentially. Here the
// sites are split by a greedy colouring of the bond graph (built on the host from the
// neighbour table); no two sites of one colour class share a coupling, so every site of
// a class is proposed and accepted or rejected in parallel, and the classes follow one
// another behind a bounded grid barrier inside one persistent cooperative launch. Each
// update reads its neighbours' current spins, so a sweep is a sequence of exact
// single-spin Metropolis updates in colour order. Random numbers are counter-based
// (Philox keyed by seed, sweep and site) or injected by the caller. The accepted ΔE and
// ΔS are summed per thread in FP64 and reduced per block (fixed order).
#include "sgb_internal.h"

#include "sgb_device.cuh"

namespace {
using namespace sgbdev;

// local_energy_change (Interactions.jl:311-373) for a dipole: S at `site` goes from o to
// n. Every bond of the site's sublattice is visited (the reversed copies carry J^T and
// the transposed biquadratic matrix), as Sunny's per-site pair list is.
template <class R>
__device__ inline R mc_local_dE(const Model<R>& M, const Tab<R>& T, int site, int a, const R* S, R ox, R oy, R oz,
                                R nx, R ny, R nz) {
    const int ns = M.ns;
    const R dx = nx - ox, dy = ny - oy, dz = nz - oz;
    R dE = 0;
    if (M.h) dE += M.h[site] * dx + M.h[ns + site] * dy + M.h[2 * ns + site] * dz;
    if (M.dipole_mode) {
        int km;
        const R* cs = stevens_at<R>(M, T, site, a, km);
        if (km > 0) {
            R c[28];
#pragma unroll
            for (int q = 0; q < 28; q++) c[q] = cs[q];
            R g0 = 0, g1 = 0, g2 = 0;
            dE += classical_aniso<R>(c, km, nx, ny, nz, g0, g1, g2) - classical_aniso<R>(c, km, ox, oy, oz, g0, g1, g2);
        }
    }
    R Qn[5], Qo[5];
    bool haveQ = false;
    if (M.ioff) {
        // per-site couplings: every row of the site's own list (reversed copies carry J^T)
        for_site_bonds<R>(M, T, site, a, [&](const DBond<R>& B, const R* bq, int j) {
            const R tx = sgb_ld(S + j), ty = sgb_ld(S + ns + j), tz = sgb_ld(S + 2 * ns + j);
            if (B.jkind == 0) {
                dE += B.J[0] * (dx * tx + dy * ty + dz * tz);
            } else {
                dE += dx * (B.J[0] * tx + B.J[3] * ty + B.J[6] * tz) + dy * (B.J[1] * tx + B.J[4] * ty + B.J[7] * tz) +
                      dz * (B.J[2] * tx + B.J[5] * ty + B.J[8] * tz);
            }
            if (M.dipole_mode && B.bqkind != 0) {
                if (!haveQ) {
                    quad5<R>(nx, ny, nz, Qn);
                    quad5<R>(ox, oy, oz, Qo);
                    haveQ = true;
                }
                R Qj[5];
                quad5<R>(tx, ty, tz, Qj);
                R acc = 0;
                if (B.bqkind == 1) {
#pragma unroll
                    for (int q = 0; q < 5; q++) acc += (Qn[q] - Qo[q]) * ((R)biquad_metric(q) * Qj[q]);
                    acc *= B.bq;
                } else {
                    const R* Bm = bq + 25 * B.bqidx;
#pragma unroll
                    for (int q = 0; q < 5; q++) {
                        R r = 0;
#pragma unroll
                        for (int p = 0; p < 5; p++) r += Bm[q + 5 * p] * Qj[p];
                        acc += (Qn[q] - Qo[q]) * r;
                    }
                }
                dE += acc;
            }
        });
        return dE;
    }
    // neighbour indices and spins are fetched MC_GATHER bonds at a time, so that their
    // loads are in flight together instead of one dependent pair of loads per bond
    constexpr int MC_GATHER = 8;
    const int b0 = T.boff[a], b1 = T.boff[a + 1];
    for (int bb = b0; bb < b1; bb += MC_GATHER) {
        int js[MC_GATHER];
        R txs[MC_GATHER], tys[MC_GATHER], tzs[MC_GATHER];
#pragma unroll
        for (int g = 0; g < MC_GATHER; g++)
            if (bb + g < b1) js[g] = __ldg(M.nbr + (size_t)(bb + g - b0) * ns + site);
#pragma unroll
        for (int g = 0; g < MC_GATHER; g++)
            if (bb + g < b1) { txs[g] = sgb_ld(S + js[g]); tys[g] = sgb_ld(S + ns + js[g]); tzs[g] = sgb_ld(S + 2 * ns + js[g]); }
#pragma unroll
        for (int g = 0; g < MC_GATHER; g++) {
            if (bb + g >= b1) break;
            const int b = bb + g;
            const DBond<R>& B = T.bonds[b];
            const R tx = txs[g], ty = tys[g], tz = tzs[g];
            if (B.jkind == 0) {
                dE += B.J[0] * (dx * tx + dy * ty + dz * tz);
            } else {
                dE += dx * (B.J[0] * tx + B.J[3] * ty + B.J[6] * tz) + dy * (B.J[1] * tx + B.J[4] * ty + B.J[7] * tz) +
                      dz * (B.J[2] * tx + B.J[5] * ty + B.J[8] * tz);
            }
            if (M.dipole_mode && B.bqkind != 0) {
                if (!haveQ) {
                    quad5<R>(nx, ny, nz, Qn);
                    quad5<R>(ox, oy, oz, Qo);
                    haveQ = true;
                }
                R Qj[5];
                quad5<R>(tx, ty, tz, Qj);
                R acc = 0;
                if (B.bqkind == 1) {
#pragma unroll
                    for (int q = 0; q < 5; q++) acc += (Qn[q] - Qo[q]) * ((R)biquad_metric(q) * Qj[q]);
                    acc *= B.bq;
                } else {
                    const R* Bm = T.bq + 25 * B.bqidx;
#pragma unroll
                    for (int q = 0; q < 5; q++) {
                        R r = 0;
#pragma unroll
                        for (int p = 0; p < 5; p++) r += Bm[q + 5 * p] * Qj[p];
                        acc += (Qn[q] - Qo[q]) * r;
                    }
                }
                dE += acc;
            }
        }
    }
    return dE;
}

// One launch runs A.nsweeps sweeps: for every colour class, each thread proposes an update
// for its sites of the class (grid-stride), then all CTAs meet at the barrier.
template <class R, bool INJECT>
__global__ void __launch_bounds__(SGB_BLOCK) k_local_sweeps(Model<R> M, R* S, Ctrl* ctrl, McArgs A, double* partials) {
    extern __shared__ __align__(16) unsigned char smem[];
    Tab<R> T = stage_tables<R>(M, smem);
    __syncthreads();
    const int ns = M.ns;
    const int nthr = gridDim.x * blockDim.x;
    double aE = 0, ax = 0, ay = 0, az = 0;
    bool ok = true;
    for (int k = 0; k < A.nsweeps && ok; k++) {
        const bool partial = (k == A.nsweeps - 1) && A.frac < 1.0;
        const uint64_t sweep = A.sweep0 + (uint64_t)k;
        for (int c = 0; c < A.ncol; c++) {
            for (int idx = A.coff[c] + blockIdx.x * blockDim.x + threadIdx.x; idx < A.coff[c + 1]; idx += nthr) {
                const int site = A.perm[idx];
                double u[4];
                const double* rr = nullptr;
                if (INJECT) {
                    rr = A.rnd + ((size_t)k * ns + site) * 6;
                    u[0] = rr[3]; u[1] = rr[4]; u[2] = rr[5];
                } else {
                    sgb_mc_uniforms4(A.seed, sweep, (uint32_t)site, u);
                }
                if (partial && !(u[2] < A.frac)) continue;
                int kind = A.kind[A.nkind - 1];
                double mag = A.mag[A.nkind - 1];
                for (int i = 0; i < A.nkind - 1; i++)
                    if (u[0] < A.cum[i]) { kind = A.kind[i]; mag = A.mag[i]; break; }
                if (kind == SGB_PROPOSE_DELTA && isinf(mag)) kind = SGB_PROPOSE_UNIFORM;
                const R kap = M.kappa[site];
                const R ox = S[site], oy = S[ns + site], oz = S[2 * ns + site];
                R nx, ny, nz;
                if (kind == SGB_PROPOSE_FLIP) {
                    nx = -ox; ny = -oy; nz = -oz;
                } else {
                    R g[4];
                    if (INJECT) { g[0] = (R)rr[0]; g[1] = (R)rr[1]; g[2] = (R)rr[2]; }
                    else sgb_normals4<R>(A.seed, SGB_MC_STREAM, sweep, (uint32_t)site, 0u, g);
                    if (kind == SGB_PROPOSE_UNIFORM) {
                        nx = g[0]; ny = g[1]; nz = g[2];
                    } else {
                        const R m = (R)mag * kap;
                        nx = ox + m * g[0]; ny = oy + m * g[1]; nz = oz + m * g[2];
                    }
                    normalize_dip<R>(nx, ny, nz, kap);
                }
                const R dE = mc_local_dE<R>(M, T, site, site / M.ncell, S, ox, oy, oz, nx, ny, nz);
                const double e = (double)dE;
                const bool accept = A.kT == 0.0 ? (e <= 0.0) : (u[1] <= exp(-e / A.kT));
                if (accept) {
                    S[site] = nx; S[ns + site] = ny; S[2 * ns + site] = nz;
                    aE += e;
                    ax += (double)nx - (double)ox;
                    ay += (double)ny - (double)oy;
                    az += (double)nz - (double)oz;
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

// Sweeps of a dipole system with dipole-dipole interactions. The term couples every pair of
// sites, so no two updates are independent: one CTA proposes at the sites in the order of
// A.perm, one at a time (thread 0: the proposal, the short-range change mc_local_dE and the
// Ewald change ΔS·F(site) + ½ Δμ·A[0,i,i]·Δμ, Ewald.jl:230-241), and after an accepted move
// every thread adds the move's field g_jᵀ A[cell_site - cell_j, a_j, a_site] g_site ΔS to its
// sites' F. Random numbers as k_local_sweeps.
template <class R, bool INJECT>
__global__ void __launch_bounds__(256) k_local_sweeps_ewald(Model<R> M, R* S, McArgs A, EwaldDev E, double* F,
                                                            double* partials) {
    extern __shared__ __align__(16) unsigned char smem[];
    Tab<R> T = stage_tables<R>(M, smem);
    __shared__ int s_acc;
    __shared__ double s_d[3];
    __syncthreads();
    const int ns = M.ns, ncell = M.ncell;
    double aE = 0, ax = 0, ay = 0, az = 0;
    for (int k = 0; k < A.nsweeps; k++) {
        const bool partial = (k == A.nsweeps - 1) && A.frac < 1.0;
        const uint64_t sweep = A.sweep0 + (uint64_t)k;
        for (int idx = 0; idx < ns; idx++) {
            const int site = A.perm[idx];
            if (threadIdx.x == 0) {
                int acc = 0;
                double u[4];
                const double* rr = nullptr;
                if (INJECT) {
                    rr = A.rnd + ((size_t)k * ns + site) * 6;
                    u[0] = rr[3]; u[1] = rr[4]; u[2] = rr[5];
                } else {
                    sgb_mc_uniforms4(A.seed, sweep, (uint32_t)site, u);
                }
                if (!(partial && !(u[2] < A.frac))) {
                    int kind = A.kind[A.nkind - 1];
                    double mag = A.mag[A.nkind - 1];
                    for (int i = 0; i < A.nkind - 1; i++)
                        if (u[0] < A.cum[i]) { kind = A.kind[i]; mag = A.mag[i]; break; }
                    if (kind == SGB_PROPOSE_DELTA && isinf(mag)) kind = SGB_PROPOSE_UNIFORM;
                    const R kap = M.kappa[site];
                    const R ox = S[site], oy = S[ns + site], oz = S[2 * ns + site];
                    R nx, ny, nz;
                    if (kind == SGB_PROPOSE_FLIP) {
                        nx = -ox; ny = -oy; nz = -oz;
                    } else {
                        R g[4];
                        if (INJECT) { g[0] = (R)rr[0]; g[1] = (R)rr[1]; g[2] = (R)rr[2]; }
                        else sgb_normals4<R>(A.seed, SGB_MC_STREAM, sweep, (uint32_t)site, 0u, g);
                        if (kind == SGB_PROPOSE_UNIFORM) {
                            nx = g[0]; ny = g[1]; nz = g[2];
                        } else {
                            const R m = (R)mag * kap;
                            nx = ox + m * g[0]; ny = oy + m * g[1]; nz = oz + m * g[2];
                        }
                        normalize_dip<R>(nx, ny, nz, kap);
                    }
                    double e = (double)mc_local_dE<R>(M, T, site, site / ncell, S, ox, oy, oz, nx, ny, nz);
                    const double d[3] = {(double)nx - (double)ox, (double)ny - (double)oy, (double)nz - (double)oz};
                    double gd[3];
                    e += ewald_site_delta(E, F, site, ncell, d, gd);
                    if (A.kT == 0.0 ? (e <= 0.0) : (u[1] <= exp(-e / A.kT))) {
                        acc = 1;
                        S[site] = nx; S[ns + site] = ny; S[2 * ns + site] = nz;
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

template <class R>
__global__ void k_local_dE(Model<R> M, const R* S, int site, R nx, R ny, R nz, double* out) {
    extern __shared__ __align__(16) unsigned char smem[];
    Tab<R> T = stage_tables<R>(M, smem);
    __syncthreads();
    if (threadIdx.x != 0) return;
    const int ns = M.ns;
    *out = (double)mc_local_dE<R>(M, T, site, site / M.ncell, S, S[site], S[ns + site], S[2 * ns + site], nx, ny, nz);
}

template <class K>
int set_smem(K kernel, size_t smem) {
    if (smem > 48 * 1024 && cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return SGB_ERR_CUDA;
    return SGB_OK;
}

}  // namespace

template <class R>
int mc_max_blocks(size_t smem, int* bps) {
    int a = 0, b = 0;
    if (set_smem(k_local_sweeps<R, false>, smem) || set_smem(k_local_sweeps<R, true>, smem)) return SGB_ERR_CUDA;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_local_sweeps<R, false>, SGB_BLOCK, smem) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_local_sweeps<R, true>, SGB_BLOCK, smem) != cudaSuccess)
        return SGB_ERR_CUDA;
    *bps = a < b ? a : b;
    return SGB_OK;
}

template <class R>
int mc_launch_sweeps(const Model<R>& M, R* S, Ctrl* ctrl, const McArgs& A, int grid, double* partials, cudaStream_t st) {
    const size_t smem = (size_t)M.tables_bytes;
    Model<R> m = M;
    McArgs a = A;
    void* args[] = {&m, &S, &ctrl, &a, &partials};
    const void* k = A.rnd ? (const void*)k_local_sweeps<R, true> : (const void*)k_local_sweeps<R, false>;
    if (A.rnd ? set_smem(k_local_sweeps<R, true>, smem) : set_smem(k_local_sweeps<R, false>, smem)) return SGB_ERR_CUDA;
    return cudaLaunchCooperativeKernel(k, dim3(grid), dim3(SGB_BLOCK), args, smem, st) == cudaSuccess ? SGB_OK
                                                                                                      : SGB_ERR_CUDA;
}

template <class R>
int mc_launch_local_dE(const Model<R>& M, const R* S, int site, double nx, double ny, double nz, double* out,
                       cudaStream_t st) {
    const size_t smem = (size_t)M.tables_bytes;
    if (set_smem(k_local_dE<R>, smem)) return SGB_ERR_CUDA;
    k_local_dE<R><<<1, 32, smem, st>>>(M, S, site, (R)nx, (R)ny, (R)nz, out);
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

template <class R>
int mc_launch_sweeps_ewald(const Model<R>& M, R* S, const McArgs& A, const EwaldDev& E, double* F, double* partials,
                           cudaStream_t st) {
    const size_t smem = (size_t)M.tables_bytes;
    const void* k = A.rnd ? (const void*)k_local_sweeps_ewald<R, true> : (const void*)k_local_sweeps_ewald<R, false>;
    if (A.rnd ? set_smem(k_local_sweeps_ewald<R, true>, smem) : set_smem(k_local_sweeps_ewald<R, false>, smem)) return SGB_ERR_CUDA;
    Model<R> m = M;
    McArgs a = A;
    EwaldDev e = E;
    void* args[] = {&m, &S, &a, &e, &F, &partials};
    return cudaLaunchKernel(k, dim3(1), dim3(256), args, smem, st) == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

#define SGB_MC_INST(R)                                                                                         \
    template int mc_max_blocks<R>(size_t, int*);                                                               \
    template int mc_launch_sweeps<R>(const Model<R>&, R*, Ctrl*, const McArgs&, int, double*, cudaStream_t);   \
    template int mc_launch_local_dE<R>(const Model<R>&, const R*, int, double, double, double, double*, cudaStream_t); \
    template int mc_launch_sweeps_ewald<R>(const Model<R>&, R*, const McArgs&, const EwaldDev&, double*, double*, cudaStream_t);
SGB_MC_INST(float)
SGB_MC_INST(double)
