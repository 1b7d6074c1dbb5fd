// sgb_batch_blk.cu -- cell-block form of the batched implicit midpoint: FP32 replica
// batches of one supercell size, i.e. the trajectories of a batched add_sample!
// (Integrators.jl:379-413 per replica, snapshots CorrelationSampling.jl:1-46).
//
// The tile kernel in sgb_batch.cu hands a CTA 256 consecutive sites of one sublattice, so
// every neighbour of every site lies in another sublattice's plane and each of the ~18
// neighbour reads per site and fixed-point iteration is an L2 round trip. Here a CTA owns
// a block of bx x by x bz whole cells (every atom) of one replica for the launch, and the
// midpoint spins that gradients read are kept, per replica, as [atom][z][y][x] over the
// supercell padded by gw ghost cells on every side (the periodic images of the boundary
// cells, written together with the cells). Each fixed-point iteration, one thread moves
// the block and its gw-cell halo, all atoms, into shared memory with a single 5-D TMA box
// load (cp.async.bulk.tensor, completion on an mbarrier); the neighbour reads are then
// shared-memory loads at a constant offset per bond. The per-site arithmetic, the
// convergence test (per-replica sums, FP64 across warps), the extrapolated first iterate,
// the speculative next-step midpoint spins and the snapshots are those of the tile
// kernel; the two differ only in rounding (the order of the convergence sums and the
// compiler's fused multiply-adds), so their trajectories agree within the tolerance.
#include <cuda.h>
#include "sgb_batch.cuh"
#include "sgb_batch_blk.h"

namespace {
using namespace sgbdev;
using namespace sgbbatch;

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init1(uint64_t* m) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(m)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t* m, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_addr(m)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for the phase with the given parity, for at most the handle's wait limit.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* m, uint32_t parity, const Ctrl* ctrl) {
    uint64_t t0 = 0, lim = 0;
    unsigned int spins = 0;
    while (!mbar_test(m, parity)) {
        if ((++spins & 63u) == 0) {
            const uint64_t t = sgb_globaltimer();
            if (t0 == 0) {
                t0 = t;
                lim = sgb_wait_limit(ctrl);
            } else if (t - t0 > lim) {
                return false;
            }
        }
    }
    return true;
}

// The block and its halo of buffer `map` into shared memory: box (4, HX, HY, HZ, na) at
// padded cell (x0, y0, z0) of replica r.
__device__ __forceinline__ void halo_load(const CUtensorMap* map, float4* dst, uint64_t* bar, unsigned int bytes, int x0,
                                          int y0, int z0, int a0) {
    asm volatile("fence.proxy.async.global;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, %6}], "
        "[%7];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(x0), "r"(y0), "r"(z0), "r"(a0), "r"(smem_addr(bar))
        : "memory");
}

struct BlkSite {
    int x, y, z, a;
};

// Midpoint spin v of cell (cx, cy, cz), atom a of replica r into the padded buffer Hb,
// with every periodic image that falls inside the ghost layers.
__device__ __forceinline__ void store_pad(float4* Hb, const BlkGeom& B, int r, int a, int cx, int cy, int cz, float4 v) {
    const int gw = B.gw;
    int xs[2] = {cx + gw, -1}, ys[2] = {cy + gw, -1}, zs[2] = {cz + gw, -1};
    if (cx < gw) xs[1] = cx + gw + B.L1; else if (cx >= B.L1 - gw) xs[1] = cx + gw - B.L1;
    if (cy < gw) ys[1] = cy + gw + B.L2; else if (cy >= B.L2 - gw) ys[1] = cy + gw - B.L2;
    if (cz < gw) zs[1] = cz + gw + B.L3; else if (cz >= B.L3 - gw) zs[1] = cz + gw - B.L3;
    const size_t base = (size_t)(r * B.na + a) * B.PZ;
#pragma unroll
    for (int k = 0; k < 2; k++) {
        if (zs[k] < 0) continue;
#pragma unroll
        for (int j = 0; j < 2; j++) {
            if (ys[j] < 0) continue;
            const size_t row = ((base + zs[k]) * B.PY + ys[j]) * B.PX;
            Hb[row + xs[0]] = v;
            if (xs[1] >= 0) Hb[row + xs[1]] = v;
        }
    }
}

__device__ __forceinline__ float4 load_pad(const float4* Hb, const BlkGeom& B, int r, int a, int cx, int cy, int cz) {
    const size_t i = ((((size_t)(r * B.na + a) * B.PZ) + cz + B.gw) * B.PY + cy + B.gw) * B.PX + cx + B.gw;
    return Hb[i];
}

template <bool GEN, int G, int NT>
__global__ void __launch_bounds__(NT, 1) k_batch_midpoint_blk(BatchArgs<float> A, MidArgs<float> X, BlkGeom B,
                                                                         const __grid_constant__ BlkMaps maps, float4* Hpad,
                                                                         int nsteps, float dt, float lam, BSnap<float> sn) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    // the TMA destination must start on a 128-byte boundary (the launch reserves the slack)
    unsigned char* smem = smem_raw + ((128u - (smem_addr(smem_raw) & 127u)) & 127u);
    float4* halo = reinterpret_cast<float4*>(smem);
    Tab<float> T = stage_tables<float>(A.M, smem + B.halo_bytes);
    int* dlt = reinterpret_cast<int*>(smem + B.halo_bytes + A.M.tables_bytes);   // [nb] halo offset of each bond row
    __shared__ uint64_t bar;
    __shared__ float s_kap[SGB_MAX_SUBLAT];
    __shared__ float s_h[3 * SGB_MAX_SUBLAT];
    __shared__ int4 s_blk[SGB_BLK_MAXB];          // (replica, x0, y0, z0) of each block of this CTA
    __shared__ float wsum[NT / 32];
    __shared__ unsigned long long conv_mask;
    const int tid = threadIdx.x;
    const int na = A.M.na, NS = A.NS;
    const bool leader = (blockIdx.x == 0 && tid == 0);
    const size_t pstride = (size_t)B.PX * B.PY * B.PZ * na * X.nrep;   // float4 elements of one padded buffer
    const int nblk = (int)blockIdx.x < B.nblk ? min(SGB_BLK_MAXB, (B.nblk - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x) : 0;
    const int nsb = na << (B.lbx + B.lby + B.lbz);
    for (int q = tid; q < na; q += blockDim.x) {
        s_kap[q] = A.kap[q];
        s_h[q] = A.h ? A.h[q] : 0.f;
        s_h[na + q] = A.h ? A.h[na + q] : 0.f;
        s_h[2 * na + q] = A.h ? A.h[2 * na + q] : 0.f;
    }
    for (int b = tid; b < A.M.nb; b += blockDim.x) {
        // bond row b of sublattice a: neighbour (cell + n, atom j) sits at this fixed offset
        // from the site in the [atom][z][y][x] halo
        int a = 0;
        while (T.boff[a + 1] <= b) a++;
        const int pk = T.bonds[b].pk;
        const int n0 = (int)(pk & 0xff) - 128, n1 = (int)((pk >> 8) & 0xff) - 128, n2 = (int)((pk >> 16) & 0xff) - 128;
        const int j = (int)((unsigned)pk >> 24);
        dlt[b] = (((j - a) * B.HZ + n2) * B.HY + n1) * B.HX + n0;
    }
    if (tid < nblk) {
        const int blk = blockIdx.x + tid * gridDim.x;
        const int r = blk / (B.nbx * B.nby * B.nbz), q = blk % (B.nbx * B.nby * B.nbz);
        s_blk[tid] = make_int4(r, (q % B.nbx) << B.lbx, ((q / B.nbx) % B.nby) << B.lby, (q / (B.nbx * B.nby)) << B.lbz);
    }
    if (tid == 0) mbar_init1(&bar);
    __syncthreads();
    const int mx = (1 << B.lbx) - 1, my = (1 << B.lby) - 1, mz = (1 << B.lbz) - 1;
    auto site_of = [&](int i) {
        BlkSite c;
        c.x = i & mx;
        c.y = (i >> B.lbx) & my;
        c.z = (i >> (B.lbx + B.lby)) & mz;
        c.a = i >> (B.lbx + B.lby + B.lbz);
        return c;
    };
    int cur = 0;
    uint32_t phase = 0;
    // first midpoint spins normalize((S + S)/2) and the first snapshot
    for (int k = 0; k < nblk; k++) {
        const int4 bk = s_blk[k];
        const int off = bk.x * B.nsr;
        for (int i = tid; i < nsb; i += blockDim.x) {
            const BlkSite c = site_of(i);
            const int cx = bk.y + c.x, cy = bk.z + c.y, cz = bk.w + c.z;
            const int s = cx + B.L1 * (cy + B.L2 * (cz + B.L3 * c.a)), g = off + s;
            const float sx = A.S[g], sy = A.S[NS + g], sz = A.S[2 * NS + g];
            float hx = (sx + sx) / 2, hy = (sy + sy) / 2, hz = (sz + sz) / 2;
            normalize_dip<float>(hx, hy, hz, s_kap[c.a]);
            store_pad(Hpad, B, bk.x, c.a, cx, cy, cz, make_float4(hx, hy, hz, 0.f));
            if (sn.enabled) snap_write<float>(sn, bk.x, sn.t0, s, B.nsr, sx, sy, sz);
        }
    }
    if (leader) {
        for (int q = 0; q < 3 * X.nrep; q++) X.racc[q] = 0.0;
    }
    if (!sgb_grid_barrier(A.ctrl, gridDim.x)) return;
    long long itg = 0;
    int done = 0;
    for (int step = 0; step < nsteps; ++step) {
        unsigned actm = (1u << nblk) - 1u;   // bit k: block k's replica is still iterating
        if (step == 0 || X.ord == 0) {
            for (int k = 0; k < nblk; k++) {
                const int4 bk = s_blk[k];
                const int off = bk.x * B.nsr;
                for (int i = tid; i < nsb; i += blockDim.x) {
                    const BlkSite c = site_of(i);
                    const int g = off + (bk.y + c.x) + B.L1 * ((bk.z + c.y) + B.L2 * ((bk.w + c.z) + B.L3 * c.a));
                    PV<float>::st(X.Sp, NS, g, A.S[g], A.S[NS + g], A.S[2 * NS + g]);
                }
            }
        }
        const int ord = min(X.ord, step + 1);
        bool all_done = false;
        for (int it = 0; it < X.max_iters; ++it) {
            const int nxt = (cur + 1) % 3, nst = (cur + 2) % 3;
            float4* Hn = Hpad + (size_t)nxt * pstride;
            float4* Hs = Hpad + (size_t)nst * pstride;
            const int slot = (int)(itg % 3);
            for (int k = 0; k < nblk; k++) {
                const int4 bk = s_blk[k];
                const bool on = (actm >> k) & 1u;
                const int off = bk.x * B.nsr;
                if (on) {
                    if (tid == 0)
                        halo_load(&maps.m[cur], halo, &bar, B.tx_bytes, bk.y, bk.z, bk.w, bk.x * na);
                    const bool ok = mbar_wait_bounded(&bar, phase, A.ctrl);
                    phase ^= 1u;
                    if (__syncthreads_or(!ok)) {
                        // a halo copy did not arrive in time: record it, give the copy a second
                        // bounded wait so that it is not in flight when the CTA exits, and leave
                        if (tid == 0) {
                            sgb_set_status(A.ctrl, SGB_ERR_TIMEOUT);
                            mbar_wait_bounded(&bar, phase ^ 1u, A.ctrl);
                        }
                        return;
                    }
                }
                float acc = 0.f;   // per-thread and warp sums in FP32; block and grid sums in FP64
                for (int i = tid; i < nsb; i += blockDim.x) {
                    const BlkSite c = site_of(i);
                    const int cx = bk.y + c.x, cy = bk.z + c.y, cz = bk.w + c.z;
                    const int g = off + cx + B.L1 * (cy + B.L2 * (cz + B.L3 * c.a));
                    if (!on) {
                        // converged replica: carry its next-step midpoint spins forward
                        store_pad(Hs, B, bk.x, c.a, cx, cy, cz, load_pad(Hn, B, bk.x, c.a, cx, cy, cz));
                        continue;
                    }
                    const int a = c.a;
                    const float kap = s_kap[a];
                    const int hi = ((a * B.HZ + c.z + B.gw) * B.HY + c.y + B.gw) * B.HX + c.x + B.gw;
                    const float sx = A.S[g], sy = A.S[NS + g], sz = A.S[2 * NS + g];
                    float qx, qy, qz;
                    PV<float>::ld(X.Sp, NS, g, qx, qy, qz);
                    const float4 hv = halo[hi];
                    const float hx = hv.x, hy = hv.y, hz = hv.z;
                    const int* dl = dlt + T.boff[a];
                    float gx, gy, gz, dx, dy, dz;
                    grad_nbi_ld<float, GEN, G>(
                        A.M, T, a, [hi, dl](int b) { return hi + dl[b]; },
                        [halo](int j, float& x, float& y, float& z) {
                            const float4 v = halo[j];
                            x = v.x; y = v.y; z = v.z;
                        },
                        s_h[a], s_h[na + a], s_h[2 * na + a], hx, hy, hz, gx, gy, gz);
                    rhs_dipole<float>(hx, hy, hz, 0.f, 0.f, 0.f, gx, gy, gz, dt, lam, dx, dy, dz);
                    const float nx = sx + dx, ny = sy + dy, nz = sz + dz;
                    const float ex = qx - nx, ey = qy - ny, ez = qz - nz;
                    acc += ex * ex + ey * ey + ez * ez;
                    PV<float>::st(X.Sp, NS, g, nx, ny, nz);
                    float mxv = (sx + nx) / 2, myv = (sy + ny) / 2, mzv = (sz + nz) / 2;
                    normalize_dip<float>(mxv, myv, mzv, kap);
                    store_pad(Hn, B, bk.x, a, cx, cy, cz, make_float4(mxv, myv, mzv, 0.f));
                    if (X.ord == 0 || X.accept0 || it > 0) {
                        float cx_ = nx, cy_ = ny, cz_ = nz;
                        normalize_dip<float>(cx_, cy_, cz_, kap);
                        float px = cx_, py = cy_, pz = cz_;
                        if (ord == 1) {
                            px = 2 * cx_ - sx; py = 2 * cy_ - sy; pz = 2 * cz_ - sz;
                        } else if (ord >= 2) {
                            float ux, uy, uz;
                            PV<float>::ld(X.H1, NS, g, ux, uy, uz);
                            if (ord == 2) {
                                px = 3 * (cx_ - sx) + ux; py = 3 * (cy_ - sy) + uy; pz = 3 * (cz_ - sz) + uz;
                            } else {
                                float vx, vy, vz;
                                PV<float>::ld(X.H2, NS, g, vx, vy, vz);
                                if (ord == 3) {
                                    px = 4 * (cx_ + ux) - 6 * sx - vx; py = 4 * (cy_ + uy) - 6 * sy - vy;
                                    pz = 4 * (cz_ + uz) - 6 * sz - vz;
                                } else {
                                    float wx0, wy0, wz0;
                                    PV<float>::ld(X.H3, NS, g, wx0, wy0, wz0);
                                    px = 5 * (cx_ - vx) + 10 * (ux - sx) + wx0;
                                    py = 5 * (cy_ - vy) + 10 * (uy - sy) + wy0;
                                    pz = 5 * (cz_ - vz) + 10 * (uz - sz) + wz0;
                                }
                            }
                        }
                        if (ord > 0) PV<float>::st(X.P1, NS, g, px, py, pz);
                        float wx = (cx_ + px) / 2, wy = (cy_ + py) / 2, wz = (cz_ + pz) / 2;
                        normalize_dip<float>(wx, wy, wz, kap);
                        store_pad(Hs, B, bk.x, a, cx, cy, cz, make_float4(wx, wy, wz, 0.f));
                    }
                }
                if (on) {
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
                    if ((tid & 31) == 0) wsum[tid >> 5] = acc;
                }
                __syncthreads();   // halo reads and warp partials done before the next block's copy
                if (on && tid == 0) {
                    double t = 0;
                    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += (double)wsum[w];
                    atomicAdd(&X.racc[slot * X.nrep + bk.x], t);
                }
            }
            if (leader) {
                for (int q = 0; q < X.nrep; q++) X.racc[((slot + 1) % 3) * X.nrep + q] = 0.0;
                A.ctrl->iters += 1;
            }
            if (!sgb_grid_barrier(A.ctrl, gridDim.x)) return;
            itg++;
            if (tid == 0) {
                unsigned long long m = 0;
                if (X.ord == 0 || X.accept0 || it > 0)
                    for (int q = 0; q < X.nrep; q++)
                        if (X.racc[slot * X.nrep + q] <= X.atol2) m |= 1ull << q;
                conv_mask = m;
            }
            __syncthreads();
            const unsigned long long mask = conv_mask;
            all_done = (X.nrep == 64) ? (mask == ~0ull) : (mask == ((1ull << X.nrep) - 1));
            for (int k = 0; k < nblk; k++) {
                const int4 bk = s_blk[k];
                if (!(((actm >> k) & 1u) && ((mask >> bk.x) & 1ull))) continue;
                actm &= ~(1u << k);
                const int off = bk.x * B.nsr;
                for (int i = tid; i < nsb; i += blockDim.x) {
                    const BlkSite c = site_of(i);
                    const int g = off + (bk.y + c.x) + B.L1 * ((bk.z + c.y) + B.L2 * ((bk.w + c.z) + B.L3 * c.a));
                    // the accepted state normalize(S''), from the last iterate
                    float x, y, z;
                    PV<float>::ld(X.Sp, NS, g, x, y, z);
                    normalize_dip<float>(x, y, z, s_kap[c.a]);
                    if (X.ord > 0) {
                        if (X.ord >= 4) {
                            float hx, hy, hz;
                            PV<float>::ld(X.H2, NS, g, hx, hy, hz);
                            PV<float>::st(X.H3, NS, g, hx, hy, hz);
                        }
                        if (X.ord >= 3) {
                            float hx, hy, hz;
                            PV<float>::ld(X.H1, NS, g, hx, hy, hz);
                            PV<float>::st(X.H2, NS, g, hx, hy, hz);
                        }
                        if (X.ord >= 2) PV<float>::st(X.H1, NS, g, A.S[g], A.S[NS + g], A.S[2 * NS + g]);
                        float px, py, pz;
                        PV<float>::ld(X.P1, NS, g, px, py, pz);
                        PV<float>::st(X.Sp, NS, g, px, py, pz);
                    }
                    A.S[g] = x; A.S[NS + g] = y; A.S[2 * NS + g] = z;
                }
            }
            if (all_done) {
                cur = nst;
                break;
            }
            cur = nxt;
        }
        if (!all_done) {
            if (leader) sgb_set_status(A.ctrl, SGB_ERR_NOCONVERGE);
            break;
        }
        done = step + 1;
        if (sn.enabled && (done % sn.measperiod) == 0) {
            for (int k = 0; k < nblk; k++) {
                const int4 bk = s_blk[k];
                const int off = bk.x * B.nsr;
                for (int i = tid; i < nsb; i += blockDim.x) {
                    const BlkSite c = site_of(i);
                    const int s = (bk.y + c.x) + B.L1 * ((bk.z + c.y) + B.L2 * ((bk.w + c.z) + B.L3 * c.a));
                    const int g = off + s;
                    snap_write<float>(sn, bk.x, sn.t0 + done / sn.measperiod, s, B.nsr, A.S[g], A.S[NS + g], A.S[2 * NS + g]);
                }
            }
        }
    }
    if (leader) A.ctrl->steps_done = done;
}

template <bool GEN>
void* blk_kernel(int nt) {
    switch (nt) {
        case 256: return (void*)k_batch_midpoint_blk<GEN, 6, 256>;
        case 512: return (void*)k_batch_midpoint_blk<GEN, 6, 512>;
        case 1024: return (void*)k_batch_midpoint_blk<GEN, 6, 1024>;
    }
    return nullptr;
}

// bonds are gathered 6 at a time (G = 6) in every variant
void* pick(bool gen, int G, int nt) {
    if (G != 6) return nullptr;
    return gen ? blk_kernel<true>(nt) : blk_kernel<false>(nt);
}

}  // namespace

int blk_occupancy(bool gen, int G, int nt, size_t smem, int* bps) {
    const void* k = pick(gen, G, nt);
    if (!k) return SGB_ERR_ARG;
    if (smem > 48 * 1024 && cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return SGB_ERR_CUDA;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, k, nt, smem) == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

int blk_launch(bool gen, int G, int nt, int grid, size_t smem, const BatchArgs<float>& A, const MidArgs<float>& X,
               const BlkGeom& B, const BlkMaps& maps, float* Hpad, int nsteps, float dt, float lam,
               const BSnap<float>& sn, cudaStream_t st) {
    const void* k = pick(gen, G, nt);
    if (!k) return SGB_ERR_ARG;
    if (smem > 48 * 1024 && cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return SGB_ERR_CUDA;
    BatchArgs<float> a = A;
    MidArgs<float> x = X;
    BlkGeom b = B;
    float4* hp = reinterpret_cast<float4*>(Hpad);
    BSnap<float> s = sn;
    void* args[] = {&a, &x, &b, const_cast<BlkMaps*>(&maps), &hp, &nsteps, &dt, &lam, &s};
    return cudaLaunchCooperativeKernel(k, dim3(grid), dim3(nt), args, smem, st) == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

// The 5-D tensor map of one padded buffer: (float4 component, x, y, z, replica*na + atom),
// box (4, HX, HY, HZ, na).
int blk_encode_map(CUtensorMap* out, float* base, const BlkGeom& B, int nrep) {
    typedef CUresult (*EncodeFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*, const cuuint64_t*,
                                 const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                 CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    static EncodeFn encode = nullptr;
    if (!encode) {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !fn)
            return SGB_ERR_CUDA;
        encode = reinterpret_cast<EncodeFn>(fn);
    }
    const cuuint64_t dims[5] = {4, (cuuint64_t)B.PX, (cuuint64_t)B.PY, (cuuint64_t)B.PZ, (cuuint64_t)B.na * nrep};
    const cuuint64_t strides[4] = {16, (cuuint64_t)16 * B.PX, (cuuint64_t)16 * B.PX * B.PY,
                                   (cuuint64_t)16 * B.PX * B.PY * B.PZ};
    const cuuint32_t box[5] = {4, (cuuint32_t)B.HX, (cuuint32_t)B.HY, (cuuint32_t)B.HZ, (cuuint32_t)B.na};
    const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
    CUresult r = encode(out, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 5, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? SGB_OK : SGB_ERR_ARG;
}
