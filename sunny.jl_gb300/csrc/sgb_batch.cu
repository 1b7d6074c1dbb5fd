// sgb_batch.cu -- replica batches: many independent dipole-mode systems (possibly of
// different sizes) that share their couplings, advanced together by persistent kernels.
//
// Reference semantics:
//   Langevin Heun per replica   src/Integrators.jl:313-332
//   energy per replica           src/System/Interactions.jl:401-508
//   replica_exchange!           src/MonteCarlo/ParallelTempering.jl:40-73
//   step_ensemble!              src/MonteCarlo/ParallelTempering.jl:80-95
//   midpoint per replica        src/Integrators.jl:379-413 (for batched add_sample!)
//
// Design: the replicas' states are concatenated in L2-resident SoA arrays and cut into
// tiles of up to SGB_TILE (288) sites of one replica. A persistent cooperative grid walks its tiles
// between bounded grid barriers, so one barrier serves every replica and the latency of
// a single small system is amortised over the batch. Per-replica reductions (energies,
// midpoint convergence sums) are formed per tile in FP64. Parallel tempering keeps a
// device-side ladder (replica at each temperature position) per group of equal-size
// replicas, swaps temperatures on device, and step_ensemble! replays one captured CUDA
// graph per exchange round.
#include <algorithm>
#include <array>
#include <cstddef>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <type_traits>
#include <vector>
#include "sgb_device.cuh"
#include "sgb_batch.cuh"
#include "sgb_batch_blk.h"
#include "sgb_tables.h"
#include "sgb_handles.h"
#include "sgb_corr.h"

namespace {
using namespace sgbdev;
using namespace sgbbatch;

struct TileCtx {
    int r, s, off;
    int4 d;
    SiteIdx ix;
};

__device__ __forceinline__ TileCtx tile_ctx(const int4* tiles, const int4* rd, const int* roff, const int* pc, int t) {
    TileCtx c;
    int4 tl = tiles[t];
    c.r = tl.x;
    c.s = tl.y + threadIdx.x;
    c.d = rd[c.r];
    c.off = roff[c.r];
    const int p = pc[c.off + c.s];
    c.ix.c1 = p & 0xff;
    c.ix.c2 = (p >> 8) & 0xff;
    c.ix.c3 = (p >> 16) & 0xff;
    c.ix.a = (int)((unsigned)p >> 24);
    return c;
}

__device__ __forceinline__ bool tile_has(const int4* tiles, int t) { return (int)threadIdx.x < tiles[t].z; }

// Per-tile context from the two-int4 descriptor (one 32-byte load, no coordinate math).
struct TileD {
    int r, s, cnt, a, off, nsr, nbo;
};
__device__ __forceinline__ TileD tile_d(const int4* td, const int* pc, int t) {
    int4 u = td[2 * t], v = td[2 * t + 1];
    TileD c;
    c.r = u.x; c.s = u.y + threadIdx.x; c.cnt = u.z; c.a = u.w;
    c.off = v.x; c.nsr = v.y; c.nbo = v.z;
    if (c.a < 0 && (int)threadIdx.x < c.cnt) c.a = (int)((unsigned)pc[c.off + c.s] >> 24);
    return c;
}

template <class R>
__device__ __forceinline__ void site_field(const BatchArgs<R>& A, int a, R& hx, R& hy, R& hz) {
    if (A.h) { hx = A.h[a]; hy = A.h[A.M.na + a]; hz = A.h[2 * A.M.na + a]; }
    else { hx = 0; hy = 0; hz = 0; }
}

template <class R>
__device__ __forceinline__ void batch_noise(uint64_t seed, int r, uint64_t step, int s, R scale, R& x, R& y, R& z) {
    if (scale == (R)0) { x = 0; y = 0; z = 0; return; }
    R g4[4];
    sgb_normals4<R>(seed, (uint32_t)r, step, (uint32_t)s, 0u, g4);
    x = g4[0] * scale; y = g4[1] * scale; z = g4[2] * scale;
}

// Heun over every replica (Integrators.jl:313-332); each replica uses its own kT. MB: CTAs
// per SM the registers are budgeted for (the launch shape the tuner picks).
template <class R, bool GEN, int MB>
__global__ void __launch_bounds__(SGB_TILE, MB) k_batch_heun(BatchArgs<R> A, const R* kTR, int nsteps, R dt,
                                                            R lam, uint64_t seed, unsigned long long* counters) {
    extern __shared__ __align__(16) unsigned char smem[];
    Tab<R> T = stage_tables<R>(A.M, smem);
    const R two_dt_lam = 2 * dt * lam;   // noise variance per unit kT (fill_noise!, Integrators.jl:288-298)
    const uint64_t step0 = *((volatile unsigned long long*)counters);
    const int NS = A.NS;
    for (int step = 0; step < nsteps; ++step) {
        for (int t = blockIdx.x; t < A.ntiles; t += gridDim.x) {
            TileD c = tile_d(A.td, A.pc, t);
            if ((int)threadIdx.x >= c.cnt) continue;
            const R* X = A.S + c.off;
            const R* Y = A.S + NS + c.off;
            const R* Z = A.S + 2 * NS + c.off;
            R sx = X[c.s], sy = Y[c.s], sz = Z[c.s];
            const R kt = kTR[c.r];
            R scale = (lam == (R)0 || kt == (R)0) ? (R)0 : sgb_sqrt<R>(two_dt_lam * kt);
            R xx, xy, xz;
            batch_noise<R>(seed, c.r, step0 + step, c.s, scale, xx, xy, xz);
            R hx, hy, hz, gx, gy, gz, d0, d1, d2;
            site_field(A, c.a, hx, hy, hz);
            grad_table<R, GEN>(A.M, T, c.a, c.s, A.nbr + c.nbo, c.nsr, hx, hy, hz, sx, sy, sz, X, Y, Z, gx, gy, gz);
            rhs_dipole<R>(sx, sy, sz, xx, xy, xz, gx, gy, gz, dt, lam, d0, d1, d2);
            const int g = c.off + c.s;
            A.D1[g] = d0; A.D1[NS + g] = d1; A.D1[2 * NS + g] = d2;
            R px = sx + d0, py = sy + d1, pz = sz + d2;
            normalize_dip<R>(px, py, pz, A.kap[c.a]);
            A.P[g] = px; A.P[NS + g] = py; A.P[2 * NS + g] = pz;
        }
        if (!sgb_grid_barrier(A.ctrl, gridDim.x)) return;
        for (int t = blockIdx.x; t < A.ntiles; t += gridDim.x) {
            TileD c = tile_d(A.td, A.pc, t);
            if ((int)threadIdx.x >= c.cnt) continue;
            const int g = c.off + c.s;
            const R* X = A.P + c.off;
            const R* Y = A.P + NS + c.off;
            const R* Z = A.P + 2 * NS + c.off;
            R px = X[c.s], py = Y[c.s], pz = Z[c.s];
            const R kt = kTR[c.r];
            R scale = (lam == (R)0 || kt == (R)0) ? (R)0 : sgb_sqrt<R>(two_dt_lam * kt);
            R xx, xy, xz;
            batch_noise<R>(seed, c.r, step0 + step, c.s, scale, xx, xy, xz);
            R hx, hy, hz, gx, gy, gz, e0, e1, e2;
            site_field(A, c.a, hx, hy, hz);
            grad_table<R, GEN>(A.M, T, c.a, c.s, A.nbr + c.nbo, c.nsr, hx, hy, hz, px, py, pz, X, Y, Z, gx, gy, gz);
            rhs_dipole<R>(px, py, pz, xx, xy, xz, gx, gy, gz, dt, lam, e0, e1, e2);
            R nx = A.S[g] + (A.D1[g] + e0) / 2;
            R ny = A.S[NS + g] + (A.D1[NS + g] + e1) / 2;
            R nz = A.S[2 * NS + g] + (A.D1[2 * NS + g] + e2) / 2;
            normalize_dip<R>(nx, ny, nz, A.kap[c.a]);
            A.S[g] = nx; A.S[NS + g] = ny; A.S[2 * NS + g] = nz;
        }
        if (step + 1 < nsteps) {
            if (!sgb_grid_barrier(A.ctrl, gridDim.x)) return;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *counters = step0 + nsteps;
}

// FP64 energy of every tile (one CTA per tile); k_batch_reduce sums a replica's tiles in
// order, so energies are deterministic.
template <class R>
__global__ void __launch_bounds__(SGB_TILE) k_batch_energy(BatchArgs<R> A, double* Epart) {
    extern __shared__ __align__(16) unsigned char smem[];
    Tab<R> T = stage_tables<R>(A.M, smem);
    const int t = blockIdx.x;
    double E = 0;
    if (tile_has(A.tiles, t)) {
        TileCtx c = tile_ctx(A.tiles, A.rd, A.roff, A.pc, t);
        const int NS = A.NS;
        const R* X = A.S + c.off;
        const R* Y = A.S + NS + c.off;
        const R* Z = A.S + 2 * NS + c.off;
        double sx = X[c.s], sy = Y[c.s], sz = Z[c.s];
        const int a = c.ix.a;
        if (A.h) E += (double)A.h[a] * sx + (double)A.h[A.M.na + a] * sy + (double)A.h[2 * A.M.na + a] * sz;
        if (A.M.dipole_mode) {
            double cc[28];
            for (int q = 0; q < 28; q++) cc[q] = (double)T.stev[28 * a + q];
            double gx = 0, gy = 0, gz = 0;
            E += classical_aniso<double>(cc, T.kmax[a], sx, sy, sz, gx, gy, gz);
        }
        for (int b = T.boff[a]; b < T.boff[a + 1]; b++) {
            const DBond<R>& B = T.bonds[b];
            if (!B.fwd) continue;
            int x1 = sgb_wrap_any(c.ix.c1 + B.n[0], c.d.x);
            int x2 = sgb_wrap_any(c.ix.c2 + B.n[1], c.d.y);
            int x3 = sgb_wrap_any(c.ix.c3 + B.n[2], c.d.z);
            int js = x1 + c.d.x * (x2 + c.d.y * (x3 + c.d.z * B.j));
            double tx = X[js], ty = Y[js], tz = Z[js];
            E += (double)B.scalar;
            if (B.jkind == 0) E += (double)B.J[0] * (sx * tx + sy * ty + sz * tz);
            else {
                double jx = (double)B.J[0] * tx + (double)B.J[3] * ty + (double)B.J[6] * tz;
                double jy = (double)B.J[1] * tx + (double)B.J[4] * ty + (double)B.J[7] * tz;
                double jz = (double)B.J[2] * tx + (double)B.J[5] * ty + (double)B.J[8] * tz;
                E += sx * jx + sy * jy + sz * jz;
            }
            if (A.M.dipole_mode && B.bqkind != 0) {
                double Qi[5], Qj[5], acc = 0;
                quad5<double>(sx, sy, sz, Qi);
                quad5<double>(tx, ty, tz, Qj);
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
    if (threadIdx.x == 0) Epart[t] = e;
}

__global__ void k_batch_reduce(const double* Epart, const int* tfirst, const int* tcount, double* E) {
    const int r = blockIdx.x;
    double v = 0;
    for (int k = threadIdx.x; k < tcount[r]; k += blockDim.x) v += Epart[tfirst[r] + k];
    double t = sgb_block_sum(v);
    if (threadIdx.x == 0) E[r] = t;
}

// replica_exchange! (ParallelTempering.jl:40-73) on device. Positions are ladder slots
// (group-major); ladder[p] is the replica currently at slot p, which holds kT[ladder[p]].
// exch_start <= 0 takes the round from counters[1] (step_ensemble! alternation).
__global__ void k_batch_exchange(int ngroups, const int* gstart, const int* gcount, int* ladder, double* kT,
                                 void* kTR, int rbytes, const double* E, int exch_start, uint64_t seed,
                                 uint64_t round_arg, unsigned long long* counters, const double* uniforms,
                                 long long* n_accept) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    uint64_t round = round_arg;
    int start = exch_start;
    if (exch_start <= 0) {
        round = counters[1];
        long long i = (long long)round + 1;   // 1-based round of step_ensemble!
        start = (int)(i % 2) + 1;
        counters[1] = round + 1;
    }
    for (int g = 0; g < ngroups; g++) {
        const int p0 = gstart[g], n = gcount[g];
        for (int rank = start - 1; rank + 1 < n; rank += 2) {
            const int p = p0 + rank;
            const int r1 = ladder[p], r2 = ladder[p + 1];
            const double E1 = E[r1], E2 = E[r2];
            const double kT1 = kT[r1], kT2 = kT[r2];
            const double dS1 = E1 / kT1 - E2 / kT1;
            const double dS2 = E2 / kT2 - E1 / kT2;
            const double lnP = dS1 + dS2;
            double u;
            if (uniforms) u = uniforms[p];
            else {
                Philox4 c;
                c.x = (uint32_t)p; c.y = (uint32_t)round; c.z = (uint32_t)(round >> 32); c.w = 0x7E4Cu;
                Philox4 o = sgb_philox(c, (uint32_t)seed, (uint32_t)(seed >> 32));
                u = ((double)o.x + 0.5) * 2.3283064365386963e-10;
            }
            if (lnP >= 0 || u < exp(lnP)) {
                kT[r1] = kT2;
                kT[r2] = kT1;
                if (rbytes == 4) { ((float*)kTR)[r1] = (float)kT2; ((float*)kTR)[r2] = (float)kT1; }
                else { ((double*)kTR)[r1] = kT2; ((double*)kTR)[r2] = kT1; }
                ladder[p] = r2;
                ladder[p + 1] = r1;
                n_accept[p] += 1;
            }
        }
    }
}

template <class R>
__global__ void k_batch_noise(int ns, int rep, uint64_t seed, uint64_t step, double* out) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += gridDim.x * blockDim.x) {
        R g4[4];
        sgb_normals4<R>(seed, (uint32_t)rep, step, (uint32_t)s, 0u, g4);
        out[3 * s] = (double)g4[0]; out[3 * s + 1] = (double)g4[1]; out[3 * s + 2] = (double)g4[2];
    }
}

// ---- batched implicit midpoint with snapshots (batched add_sample!) ---------------------

// Batched implicit midpoint (Integrators.jl:379-413 per replica) recording snapshots.
// Each CTA owns at most SGB_MAXT tiles for the whole launch. Their descriptors, the
// sublattice of every site, kappa and the Zeeman field per sublattice, and (IDX != 0)
// the neighbour index of every bond of every site are copied to shared memory once, so
// the iteration loop issues no dependent index loads: the only global loads left are the
// site's own spins and its neighbours' midpoint spins, fetched G bonds at a time.
// IDX 2 keeps indices as uint16 (replicas of at most 65,536 sites), IDX 4 as int32,
// IDX 0 reads them from the global table. G is the number of bonds gathered together.
template <class R, bool GEN, int IDX, int G, int MB>
__global__ void __launch_bounds__(SGB_TILE, MB) k_batch_midpoint(BatchArgs<R> A, MidArgs<R> X, int nsteps, R dt,
                                                                R lam, BSnap<R> sn, int kb) {
    using IT = typename std::conditional<IDX == 2, unsigned short, int>::type;
    extern __shared__ __align__(16) unsigned char smem[];
    Tab<R> T = stage_tables<R>(A.M, smem);
    IT* sidx = reinterpret_cast<IT*>(smem + A.M.tables_bytes);   // [tile][bond][SGB_TILE]
    __shared__ R wpart[SGB_MAXT][SGB_TILE / 32];   // per-warp convergence partials of each tile
    __shared__ unsigned long long conv_mask;   // bit q: replica q met the tolerance this iteration
    __shared__ int4 st_a[SGB_MAXT];            // (replica, first site, count, replica offset)
    __shared__ int2 st_b[SGB_MAXT];            // (replica sites, neighbour-table offset)
    __shared__ unsigned char st_atom[SGB_MAXT][SGB_TILE];
    __shared__ R s_kap[SGB_MAX_SUBLAT];
    __shared__ R s_h[3 * SGB_MAX_SUBLAT];
    const int NS = A.NS, na = A.M.na;
    const int tid = threadIdx.x;
    const bool leader = (blockIdx.x == 0 && tid == 0);
    const int ntb = (int)blockIdx.x < A.ntiles
                        ? min(SGB_MAXT, (A.ntiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x)
                        : 0;
    for (int q = tid; q < na; q += blockDim.x) {
        s_kap[q] = A.kap[q];
        s_h[q] = A.h ? A.h[q] : (R)0;
        s_h[na + q] = A.h ? A.h[na + q] : (R)0;
        s_h[2 * na + q] = A.h ? A.h[2 * na + q] : (R)0;
    }
    for (int k = 0; k < ntb; k++) {
        const int t = blockIdx.x + k * gridDim.x;
        TileD c = tile_d(A.td, A.pc, t);
        if (tid == 0) {
            st_a[k] = make_int4(c.r, c.s, c.cnt, c.off);
            st_b[k] = make_int2(c.nsr, c.nbo);
        }
        if (tid < c.cnt) {
            st_atom[k][tid] = (unsigned char)c.a;
            if (IDX != 0) {
                const int nb = T.boff[c.a + 1] - T.boff[c.a];
                for (int b = 0; b < nb; b++)
                    sidx[((size_t)k * kb + b) * SGB_TILE + tid] = (IT)__ldg(A.nbr + c.nbo + (size_t)b * c.nsr + c.s);
            }
        }
    }
    __syncthreads();
    int cur = 0;
    // first midpoint spins normalize((S + S)/2) and the first snapshot
    for (int k = 0; k < ntb; k++) {
        const int4 ti = st_a[k];
        if (tid >= ti.z) continue;
        const int s = ti.y + tid, g = ti.w + s;
        R sx = A.S[g], sy = A.S[NS + g], sz = A.S[2 * NS + g];
        R hx = (sx + sx) / 2, hy = (sy + sy) / 2, hz = (sz + sz) / 2;
        normalize_dip<R>(hx, hy, hz, s_kap[st_atom[k][tid]]);
        MV<R>::st(X.H, NS, g, hx, hy, hz);
        if (sn.enabled) snap_write<R>(sn, ti.x, sn.t0, s, st_b[k].x, sx, sy, sz);
    }
    if (leader) {
        for (int q = 0; q < 3 * X.nrep; q++) X.racc[q] = 0.0;
    }
    if (!sgb_grid_barrier(A.ctrl, gridDim.x)) return;
    long long itg = 0;
    int done = 0;
    // With an extrapolated first iterate (ord > 0) a step is accepted lazily: the first
    // iteration of the next step computes normalize(S'') from the last iterate, which the
    // iterate buffer still holds, stores it as the state and shifts the history, beside its
    // other loads; the iterate comes from the first-iterate buffer. Every replica accepts
    // exactly once per step, so each step after the first starts with all tiles pending.
    const bool lazy = X.ord > 0;
    for (int step = 0; step < nsteps; ++step) {
        unsigned actm = (1u << ntb) - 1u;   // bit k: tile k's replica is still iterating
        // first iterate S' = S; with extrapolation (ord > 0) the converging iteration of the
        // previous step already stored it
        if (step == 0 || X.ord == 0) {
            for (int k = 0; k < ntb; k++) {
                const int4 ti = st_a[k];
                if (tid >= ti.z) continue;
                const int g = ti.w + ti.y + tid;
                PV<R>::st(X.Sp, NS, g, A.S[g], A.S[NS + g], A.S[2 * NS + g]);
            }
        }
        const int ord = min(X.ord, step + 1);   // extrapolation order available for the next step
        bool all_done = false;
        for (int it = 0; it < X.max_iters; ++it) {
            const bool pend = lazy && step > 0 && it == 0;   // accept the previous step here
            const int nxt = (cur + 1) % 3, nst = (cur + 2) % 3;
            const R* Hc = X.H + (size_t)cur * MV<R>::W * NS;
            R* Hn = X.H + (size_t)nxt * MV<R>::W * NS;
            R* Hs = X.H + (size_t)nst * MV<R>::W * NS;
            const int slot = (int)(itg % 3);
            for (int k = 0; k < ntb; k++) {
                const int4 ti = st_a[k];
                const bool on = (actm >> k) & 1u;
                R acc = 0;   // per-site terms in R; the warp sums in R, tile and grid sums in FP64
                if (tid < ti.z) {
                    const int s = ti.y + tid, g = ti.w + s;
                    if (on) {
                        const int a = st_atom[k][tid];
                        const R kap = s_kap[a];
                        R sx, sy, sz, qx, qy, qz, hx, hy, hz;
                        if (pend) {
                            // the previous step's accepted state normalize(S''). This step
                            // (S_n -> S_{n+1}) extrapolates its next first iterate from
                            // S_{n+1}, S_n and the history term K of S_{n-1}, S_{n-2},
                            // S_{n-3}, formed here once: H1 <- S_{n-1}, H2 <- S_{n-2}, K -> H3
                            const R ox = A.S[g], oy = A.S[NS + g], oz = A.S[2 * NS + g];
                            PV<R>::ld(X.Sp, NS, g, sx, sy, sz);
                            PV<R>::ld(X.P1, NS, g, qx, qy, qz);
                            normalize_dip<R>(sx, sy, sz, kap);
                            R ux = 0, uy = 0, uz = 0, vx = 0, vy = 0, vz = 0;   // S_{n-2}, S_{n-3}
                            if (ord >= 3 || X.ord >= 4) PV<R>::ld(X.H1, NS, g, ux, uy, uz);
                            if (ord >= 4) PV<R>::ld(X.H2, NS, g, vx, vy, vz);
                            if (X.ord >= 4) PV<R>::st(X.H2, NS, g, ux, uy, uz);
                            if (X.ord >= 3) PV<R>::st(X.H1, NS, g, ox, oy, oz);
                            if (ord == 2) PV<R>::st(X.H3, NS, g, ox, oy, oz);
                            else if (ord == 3) PV<R>::st(X.H3, NS, g, 4 * ox - ux, 4 * oy - uy, 4 * oz - uz);
                            else if (ord >= 4)
                                PV<R>::st(X.H3, NS, g, 10 * ox - 5 * ux + vx, 10 * oy - 5 * uy + vy, 10 * oz - 5 * uz + vz);
                            A.S[g] = sx; A.S[NS + g] = sy; A.S[2 * NS + g] = sz;
                        } else {
                            sx = A.S[g]; sy = A.S[NS + g]; sz = A.S[2 * NS + g];
                            PV<R>::ld(X.Sp, NS, g, qx, qy, qz);
                        }
                        // own midpoint spin normalize((S + S')/2): stored by the previous
                        // iteration (or step) with exactly this arithmetic
                        MV<R>::ld(Hc, NS, g, hx, hy, hz);
                        const bool prep = X.ord == 0 || X.accept0 || it > 0;
                        R gx, gy, gz, dx, dy, dz;
                        const R* HB = Hc + (size_t)MV<R>::K * ti.w;
                        auto nld = [HB, NS](int j, R& x, R& y, R& z) { MV<R>::ld(HB, NS, j, x, y, z); };
                        if (IDX != 0) {
                            const IT* ip = sidx + (size_t)k * kb * SGB_TILE + tid;
                            grad_nbi_ld<R, GEN, G>(A.M, T, a, [ip](int b) { return (int)ip[b * SGB_TILE]; }, nld,
                                                   s_h[a], s_h[na + a], s_h[2 * na + a], hx, hy, hz, gx, gy, gz);
                        } else {
                            const int* ip = A.nbr + st_b[k].y + s;
                            const int nsr = st_b[k].x;
                            grad_nbi_ld<R, GEN, G>(A.M, T, a, [ip, nsr](int b) { return __ldg(ip + (size_t)b * nsr); },
                                                   nld, s_h[a], s_h[na + a], s_h[2 * na + a], hx, hy, hz, gx, gy, gz);
                        }
                        rhs_dipole<R>(hx, hy, hz, (R)0, (R)0, (R)0, gx, gy, gz, dt, lam, dx, dy, dz);
                        R nx = sx + dx, ny = sy + dy, nz = sz + dz;
                        R ex = qx - nx, ey = qy - ny, ez = qz - nz;
                        acc = ex * ex + ey * ey + ez * ez;
                        PV<R>::st(X.Sp, NS, g, nx, ny, nz);
                        R mx = (sx + nx) / 2, my = (sy + ny) / 2, mz = (sz + nz) / 2;
                        normalize_dip<R>(mx, my, mz, kap);
                        MV<R>::st(Hn, NS, g, mx, my, mz);
                        // With an extrapolated first iterate the step is never accepted at its
                        // first iteration (see the convergence mask below), so the next-step data
                        // are only prepared from the second iteration on.
                        if (prep) {
                        R cx = nx, cy = ny, cz = nz;
                        normalize_dip<R>(cx, cy, cz, kap);
                        // next step's first iterate p and midpoint spin normalize((c + p)/2)
                        R px = cx, py = cy, pz = cz;
                        if (ord == 1) {
                            px = 2 * cx - sx; py = 2 * cy - sy; pz = 2 * cz - sz;
                        } else if (ord >= 2) {
                            // the polynomial of degree ord through c = S_{n+1}, s = S_n and the
                            // ord - 1 states before, at S_{n+2}: p = a c - b s + K
                            const R ca = (R)(ord + 1), sb = (R)(ord == 2 ? 3 : (ord == 3 ? 6 : 10));
                            R kx, ky, kz;
                            PV<R>::ld(X.H3, NS, g, kx, ky, kz);
                            px = ca * cx - sb * sx + kx;
                            py = ca * cy - sb * sy + ky;
                            pz = ca * cz - sb * sz + kz;
                        }
                        if (ord > 0) PV<R>::st(X.P1, NS, g, px, py, pz);
                        R wx = (cx + px) / 2, wy = (cy + py) / 2, wz = (cz + pz) / 2;
                        normalize_dip<R>(wx, wy, wz, kap);
                        MV<R>::st(Hs, NS, g, wx, wy, wz);
                        }
                    } else {
                        // converged replica: carry its next-step midpoint spins forward
                        R x, y, z;
                        MV<R>::ld(Hn, NS, g, x, y, z);
                        MV<R>::st(Hs, NS, g, x, y, z);
                    }
                }
                if (on) {
                    // warp sum in R, kept per warp (no shared-memory FP64 atomics)
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
                    if ((tid & 31) == 0) wpart[k][tid >> 5] = acc;
                }
            }
            __syncthreads();
            // one thread per active tile: the tile's sum of its warps' partials, added in FP64
            // to its replica's grid sum (tiles never straddle replicas)
            if (tid < ntb && ((actm >> tid) & 1u)) {
                double t = 0;
#pragma unroll
                for (int w = 0; w < SGB_TILE / 32; w++) t += (double)wpart[tid][w];
                atomicAdd(&X.racc[slot * X.nrep + (st_a[tid].x - X.r0)], t);
            }
            if (leader) {
                for (int q = 0; q < X.nrep; q++) X.racc[((slot + 1) % 3) * X.nrep + q] = 0.0;
                A.ctrl->iters += 1;
            }
            if (!sgb_grid_barrier(A.ctrl, gridDim.x)) return;
            itg++;
            // one thread per block compares the FP64 sums with the tolerance
            if (tid == 0) {
                unsigned long long m = 0;
                // the convergence test of the reference, Σ|S' - S''|² <= atol²; with an
                // extrapolated first iterate it is applied from the second iteration on
                if (X.ord == 0 || X.accept0 || it > 0)
                    for (int q = 0; q < X.nrep; q++)
                        if (X.racc[slot * X.nrep + q] <= X.atol2) m |= 1ull << q;
                conv_mask = m;
            }
            __syncthreads();
            const unsigned long long mask = conv_mask;
            all_done = (X.nrep == 64) ? (mask == ~0ull) : (mask == ((1ull << X.nrep) - 1));
            for (int k = 0; k < ntb; k++) {
                const int4 ti = st_a[k];
                if (((actm >> k) & 1u) && ((mask >> (ti.x - X.r0)) & 1ull)) {
                    actm &= ~(1u << k);
                    if (!lazy && tid < ti.z) {
                        const int g = ti.w + ti.y + tid;
                        // the accepted state normalize(S''), from the last iterate
                        R x, y, z;
                        PV<R>::ld(X.Sp, NS, g, x, y, z);
                        normalize_dip<R>(x, y, z, s_kap[st_atom[k][tid]]);
                        A.S[g] = x; A.S[NS + g] = y; A.S[2 * NS + g] = z;
                    }
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
            for (int k = 0; k < ntb; k++) {
                const int4 ti = st_a[k];
                if (tid >= ti.z) continue;
                const int s = ti.y + tid, g = ti.w + s;
                R x = A.S[g], y = A.S[NS + g], z = A.S[2 * NS + g];
                if (lazy) {
                    PV<R>::ld(X.Sp, NS, g, x, y, z);
                    normalize_dip<R>(x, y, z, s_kap[st_atom[k][tid]]);
                }
                snap_write<R>(sn, ti.x, sn.t0 + done / sn.measperiod, s, st_b[k].x, x, y, z);
            }
        }
    }
    // the last step's pending acceptance (a failed step has already taken its predecessor's)
    if (lazy && nsteps > 0 && done == nsteps) {
        for (int k = 0; k < ntb; k++) {
            const int4 ti = st_a[k];
            if (tid >= ti.z) continue;
            const int g = ti.w + ti.y + tid;
            R x, y, z;
            PV<R>::ld(X.Sp, NS, g, x, y, z);
            normalize_dip<R>(x, y, z, s_kap[st_atom[k][tid]]);
            A.S[g] = x; A.S[NS + g] = y; A.S[2 * NS + g] = z;
        }
    }
    if (leader) A.ctrl->steps_done = done;
}

// ---- host helpers --------------------------------------------------------------------------

thread_local std::string g_batch_error;

int bfail(sgb_batch* b, int code, const std::string& msg) {
    if (b) b->err = msg;
    g_batch_error = msg;
    return code;
}

#define BCK(call)                                                                                 \
    do {                                                                                          \
        cudaError_t _e = (call);                                                                  \
        if (_e != cudaSuccess) return bfail(b, SGB_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
    } while (0)

int bmalloc(sgb_batch* b, void** p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
    if (e != cudaSuccess) {
        *p = nullptr;
        return bfail(b, SGB_ERR_NOMEM, std::string("device allocation failed: ") + cudaGetErrorString(e));
    }
    return SGB_OK;
}

void bfree(void*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

size_t bsize(const sgb_batch* b) { return b->fp32 ? 4 : 8; }

template <class R>
Model<R>& bmodel(sgb_batch* b);
template <>
Model<float>& bmodel<float>(sgb_batch* b) { return b->mf; }
template <>
Model<double>& bmodel<double>(sgb_batch* b) { return b->md; }

template <class R>
BatchArgs<R> bargs(sgb_batch* b) {
    BatchArgs<R> A;
    A.M = bmodel<R>(b);
    A.tiles = b->tiles;
    A.ntiles = b->ntiles;
    A.rd = b->rd;
    A.roff = b->roff;
    A.pc = b->pc;
    A.nbr = b->nbr;
    A.nbo = b->nbo;
    A.td = b->td;
    A.NS = b->NS;
    A.kap = (const R*)b->kap;
    A.h = b->has_field ? (const R*)b->h : nullptr;
    A.S = (R*)b->S;
    A.P = (R*)b->P;
    A.D1 = (R*)b->D1;
    A.ctrl = b->ctrl;
    return A;
}

template <class K>
int bcoop(sgb_batch* b, K kernel, int grid, size_t smem, void** args) {
    if (smem > 48 * 1024 && cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return bfail(b, SGB_ERR_CUDA, "cudaFuncSetAttribute failed");
    cudaError_t e = cudaLaunchCooperativeKernel((const void*)kernel, dim3(grid), dim3(SGB_TILE), args, smem, b->stream);
    b->launches++;
    if (e != cudaSuccess) return bfail(b, SGB_ERR_CUDA, std::string("cooperative launch: ") + cudaGetErrorString(e));
    return SGB_OK;
}

template <class K>
int bgrid(sgb_batch* b, K kernel, size_t smem, int maxtiles_per_block, int* grid) {
    if (smem > 48 * 1024 && cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return bfail(b, SGB_ERR_CUDA, "cudaFuncSetAttribute failed");
    int bps = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kernel, SGB_TILE, smem) != cudaSuccess)
        return bfail(b, SGB_ERR_CUDA, "occupancy query failed");
    long long cap = (long long)bps * b->nsm;
    long long g = std::min<long long>(cap, b->ntiles);
    if (maxtiles_per_block > 0 && g * maxtiles_per_block < b->ntiles)
        return bfail(b, SGB_ERR_ARG, "replica batch too large for one persistent launch of the midpoint kernel");
    *grid = (int)std::max<long long>(1, g);
    return SGB_OK;
}

int read_status(sgb_batch* b, Ctrl* out) {
    BCK(cudaMemcpyAsync(out, b->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    return SGB_OK;
}

template <class R>
const void* heun_kernel(bool gen, int bps) {
    if (sizeof(R) == 4 && bps >= 4) return gen ? (const void*)k_batch_heun<R, true, 4> : (const void*)k_batch_heun<R, false, 4>;
    if (sizeof(R) == 4 && bps == 3) return gen ? (const void*)k_batch_heun<R, true, 3> : (const void*)k_batch_heun<R, false, 3>;
    return gen ? (const void*)k_batch_heun<R, true, 2> : (const void*)k_batch_heun<R, false, 2>;
}

int heun_fit(sgb_batch* b, const void* k, size_t smem, int* bps) {
    if (smem > 48 * 1024 && cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return SGB_ERR_CUDA;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, k, SGB_TILE, smem) == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

template <class R>
int enqueue_langevin(sgb_batch* b, double dt, double damping, uint64_t seed, int nsteps) {
    BatchArgs<R> A = bargs<R>(b);
    size_t smem = (size_t)b->tables_bytes;
    const R* kTR = reinterpret_cast<const R*>(b->kTR);
    unsigned long long* ctr = b->counters;
    R rdt = (R)dt, rlam = (R)damping;
    void* args[] = {&A, &kTR, &nsteps, &rdt, &rlam, &seed, &ctr};
    const int bps = b->heun_bps > 0 ? b->heun_bps : (sizeof(R) == 4 ? 3 : 2);
    const void* k = heun_kernel<R>(A.M.general != 0, bps);
    int fit = 0;
    if (heun_fit(b, k, smem, &fit) || fit < 1) return bfail(b, SGB_ERR_CUDA, "occupancy query failed");
    const int grid = (int)std::max<long long>(1, std::min<long long>((long long)std::min(bps, fit) * b->nsm, b->ntiles));
    return bcoop(b, k, grid, smem, args);
}

// Times the batched Langevin launch shapes (4, 3 or 2 CTAs per SM in FP32; FP64 has one)
// on 10 steps each, the replicas' states and the step counter saved and restored around
// the runs, and keeps the fastest for these couplings.
template <class R>
int tune_langevin(sgb_batch* b, double dt, double damping, uint64_t seed) {
    if (b->heun_bps > 0) return SGB_OK;
    const int cand[3] = {4, 3, 2};
    if (sizeof(R) == 8) { b->heun_bps = 2; return SGB_OK; }
    const size_t bytes = bsize(b) * 3 * (size_t)b->NS;
    void* save = nullptr;
    if (bmalloc(b, &save, bytes)) return SGB_ERR_NOMEM;
    unsigned long long ctr0 = 0;
    BCK(cudaMemcpyAsync(&ctr0, b->counters, sizeof(ctr0), cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaMemcpyAsync(save, b->S, bytes, cudaMemcpyDeviceToDevice, b->stream));
    int best = -1;
    for (int v = 0; v < 3; v++) {
        b->heun_bps = cand[v];
        int fit = 0;
        if (heun_fit(b, heun_kernel<R>(b->mf.general != 0 || b->md.general != 0, cand[v]), (size_t)b->tables_bytes, &fit) || fit < cand[v]) {
            cudaGetLastError();
            b->heun_ms[v] = 1e30f;
            continue;
        }
        float ms = 0.f;
        bool ok = true;
        for (int rep = 0; rep < 2 && ok; rep++) {   // the first repetition warms up
            ok = cudaMemsetAsync(b->ctrl, 0, sgb_ctrl_clear_bytes(), b->stream) == cudaSuccess &&
                 cudaEventRecord(b->ev[6], b->stream) == cudaSuccess && enqueue_langevin<R>(b, dt, damping, seed, 10) == SGB_OK &&
                 cudaEventRecord(b->ev[7], b->stream) == cudaSuccess && cudaEventSynchronize(b->ev[7]) == cudaSuccess &&
                 cudaEventElapsedTime(&ms, b->ev[6], b->ev[7]) == cudaSuccess &&
                 cudaMemcpyAsync(b->S, save, bytes, cudaMemcpyDeviceToDevice, b->stream) == cudaSuccess &&
                 cudaMemcpyAsync(b->counters, &ctr0, sizeof(ctr0), cudaMemcpyHostToDevice, b->stream) == cudaSuccess;
        }
        Ctrl st;
        if (read_status(b, &st) != SGB_OK || st.status != 0) ok = false;
        b->heun_ms[v] = ok ? ms : 1e30f;
        if (!ok) cudaGetLastError();
        if (ok && (best < 0 || ms < b->heun_ms[best])) best = v;
    }
    cudaStreamSynchronize(b->stream);
    bfree(save);
    BCK(cudaMemsetAsync(b->ctrl, 0, sgb_ctrl_clear_bytes(), b->stream));
    if (best < 0) return bfail(b, SGB_ERR_CUDA, "no batched Langevin launch shape ran");
    b->heun_bps = cand[best];
    return SGB_OK;
}

template <class R>
int enqueue_energy(sgb_batch* b) {
    BatchArgs<R> A = bargs<R>(b);
    size_t smem = (size_t)b->tables_bytes;
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(k_batch_energy<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return bfail(b, SGB_ERR_CUDA, "cudaFuncSetAttribute failed");
    k_batch_energy<R><<<b->ntiles, SGB_TILE, smem, b->stream>>>(A, b->Epart);
    k_batch_reduce<<<b->nrep, SGB_TILE, 0, b->stream>>>(b->Epart, b->tfirst_d, b->tcount_d, b->E);
    b->launches += 2;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? SGB_OK : bfail(b, SGB_ERR_CUDA, std::string("energy launch: ") + cudaGetErrorString(e));
}

int enqueue_exchange(sgb_batch* b, int exch_start, uint64_t seed, uint64_t round, const double* uniforms_dev) {
    k_batch_exchange<<<1, 32, 0, b->stream>>>(b->ngroups, b->gstart, b->gcount, b->ladder, b->kT, b->kTR,
                                              (int)bsize(b), b->E, exch_start, seed, round, b->counters, uniforms_dev,
                                              b->n_accept);
    b->launches++;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? SGB_OK : bfail(b, SGB_ERR_CUDA, std::string("exchange launch: ") + cudaGetErrorString(e));
}

int ensure_bstage(sgb_batch* b, size_t bytes) {
    if (b->stage_cap >= bytes) return SGB_OK;
    if (b->stage) cudaFreeHost(b->stage);
    b->stage = nullptr;
    b->stage_cap = 0;
    if (cudaMallocHost((void**)&b->stage, bytes) != cudaSuccess) return bfail(b, SGB_ERR_NOMEM, "pinned allocation failed");
    b->stage_cap = bytes;
    return SGB_OK;
}

int rebuild_groups(sgb_batch* b) {
    // groups of equal dims, in order of first appearance; each sorted by kT ascending
    std::vector<int> gid(b->nrep, -1);
    std::vector<std::vector<int>> groups;
    for (int r = 0; r < b->nrep; r++) {
        if (gid[r] >= 0) continue;
        groups.push_back({});
        for (int q = r; q < b->nrep; q++)
            if (gid[q] < 0 && b->dims[3 * q] == b->dims[3 * r] && b->dims[3 * q + 1] == b->dims[3 * r + 1] &&
                b->dims[3 * q + 2] == b->dims[3 * r + 2]) {
                gid[q] = (int)groups.size() - 1;
                groups.back().push_back(q);
            }
    }
    b->ladder_h.clear();
    b->gstart_h.clear();
    b->gcount_h.clear();
    for (auto& g : groups) {
        std::stable_sort(g.begin(), g.end(), [&](int x, int y) { return b->kT_h[x] < b->kT_h[y]; });
        b->gstart_h.push_back((int)b->ladder_h.size());
        b->gcount_h.push_back((int)g.size());
        for (int r : g) b->ladder_h.push_back(r);
    }
    b->ngroups = (int)groups.size();
    BCK(cudaMemcpy(b->ladder, b->ladder_h.data(), sizeof(int) * b->nrep, cudaMemcpyHostToDevice));
    BCK(cudaMemcpy(b->gstart, b->gstart_h.data(), sizeof(int) * b->ngroups, cudaMemcpyHostToDevice));
    BCK(cudaMemcpy(b->gcount, b->gcount_h.data(), sizeof(int) * b->ngroups, cudaMemcpyHostToDevice));
    return SGB_OK;
}

}  // namespace

// ---- batched add_sample! (called from sgb_corr_add_sample) ----------------------------------
// ---- launch shapes of the batched midpoint kernel and their autotuner ----------------------
//
// A shape is (neighbour-index staging, bonds gathered together, CTAs per SM). The staged
// shapes need their tiles' indices to fit in shared memory next to the coupling tables;
// the global-index shapes always fit. The first trajectory after the couplings are set
// times every shape that fits on a short run (3 steps without snapshots, the replicas'
// state saved and restored around it) and keeps the fastest for this batch.
template <class R>
using MidKernel = void (*)(BatchArgs<R>, MidArgs<R>, int, R, R, BSnap<R>, int);

template <class R, bool GEN>
static MidKernel<R> mid_kernel(int idx, int G, int bps) {
    // G = 6 runs 3 CTAs per SM within 80 registers, or in FP32 4 CTAs per SM within 64
    // (a few spilled bytes); G = 12 keeps twice as many neighbour loads in flight per thread
    // and runs 2 CTAs per SM within 128 registers (no spills)
    constexpr int M6 = sizeof(R) == 4 ? 3 : 2;
    if (G == 12) {
        if (idx == 2) return k_batch_midpoint<R, GEN, 2, 12, 2>;
        if (idx == 4) return k_batch_midpoint<R, GEN, 4, 12, 2>;
        return k_batch_midpoint<R, GEN, 0, 12, 2>;
    }
    if (sizeof(R) == 4 && bps >= 4) {
        if (idx == 2) return k_batch_midpoint<R, GEN, 2, 6, 4>;
        if (idx == 4) return k_batch_midpoint<R, GEN, 4, 6, 4>;
        return k_batch_midpoint<R, GEN, 0, 6, 4>;
    }
    if (idx == 2) return k_batch_midpoint<R, GEN, 2, 6, M6>;
    if (idx == 4) return k_batch_midpoint<R, GEN, 4, 6, M6>;
    return k_batch_midpoint<R, GEN, 0, 6, M6>;
}

static void blk_shapes(sgb_batch* b, bool gen, std::vector<MidShape>& out);

template <class R, bool GEN>
static int mid_shapes(sgb_batch* b, std::vector<MidShape>& out) {
    out.clear();
    const size_t tab = (size_t)b->tables_bytes;
    const int isz = b->nsr_max <= 65536 ? 2 : 4;
    const int maxbps = sizeof(R) == 4 ? 4 : 2;
    for (int idx : {isz, 0}) {
        if (idx != 0 && b->kb == 0) continue;
        for (int G : {6, 12}) {
            const int top = G == 12 ? 2 : maxbps;
            for (int bps = top; bps >= std::max(1, top - (top == 4 ? 2 : 1)); bps--) {
                const long long g = std::min<long long>((long long)bps * b->nsm, b->mid_ntiles);
                const long long ntb = (b->mid_ntiles + g - 1) / g;
                if (ntb > SGB_MAXT) continue;
                const size_t smem = tab + (idx ? (size_t)ntb * b->kb * SGB_TILE * idx : 0);
                MidKernel<R> kern = mid_kernel<R, GEN>(idx, G, bps);
                if (smem > 48 * 1024 &&
                    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
                    cudaGetLastError();
                    continue;
                }
                int fit = 0;
                if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, kern, SGB_TILE, smem) != cudaSuccess)
                    return bfail(b, SGB_ERR_CUDA, "occupancy query failed");
                if (fit < bps) continue;
                out.push_back(MidShape{idx, G, bps, (int)g, smem, 0.f});
            }
        }
    }
    if (std::is_same<R, float>::value && b->mid_nchunk == 1) blk_shapes(b, GEN, out);
    if (out.empty()) return bfail(b, SGB_ERR_ARG, "replica batch too large for one persistent launch of the midpoint kernel");
    return SGB_OK;
}

// Geometry of a cell-block shape for this batch (replicas of equal size).
static BlkGeom blk_geom(const sgb_batch* b, int lbx, int lby, int lbz) {
    BlkGeom g{};
    g.L1 = b->dims[0]; g.L2 = b->dims[1]; g.L3 = b->dims[2];
    g.na = b->na;
    g.gw = b->blk_gw;
    g.lbx = lbx; g.lby = lby; g.lbz = lbz;
    g.HX = (1 << lbx) + 2 * g.gw; g.HY = (1 << lby) + 2 * g.gw; g.HZ = (1 << lbz) + 2 * g.gw;
    g.PX = g.L1 + 2 * g.gw; g.PY = g.L2 + 2 * g.gw; g.PZ = g.L3 + 2 * g.gw;
    g.nbx = g.L1 >> lbx; g.nby = g.L2 >> lby; g.nbz = g.L3 >> lbz;
    g.nblk = g.nbx * g.nby * g.nbz * b->nrep;
    g.nsr = g.L1 * g.L2 * g.L3 * g.na;
    g.tx_bytes = (unsigned)(16ull * g.HX * g.HY * g.HZ * g.na);
    g.halo_bytes = g.tx_bytes;
    return g;
}

// Cell-block shapes (sgb_batch_blk.cu): FP32 batches of equal replicas whose bonds reach at
// most gw cells with 2 gw <= L. Blocks are powers of two dividing the supercell; the shapes
// kept are those of least halo per site whose box, tables and bond offsets fit in shared
// memory and whose blocks fit in one co-resident launch.
static void blk_shapes(sgb_batch* b, bool gen, std::vector<MidShape>& out) {
    for (int r = 1; r < b->nrep; r++)
        for (int k = 0; k < 3; k++)
            if (b->dims[3 * r + k] != b->dims[k]) return;
    int gw = 0;
    for (const sgb_bond& e : b->bonds)
        for (int k = 0; k < 3; k++) gw = std::max(gw, std::abs(e.n[k]));
    gw = std::max(gw, 1);
    for (int k = 0; k < 3; k++)
        if (b->dims[k] < 2 * gw) return;
    const size_t pad = (size_t)(b->dims[0] + 2 * gw) * (b->dims[1] + 2 * gw) * (b->dims[2] + 2 * gw) * b->na * b->nrep;
    if (b->Hpad && (b->blk_gw != gw || b->hpad_bytes != 3 * 16 * pad)) {
        bfree(b->Hpad);
        b->hpad_bytes = 0;
    }
    if (!b->Hpad) {
        if (cudaMalloc(&b->Hpad, 3 * 16 * pad) != cudaSuccess) {
            cudaGetLastError();
            b->Hpad = nullptr;
            return;
        }
        b->hpad_bytes = 3 * 16 * pad;
    }
    b->blk_gw = gw;
    b->blk_maps.clear();
    struct Cand {
        double cost;
        int lbx, lby, lbz;
    };
    std::vector<Cand> cands;
    auto log2_div = [](int L, int l) { return (L % (1 << l)) == 0; };
    for (int lx = 0; (1 << lx) <= b->dims[0]; lx++)
        for (int ly = 0; (1 << ly) <= b->dims[1]; ly++)
            for (int lz = 0; (1 << lz) <= b->dims[2]; lz++) {
                if (!log2_div(b->dims[0], lx) || !log2_div(b->dims[1], ly) || !log2_div(b->dims[2], lz)) continue;
                const long long nsb = (long long)b->na << (lx + ly + lz);
                if (nsb < 256 || nsb > 16 * SGB_BLK_THREADS_MAX) continue;
                BlkGeom g = blk_geom(b, lx, ly, lz);
                if (g.HX > 256 || g.HY > 256 || g.HZ > 256) continue;
                const size_t smem = 128 + g.halo_bytes + (size_t)b->tables_bytes + 4 * (size_t)((b->fp32 ? b->mf.nb : b->md.nb) + 4);
                if (smem > 200 * 1024) continue;
                cands.push_back({(double)g.HX * g.HY * g.HZ / (double)((1 << lx) * (1 << ly) * (1 << lz)), lx, ly, lz});
            }
    // rank, per thread count: fewest blocks per CTA (rounds of the block loop), then most
    // CTAs per SM, then least halo per site; the two best geometries of each thread count
    // are timed
    struct Fit {
        Cand c;
        int bps, rounds, nt;
        size_t smem;
    };
    std::vector<Fit> fits;
    for (int nt : {1024, 512, 256}) {
        std::vector<Fit> f1;
        for (const Cand& c : cands) {
            if (((long long)b->na << (c.lbx + c.lby + c.lbz)) < nt) continue;
            BlkGeom g = blk_geom(b, c.lbx, c.lby, c.lbz);
            const size_t smem = 128 + g.halo_bytes + (size_t)b->tables_bytes + 4 * (size_t)((b->fp32 ? b->mf.nb : b->md.nb) + 4);
            int bps = 0;
            if (blk_occupancy(gen, 6, nt, smem, &bps) != SGB_OK || bps < 1) {
                cudaGetLastError();
                continue;
            }
            const long long grid = std::min<long long>((long long)bps * b->nsm, g.nblk);
            const int rounds = (int)((g.nblk + grid - 1) / grid);
            if (rounds > SGB_BLK_MAXB) continue;
            f1.push_back({c, bps, rounds, nt, smem});
        }
        std::sort(f1.begin(), f1.end(), [](const Fit& p, const Fit& q) {
            if (p.rounds != q.rounds) return p.rounds < q.rounds;
            if (p.bps != q.bps) return p.bps > q.bps;
            return p.c.cost < q.c.cost;
        });
        for (size_t k = 0; k < f1.size() && k < 2; k++) fits.push_back(f1[k]);
    }
    int kept = 0;
    for (const Fit& f : fits) {
        if (kept >= 6) break;
        const Cand& c = f.c;
        BlkGeom g = blk_geom(b, c.lbx, c.lby, c.lbz);
        const size_t smem = f.smem;
        bool any = false;
        for (int G : {6}) {
            const int bps = f.bps;
            const long long grid = std::min<long long>((long long)bps * b->nsm, g.nblk);
            if (!any) {
                BlkMaps m;
                bool ok = true;
                for (int k = 0; k < 3 && ok; k++)
                    ok = blk_encode_map(&m.m[k], reinterpret_cast<float*>(b->Hpad) + (size_t)k * 4 * pad, g, b->nrep) == SGB_OK;
                if (!ok) break;
                b->blk_maps.push_back(m);
                any = true;
            }
            MidShape sh{0, G, bps, (int)grid, smem, 0.f};
            sh.kind = 1;
            sh.nt = f.nt;
            sh.lbx = c.lbx; sh.lby = c.lby; sh.lbz = c.lbz;
            sh.maps = (int)b->blk_maps.size() - 1;
            out.push_back(sh);
        }
        if (any) kept++;
    }
}

template <class R, bool GEN>
static int mid_launch(sgb_batch* b, const MidShape& sh, BatchArgs<R>& A, MidArgs<R>& X, int nsteps, R dt, R lam,
                      BSnap<R>& sn) {
    if constexpr (std::is_same<R, float>::value) {
        if (sh.kind == 1) {
            const BlkGeom g = blk_geom(b, sh.lbx, sh.lby, sh.lbz);
            b->launches++;
            if (blk_launch(GEN, sh.G, sh.nt, sh.grid, sh.smem, A, X, g, b->blk_maps[sh.maps], reinterpret_cast<float*>(b->Hpad), nsteps,
                           dt, lam, sn, b->stream) != SGB_OK)
                return bfail(b, SGB_ERR_CUDA, std::string("cell-block midpoint launch: ") + cudaGetErrorString(cudaGetLastError()));
            return SGB_OK;
        }
    }
    int kb = b->kb;
    void* args[] = {&A, &X, &nsteps, &dt, &lam, &sn, &kb};
    return bcoop(b, mid_kernel<R, GEN>(sh.idx, sh.G, sh.bps), sh.grid, sh.smem, args);
}

template <class R, bool GEN>
static int mid_tune(sgb_batch* b, BatchArgs<R>& A, MidArgs<R>& X, R dt, R lam, BSnap<R> sn) {
    std::vector<MidShape> shapes;
    int rc = mid_shapes<R, GEN>(b, shapes);
    if (rc) return rc;
    b->mid_shapes = shapes;
    if (shapes.size() == 1) {
        b->mid_choice = 0;
        return SGB_OK;
    }
    const size_t bytes = bsize(b) * 3 * (size_t)b->NS;
    BCK(cudaMemcpyAsync(b->P, b->S, bytes, cudaMemcpyDeviceToDevice, b->stream));   // P is free outside Langevin
    sn.enabled = 0;
    const int tsteps = 3;
    int best = 0;
    for (size_t k = 0; k < shapes.size(); k++) {
        float ms = 0.f;
        // an untimed launch, then the timed one behind it on the stream: the host's work for
        // the second launch (attributes, occupancy, tensor maps) overlaps the first's run,
        // so only the kernel is timed
        for (int rep = 0; rep < 2; rep++) {
            BCK(cudaMemcpyAsync(b->S, b->P, bytes, cudaMemcpyDeviceToDevice, b->stream));
            BCK(cudaMemsetAsync(b->ctrl, 0, sgb_ctrl_clear_bytes(), b->stream));
            if (rep == 1) BCK(cudaEventRecord(b->ev[6], b->stream));
            if ((rc = mid_launch<R, GEN>(b, shapes[k], A, X, tsteps, dt, lam, sn))) return rc;
        }
        BCK(cudaEventRecord(b->ev[7], b->stream));
        BCK(cudaEventSynchronize(b->ev[7]));
        BCK(cudaEventElapsedTime(&ms, b->ev[6], b->ev[7]));
        Ctrl st;
        if ((rc = read_status(b, &st))) return rc;
        b->mid_shapes[k].ms = st.status == 0 ? ms : 1e30f;
        if (b->mid_shapes[k].ms < b->mid_shapes[best].ms) best = (int)k;
    }
    BCK(cudaMemcpyAsync(b->S, b->P, bytes, cudaMemcpyDeviceToDevice, b->stream));
    b->mid_choice = best;
    return SGB_OK;
}

template <class R, bool GEN>
static int launch_midpoint(sgb_batch* b, BatchArgs<R>& A, MidArgs<R>& X, int nsteps, R dt, R lam, BSnap<R>& sn) {
    if (b->mid_choice < 0) {
        int rc = mid_tune<R, GEN>(b, A, X, dt, lam, sn);
        if (rc) return rc;
    }
    BCK(cudaMemsetAsync(b->ctrl, 0, sgb_ctrl_clear_bytes(), b->stream));
    return mid_launch<R, GEN>(b, b->mid_shapes[b->mid_choice], A, X, nsteps, dt, lam, sn);
}

// Replicas per midpoint launch: as many as keep the launch's working set (about 120 bytes
// per site in FP32, the state, iterate, history and three midpoint buffers) within about
// 72 MB of L2, in equal chunks; sgb_batch_set_midpoint_chunk overrides.
static void mid_chunking(sgb_batch* b) {
    const int nsr = b->off[1] - b->off[0];
    int cmax = b->mid_chunk;
    if (cmax <= 0) {
        const double per_site = b->fp32 ? 120.0 : 216.0;
        cmax = (int)std::max(1.0, std::floor(72.0e6 / (per_site * (double)nsr)));
    }
    cmax = std::min(cmax, b->nrep);
    const int nchunk = (b->nrep + cmax - 1) / cmax;
    const int per = (b->nrep + nchunk - 1) / nchunk;
    if (nchunk != b->mid_nchunk || per != b->mid_per) {
        b->mid_nchunk = nchunk;
        b->mid_per = per;
        b->mid_choice = -1;   // shapes depend on the tiles per launch
    }
    b->mid_ntiles = 0;
    for (int r = 0; r < std::min(per, b->nrep); r++) b->mid_ntiles += b->tcount[r];
}

template <class R>
static int batch_trajectory(sgb_corr* c, sgb_batch* b) {
    mid_chunking(b);
    MidArgs<R> X;
    X.Sp = (R*)b->Sp;
    X.H = (R*)b->H;
    X.racc = b->racc;
    X.P1 = (R*)b->P1;
    X.H1 = (R*)b->H1;
    X.H2 = (R*)b->H2;
    X.H3 = (R*)b->H3;
    X.ord = b->mid_order;
    X.accept0 = b->mid_accept0;
    double atol = c->tol * std::sqrt((double)(b->off[1] - b->off[0]));
    X.atol2 = atol * atol;
    X.max_iters = c->max_iters;
    BSnap<R> sn;
    sn.enabled = 1;
    sn.nobs = c->nobs;
    sn.measperiod = c->measperiod;
    sn.t0 = 0;
    sn.ncell = c->ncell;
    sn.na = c->npos;
    sn.ops = (const R*)c->ops;
    sn.buf = (R*)c->A;
    sn.rep_stride = (size_t)c->nomega * c->nobs * c->npos * c->ncell;
    sn.scale = (R)(1.0 / std::sqrt((double)c->ncell));
    int nsteps = c->measperiod * (c->nsnaps - 1);
    if (b->nrep > SGB_MAXREP_CORR) return bfail(b, SGB_ERR_ARG, "batched sampling supports at most 64 replicas");
    R dt = (R)c->dt, lam = (R)c->damping;
    int64_t iters = 0;
    // one launch per chunk of replicas; their snapshots land in their own rows of the
    // accumulator's time series, which one rank-nrep pass then accumulates
    for (int r0 = 0; r0 < b->nrep; r0 += b->mid_per) {
        const int cn = std::min(b->mid_per, b->nrep - r0);
        BatchArgs<R> A = bargs<R>(b);
        const int t0 = b->tfirst[r0], t1 = b->tfirst[r0 + cn - 1] + b->tcount[r0 + cn - 1];
        A.td = b->td + 2 * (size_t)t0;
        A.ntiles = t1 - t0;
        X.nrep = cn;
        X.r0 = r0;
        int rc = A.M.general ? launch_midpoint<R, true>(b, A, X, nsteps, dt, lam, sn)
                             : launch_midpoint<R, false>(b, A, X, nsteps, dt, lam, sn);
        if (rc) return rc;
        Ctrl st;
        if ((rc = read_status(b, &st))) return rc;
        iters += st.iters;
        if (st.status == SGB_ERR_NOCONVERGE)
            return bfail(b, SGB_ERR_NOCONVERGE, "Spherical midpoint method failed to converge to tolerance " +
                                                    std::to_string(c->tol) + " after " + std::to_string(c->max_iters) +
                                                    " iterations.");
        if (st.status != 0) return bfail(b, st.status, "batched midpoint kernel reported an error");
    }
    c->prof_iters_last = iters;
    return SGB_OK;
}

int batch_corr_trajectory(sgb_corr* c) {
    sgb_batch* b = c->batch;
    if (!b->grp.empty()) return group_trajectory(c);
    return b->fp32 ? batch_trajectory<float>(c, b) : batch_trajectory<double>(c, b);
}

const char* batch_error(sgb_batch* b) { return b->err.c_str(); }

// ---------------------------------------------------------------------------------------------
extern "C" {

const char* sgb_batch_last_error(const sgb_batch* b) { return b ? b->err.c_str() : g_batch_error.c_str(); }

void sgb_batch_destroy(sgb_batch* b) {
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    sgb_detach_corrs(b->corrs);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    bfree(b->tables); bfree(b->kap); bfree(b->h);
    void* p;
    p = b->rd; bfree(p); p = b->roff; bfree(p); p = b->kT; bfree(p); bfree(b->kTR); p = b->ladder; bfree(p);
    p = b->gstart; bfree(p); p = b->gcount; bfree(p); p = b->tiles; bfree(p); p = b->tfirst_d; bfree(p);
    p = b->tcount_d; bfree(p);
    p = b->pc; bfree(p);
    p = b->nbr; bfree(p);
    p = b->nbo; bfree(p);
    p = b->td; bfree(p);
    bfree(b->S); bfree(b->P); bfree(b->D1); bfree(b->Sp); bfree(b->H); bfree(b->P1); bfree(b->H1); bfree(b->H2); bfree(b->H3);
    bfree(b->Hpad);
    p = b->racc; bfree(p); p = b->ctrl; bfree(p); p = b->Epart; bfree(p); p = b->E; bfree(p);
    p = b->counters; bfree(p); p = b->n_accept; bfree(p);
    if (b->stage) cudaFreeHost(b->stage);
    for (int i = 0; i < 8; i++) if (b->ev[i]) cudaEventDestroy(b->ev[i]);
    for (cudaEvent_t e : b->gev) if (e) cudaEventDestroy(e);
    if (b->gfork) cudaEventDestroy(b->gfork);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

int sgb_batch_create_group(sgb_system* const* systems, int32_t nrep, sgb_batch** out) {
    if (!systems || !out || nrep < 1 || nrep > 64) return bfail(nullptr, SGB_ERR_ARG, "a replica group has 1 to 64 systems");
    *out = nullptr;
    const sgb_system* s0 = systems[0];
    if (!s0) return bfail(nullptr, SGB_ERR_ARG, "null system");
    for (int r = 0; r < nrep; r++) {
        const sgb_system* s = systems[r];
        if (!s) return bfail(nullptr, SGB_ERR_ARG, "null system");
        if (s->d.mode != s0->d.mode || s->N != s0->N || s->fp32 != s0->fp32 || s->d.natoms != s0->d.natoms ||
            s->d.device != s0->d.device || s->d.dims[0] != s0->d.dims[0] || s->d.dims[1] != s0->d.dims[1] ||
            s->d.dims[2] != s0->d.dims[2])
            return bfail(nullptr, SGB_ERR_ARG, "the systems of a replica group must share mode, precision, device and dims");
        for (int q = 0; q < r; q++)
            if (systems[q] == s) return bfail(nullptr, SGB_ERR_ARG, "a system appears twice in the replica group");
    }
    sgb_batch* b = new sgb_batch();
    b->proto = s0->d;
    b->nrep = nrep;
    b->na = s0->d.natoms;
    b->fp32 = s0->fp32;
    b->nsm = s0->nsm;
    b->grp.assign(systems, systems + nrep);
    b->dims.clear();
    b->off.assign(nrep + 1, 0);
    for (int r = 0; r < nrep; r++) {
        for (int k = 0; k < 3; k++) b->dims.push_back(s0->d.dims[k]);
        b->off[r + 1] = b->off[r] + s0->ns;
    }
    b->NS = b->off[nrep];
    b->nsr_max = s0->ns;
    b->kT_h.assign(nrep, 0.0);
    b->coup_set = true;
    b->state_set = true;
    auto bad = [&]() { std::string m = b->err; b->grp.clear(); sgb_batch_destroy(b); g_batch_error = m; return SGB_ERR_CUDA; };
    if (cudaSetDevice(s0->d.device) != cudaSuccess) { bfail(b, SGB_ERR_CUDA, "cudaSetDevice failed"); return bad(); }
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) { bfail(b, SGB_ERR_CUDA, "stream"); return bad(); }
    for (int i = 0; i < 8; i++) cudaEventCreate(&b->ev[i]);
    b->gev.assign(nrep, nullptr);
    for (int r = 0; r < nrep; r++)
        if (cudaEventCreateWithFlags(&b->gev[r], cudaEventDisableTiming) != cudaSuccess) { bfail(b, SGB_ERR_CUDA, "event"); return bad(); }
    if (cudaEventCreateWithFlags(&b->gfork, cudaEventDisableTiming) != cudaSuccess) { bfail(b, SGB_ERR_CUDA, "event"); return bad(); }
    *out = b;
    return SGB_OK;
}

int sgb_batch_create(const sgb_desc* d, int32_t nrep, const int32_t* dims, sgb_batch** out) {
    if (!d || !dims || !out || nrep < 1) return bfail(nullptr, SGB_ERR_ARG, "invalid arguments");
    *out = nullptr;
    if (d->mode == SGB_MODE_SUN) return bfail(nullptr, SGB_ERR_ARG, "replica batches support the dipole modes");
    if (d->natoms < 1 || d->natoms > SGB_MAX_SUBLAT) return bfail(nullptr, SGB_ERR_ARG, "natoms must be in [1, 64]");
    if (d->precision != SGB_FP32 && d->precision != SGB_FP64) return bfail(nullptr, SGB_ERR_ARG, "bad precision");
    sgb_batch* b = new sgb_batch();
    b->proto = *d;
    b->nrep = nrep;
    b->na = d->natoms;
    b->fp32 = d->precision == SGB_FP32;
    b->mid_order = b->fp32 ? 4 : 0;
    b->dims.assign(dims, dims + 3 * nrep);
    b->off.assign(nrep + 1, 0);
    long long tot = 0;
    for (int r = 0; r < nrep; r++) {
        for (int k = 0; k < 3; k++)
            if (dims[3 * r + k] < 1 || dims[3 * r + k] > 255) {
                sgb_batch_destroy(b);
                return bfail(nullptr, SGB_ERR_ARG, "replica dims must be in [1, 255]");
            }
        b->off[r] = (int)tot;
        tot += (long long)dims[3 * r] * dims[3 * r + 1] * dims[3 * r + 2] * b->na;
        if (tot > (1LL << 30)) { sgb_batch_destroy(b); return bfail(nullptr, SGB_ERR_ARG, "too many sites"); }
    }
    b->off[nrep] = (int)tot;
    b->NS = (int)tot;
    for (int r = 0; r < nrep; r++) b->nsr_max = std::max(b->nsr_max, b->off[r + 1] - b->off[r]);
    auto bad = [&](int code) { std::string m = b->err; sgb_batch_destroy(b); g_batch_error = m; return code; };
    if (cudaSetDevice(d->device) != cudaSuccess) { bfail(b, SGB_ERR_CUDA, "cudaSetDevice failed"); return bad(SGB_ERR_CUDA); }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, d->device) != cudaSuccess) { bfail(b, SGB_ERR_CUDA, "no device"); return bad(SGB_ERR_CUDA); }
    b->nsm = prop.multiProcessorCount;
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) { bfail(b, SGB_ERR_CUDA, "stream"); return bad(SGB_ERR_CUDA); }
    for (int i = 0; i < 8; i++) cudaEventCreate(&b->ev[i]);
    // tiles: contiguous per replica
    std::vector<int4> tiles;
    b->tfirst.assign(nrep, 0);
    b->tcount.assign(nrep, 0);
    for (int r = 0; r < nrep; r++) {
        int ns = b->off[r + 1] - b->off[r];
        b->tfirst[r] = (int)tiles.size();
        for (int s0 = 0; s0 < ns; s0 += SGB_TILE) tiles.push_back(make_int4(r, s0, std::min(SGB_TILE, ns - s0), 0));
        b->tcount[r] = (int)tiles.size() - b->tfirst[r];
    }
    b->ntiles = (int)tiles.size();
    std::vector<int4> rd(nrep);
    for (int r = 0; r < nrep; r++) rd[r] = make_int4(dims[3 * r], dims[3 * r + 1], dims[3 * r + 2], dims[3 * r] * dims[3 * r + 1] * dims[3 * r + 2]);
    size_t R = bsize(b);
    int rc = SGB_OK;
    rc |= bmalloc(b, (void**)&b->rd, sizeof(int4) * nrep);
    rc |= bmalloc(b, (void**)&b->roff, sizeof(int) * (nrep + 1));
    rc |= bmalloc(b, (void**)&b->kT, sizeof(double) * nrep);
    rc |= bmalloc(b, (void**)&b->kTR, sizeof(double) * nrep);
    rc |= bmalloc(b, (void**)&b->ladder, sizeof(int) * nrep);
    rc |= bmalloc(b, (void**)&b->gstart, sizeof(int) * nrep);
    rc |= bmalloc(b, (void**)&b->gcount, sizeof(int) * nrep);
    rc |= bmalloc(b, (void**)&b->tiles, sizeof(int4) * b->ntiles);
    rc |= bmalloc(b, (void**)&b->tfirst_d, sizeof(int) * nrep);
    rc |= bmalloc(b, (void**)&b->tcount_d, sizeof(int) * nrep);
    rc |= bmalloc(b, (void**)&b->pc, sizeof(int) * b->NS);
    rc |= bmalloc(b, &b->S, R * 3 * b->NS);
    rc |= bmalloc(b, &b->P, R * 3 * b->NS);
    rc |= bmalloc(b, &b->D1, R * 3 * b->NS);
    rc |= bmalloc(b, (void**)&b->ctrl, sizeof(Ctrl));
    rc |= bmalloc(b, (void**)&b->Epart, sizeof(double) * b->ntiles);
    rc |= bmalloc(b, (void**)&b->E, sizeof(double) * nrep);
    rc |= bmalloc(b, (void**)&b->counters, sizeof(unsigned long long) * 2);
    rc |= bmalloc(b, (void**)&b->n_accept, sizeof(long long) * nrep);
    if (rc) return bad(SGB_ERR_NOMEM);
    cudaMemcpy(b->rd, rd.data(), sizeof(int4) * nrep, cudaMemcpyHostToDevice);
    cudaMemcpy(b->roff, b->off.data(), sizeof(int) * (nrep + 1), cudaMemcpyHostToDevice);
    cudaMemcpy(b->tiles, tiles.data(), sizeof(int4) * b->ntiles, cudaMemcpyHostToDevice);
    cudaMemcpy(b->tfirst_d, b->tfirst.data(), sizeof(int) * nrep, cudaMemcpyHostToDevice);
    cudaMemcpy(b->tcount_d, b->tcount.data(), sizeof(int) * nrep, cudaMemcpyHostToDevice);
    {
        std::vector<int> pcv(b->NS);
        for (int r = 0; r < nrep; r++) {
            const int L1 = dims[3 * r], L2 = dims[3 * r + 1], L3 = dims[3 * r + 2];
            int k = b->off[r];
            for (int a = 0; a < b->na; a++)
                for (int c3 = 0; c3 < L3; c3++)
                    for (int c2 = 0; c2 < L2; c2++)
                        for (int c1 = 0; c1 < L1; c1++) pcv[k++] = c1 | (c2 << 8) | (c3 << 16) | (a << 24);
        }
        cudaMemcpy(b->pc, pcv.data(), sizeof(int) * b->NS, cudaMemcpyHostToDevice);
    }
    cudaMemset(b->S, 0, R * 3 * b->NS);
    cudaMemset(b->ctrl, 0, sizeof(Ctrl));
    cudaMemset(b->counters, 0, sizeof(unsigned long long) * 2);
    cudaMemset(b->n_accept, 0, sizeof(long long) * nrep);
    b->kT_h.assign(nrep, 0.0);
    cudaMemset(b->kT, 0, sizeof(double) * nrep);
    cudaMemset(b->kTR, 0, sizeof(double) * nrep);
    if (rebuild_groups(b)) return bad(SGB_ERR_CUDA);
    *out = b;
    return SGB_OK;
}

int64_t sgb_batch_nsites(const sgb_batch* b, int32_t rep) {
    if (!b || rep < 0 || rep >= b->nrep) return 0;
    return b->off[rep + 1] - b->off[rep];
}

int sgb_batch_set_couplings(sgb_batch* b, const double* kappa, const double* g, const double* field,
                            const double* onsite, const sgb_bond* bonds, int32_t nbonds) {
    if (!b || !kappa || !g || (nbonds > 0 && !bonds) || nbonds < 0) return bfail(b, SGB_ERR_ARG, "invalid arguments");
    const int na = b->na;
    for (int k = 0; k < nbonds; k++) {
        const sgb_bond& e = bonds[k];
        if (e.i == e.j && e.n[0] == 0 && e.n[1] == 0 && e.n[2] == 0) return bfail(b, SGB_ERR_ARG, "Bond must connect different atoms.");
        if (e.i < 0 || e.i >= na || e.j < 0 || e.j >= na) return bfail(b, SGB_ERR_ARG, "atom index out of range");
        for (int r = 0; r < b->nrep; r++)
            for (int q = 0; q < 3; q++)
                if (std::abs(e.n[q]) > b->dims[3 * r + q])
                    return bfail(b, SGB_ERR_ARG, "bond offset larger than a replica's supercell");
    }
    b->kappa_a.assign(kappa, kappa + na);
    b->g_a.assign(g, g + 9 * na);
    b->field_a.assign(3 * na, 0.0);
    if (field) b->field_a.assign(field, field + 3 * na);
    b->onsite.assign(28 * na, 0.0);
    if (onsite) b->onsite.assign(onsite, onsite + 28 * na);
    b->bonds.assign(bonds, bonds + nbonds);
    std::vector<double> hh(3 * na, 0.0);
    b->has_field = false;
    for (int a = 0; a < na; a++)
        for (int r = 0; r < 3; r++) {
            const double* ga = b->g_a.data() + 9 * a;
            const double* B = b->field_a.data() + 3 * a;
            double v = ga[0 + 3 * r] * B[0] + ga[1 + 3 * r] * B[1] + ga[2 + 3 * r] * B[2];
            hh[r * na + a] = v;
            b->has_field |= v != 0.0;
        }
    size_t R = bsize(b);
    bfree(b->kap);
    bfree(b->h);
    int rc = bmalloc(b, &b->kap, R * na);
    rc |= bmalloc(b, &b->h, R * 3 * na);
    if (rc) return SGB_ERR_NOMEM;
    std::vector<unsigned char> buf;
    bool any_bq = false;
    std::string e;
    if (b->fp32) {
        std::vector<float> k(na), hf(3 * na);
        for (int a = 0; a < na; a++) k[a] = (float)kappa[a];
        for (int i = 0; i < 3 * na; i++) hf[i] = (float)hh[i];
        BCK(cudaMemcpy(b->kap, k.data(), 4 * na, cudaMemcpyHostToDevice));
        BCK(cudaMemcpy(b->h, hf.data(), 4 * 3 * na, cudaMemcpyHostToDevice));
        e = sgbhost::pack_tables<float>(na, 0, false, nullptr, b->bonds, b->onsite, b->mf, buf, any_bq);
    } else {
        BCK(cudaMemcpy(b->kap, kappa, 8 * na, cudaMemcpyHostToDevice));
        BCK(cudaMemcpy(b->h, hh.data(), 8 * 3 * na, cudaMemcpyHostToDevice));
        e = sgbhost::pack_tables<double>(na, 0, false, nullptr, b->bonds, b->onsite, b->md, buf, any_bq);
    }
    if (!e.empty()) return bfail(b, SGB_ERR_ARG, e);
    bfree(b->tables);
    if ((rc = bmalloc(b, &b->tables, buf.size()))) return rc;
    BCK(cudaMemcpy(b->tables, buf.data(), buf.size(), cudaMemcpyHostToDevice));
    b->tables_bytes = (int)buf.size();
    {
        // neighbour tables: one per distinct replica size, [k][s] for bond k of the site's sublattice
        const int off_boff = b->fp32 ? b->mf.off_boff : b->md.off_boff;
        const int off_bonds = b->fp32 ? b->mf.off_bonds : b->md.off_bonds;
        const size_t bsz = b->fp32 ? sizeof(DBond<float>) : sizeof(DBond<double>);
        const size_t pk_off = b->fp32 ? offsetof(DBond<float>, pk) : offsetof(DBond<double>, pk);
        const int* boff = reinterpret_cast<const int*>(buf.data() + off_boff);
        int kb = 0;
        for (int a = 0; a < na; a++) kb = std::max(kb, boff[a + 1] - boff[a]);
        b->kb = kb;
        std::vector<int> table, nbo(b->nrep, 0);
        std::vector<std::array<int, 4>> seen;   // (L1, L2, L3, offset)
        for (int r = 0; r < b->nrep; r++) {
            const int L1 = b->dims[3 * r], L2 = b->dims[3 * r + 1], L3 = b->dims[3 * r + 2];
            int found = -1;
            for (auto& e : seen)
                if (e[0] == L1 && e[1] == L2 && e[2] == L3) found = e[3];
            if (found >= 0) { nbo[r] = found; continue; }
            const int nsr = L1 * L2 * L3 * na;
            const int base = (int)table.size();
            table.resize(table.size() + (size_t)std::max(kb, 1) * nsr, 0);
            for (int a = 0; a < na; a++)
                for (int c3 = 0; c3 < L3; c3++)
                    for (int c2 = 0; c2 < L2; c2++)
                        for (int c1 = 0; c1 < L1; c1++) {
                            const int site = c1 + L1 * (c2 + L2 * (c3 + L3 * a));
                            for (int k = 0; k < boff[a + 1] - boff[a]; k++) {
                                int pk;
                                std::memcpy(&pk, buf.data() + off_bonds + (size_t)(boff[a] + k) * bsz + pk_off, sizeof(int));
                                int x1 = sgbhost::imod(c1 + (pk & 0xff) - 128, L1);
                                int x2 = sgbhost::imod(c2 + ((pk >> 8) & 0xff) - 128, L2);
                                int x3 = sgbhost::imod(c3 + ((pk >> 16) & 0xff) - 128, L3);
                                int j = (int)((unsigned)pk >> 24);
                                table[base + (size_t)k * nsr + site] = x1 + L1 * (x2 + L2 * (x3 + L3 * j));
                            }
                        }
            seen.push_back({L1, L2, L3, base});
            nbo[r] = base;
        }
        void* p;
        p = b->nbr; bfree(p); p = b->nbo; bfree(p);
        if ((rc = bmalloc(b, (void**)&b->nbr, sizeof(int) * std::max<size_t>(1, table.size())))) return rc;
        if ((rc = bmalloc(b, (void**)&b->nbo, sizeof(int) * b->nrep))) return rc;
        if (!table.empty()) BCK(cudaMemcpy(b->nbr, table.data(), sizeof(int) * table.size(), cudaMemcpyHostToDevice));
        BCK(cudaMemcpy(b->nbo, nbo.data(), sizeof(int) * b->nrep, cudaMemcpyHostToDevice));
        // tile descriptors
        std::vector<int4> td(2 * (size_t)b->ntiles);
        std::vector<int4> tl(b->ntiles);
        BCK(cudaMemcpy(tl.data(), b->tiles, sizeof(int4) * b->ntiles, cudaMemcpyDeviceToHost));
        for (int t = 0; t < b->ntiles; t++) {
            const int r = tl[t].x, s0 = tl[t].y, cnt = tl[t].z;
            const int ncell = b->dims[3 * r] * b->dims[3 * r + 1] * b->dims[3 * r + 2];
            const int a0 = s0 / ncell, a1 = (s0 + cnt - 1) / ncell;
            td[2 * t] = make_int4(r, s0, cnt, a0 == a1 ? a0 : -1);
            td[2 * t + 1] = make_int4(b->off[r], b->off[r + 1] - b->off[r], nbo[r], 0);
        }
        p = b->td; bfree(p);
        if ((rc = bmalloc(b, (void**)&b->td, sizeof(int4) * td.size()))) return rc;
        BCK(cudaMemcpy(b->td, td.data(), sizeof(int4) * td.size(), cudaMemcpyHostToDevice));
    }
    for (Model<float>* m : {&b->mf}) { m->tables = (const unsigned char*)b->tables; m->dipole_mode = 1; m->na = na; }
    for (Model<double>* m : {&b->md}) { m->tables = (const unsigned char*)b->tables; m->dipole_mode = 1; m->na = na; }
    if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
    b->mid_choice = -1;
    b->heun_bps = 0;
    for (float& m : b->heun_ms) m = 0.f;
    b->coup_set = true;
    return SGB_OK;
}

int sgb_batch_set_state(sgb_batch* b, int32_t rep, const double* dip) {
    if (!b || !dip || rep < 0 || rep >= b->nrep) return bfail(b, SGB_ERR_ARG, "invalid arguments");
    if (!b->grp.empty()) {
        sgb_system* s = b->grp[rep];
        if (s->sun) return bfail(b, SGB_ERR_ARG, "set the coherent states of the member system");
        const int rc = sgb_set_state(s, dip, nullptr);
        return rc ? bfail(b, rc, s->err) : SGB_OK;
    }
    const int ns = b->off[rep + 1] - b->off[rep], NS = b->NS, o = b->off[rep];
    size_t R = bsize(b);
    int rc = ensure_bstage(b, R * 3 * ns);
    if (rc) return rc;
    for (int c = 0; c < 3; c++) {
        for (int i = 0; i < ns; i++) {
            if (b->fp32) reinterpret_cast<float*>(b->stage)[i] = (float)dip[3 * (size_t)i + c];
            else reinterpret_cast<double*>(b->stage)[i] = dip[3 * (size_t)i + c];
        }
        BCK(cudaMemcpyAsync((char*)b->S + R * ((size_t)c * NS + o), b->stage, R * ns, cudaMemcpyHostToDevice, b->stream));
        BCK(cudaStreamSynchronize(b->stream));
    }
    b->state_set = true;
    return SGB_OK;
}

int sgb_batch_get_state(sgb_batch* b, int32_t rep, double* dip) {
    if (!b || !dip || rep < 0 || rep >= b->nrep) return bfail(b, SGB_ERR_ARG, "invalid arguments");
    if (!b->grp.empty()) {
        sgb_system* s = b->grp[rep];
        const int rc = sgb_get_state(s, dip, nullptr);   // SU(N): the expected dipoles
        return rc ? bfail(b, rc, s->err) : SGB_OK;
    }
    const int ns = b->off[rep + 1] - b->off[rep], NS = b->NS, o = b->off[rep];
    size_t R = bsize(b);
    int rc = ensure_bstage(b, R * 3 * ns);
    if (rc) return rc;
    for (int c = 0; c < 3; c++) {
        BCK(cudaMemcpyAsync(b->stage, (char*)b->S + R * ((size_t)c * NS + o), R * ns, cudaMemcpyDeviceToHost, b->stream));
        BCK(cudaStreamSynchronize(b->stream));
        for (int i = 0; i < ns; i++)
            dip[3 * (size_t)i + c] = b->fp32 ? (double)reinterpret_cast<float*>(b->stage)[i] : reinterpret_cast<double*>(b->stage)[i];
    }
    return SGB_OK;
}

int sgb_batch_set_kT(sgb_batch* b, const double* kT) {
    if (!b || !kT) return bfail(b, SGB_ERR_ARG, "invalid arguments");
    for (int r = 0; r < b->nrep; r++)
        if (!(kT[r] >= 0)) return bfail(b, SGB_ERR_ARG, "Select nonnegative kT");
    b->kT_h.assign(kT, kT + b->nrep);
    if (!b->grp.empty()) return SGB_OK;
    BCK(cudaMemcpy(b->kT, kT, sizeof(double) * b->nrep, cudaMemcpyHostToDevice));
    if (b->fp32) {
        std::vector<float> f(kT, kT + b->nrep);
        BCK(cudaMemcpy(b->kTR, f.data(), sizeof(float) * b->nrep, cudaMemcpyHostToDevice));
    } else {
        BCK(cudaMemcpy(b->kTR, kT, sizeof(double) * b->nrep, cudaMemcpyHostToDevice));
    }
    return rebuild_groups(b);
}

int sgb_batch_get_kT(sgb_batch* b, double* kT) {
    if (!b || !kT) return bfail(b, SGB_ERR_ARG, "invalid arguments");
    if (!b->grp.empty()) {
        for (int r = 0; r < b->nrep; r++) kT[r] = b->kT_h[r];
        return SGB_OK;
    }
    BCK(cudaMemcpyAsync(kT, b->kT, sizeof(double) * b->nrep, cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    return SGB_OK;
}

int sgb_batch_langevin(sgb_batch* b, double dt, double damping, uint64_t seed, uint64_t step0, int32_t nsteps) {
    if (!b) return bfail(b, SGB_ERR_ARG, "null handle");
    if (damping == 0.0) return bfail(b, SGB_ERR_ARG, "Use ImplicitMidpoint instead for energy-conserving dynamics");
    if (!(dt > 0)) return bfail(b, SGB_ERR_ARG, "Select positive dt");
    if (damping < 0) return bfail(b, SGB_ERR_ARG, "Select positive damping");
    if (!b->coup_set || !b->state_set) return bfail(b, SGB_ERR_STATE, "couplings and states must be set first");
    if (nsteps <= 0) return nsteps == 0 ? SGB_OK : bfail(b, SGB_ERR_ARG, "nsteps must be nonnegative");
    if (!b->grp.empty()) return group_langevin(b, dt, damping, seed, step0, nsteps);
    int rc = b->fp32 ? tune_langevin<float>(b, dt, damping, seed) : tune_langevin<double>(b, dt, damping, seed);
    if (rc) return rc;
    unsigned long long s0 = step0;
    BCK(cudaMemcpyAsync(b->counters, &s0, sizeof(s0), cudaMemcpyHostToDevice, b->stream));
    BCK(cudaMemsetAsync(b->ctrl, 0, sgb_ctrl_clear_bytes(), b->stream));
    rc = b->fp32 ? enqueue_langevin<float>(b, dt, damping, seed, nsteps) : enqueue_langevin<double>(b, dt, damping, seed, nsteps);
    if (rc) return rc;
    Ctrl st;
    if ((rc = read_status(b, &st))) return rc;
    if (st.status != 0) return bfail(b, st.status, "batched Langevin kernel reported an error");
    return SGB_OK;
}

int sgb_batch_langevin_noise(sgb_batch* b, int32_t rep, uint64_t seed, uint64_t step, double* out) {
    if (!b || !out || rep < 0 || rep >= b->nrep) return bfail(b, SGB_ERR_ARG, "invalid arguments");
    if (!b->grp.empty()) {   // member r draws with seed + r
        sgb_system* s = b->grp[rep];
        const int rc = sgb_langevin_noise(s, seed + (uint64_t)rep, step, out);
        return rc ? bfail(b, rc, s->err) : SGB_OK;
    }
    const int ns = b->off[rep + 1] - b->off[rep];
    double* d = nullptr;
    if (bmalloc(b, (void**)&d, sizeof(double) * 3 * ns)) return SGB_ERR_NOMEM;
    int grid = std::min(4096, (ns + 255) / 256);
    if (b->fp32) k_batch_noise<float><<<grid, 256, 0, b->stream>>>(ns, rep, seed, step, d);
    else k_batch_noise<double><<<grid, 256, 0, b->stream>>>(ns, rep, seed, step, d);
    b->launches++;
    cudaError_t e = cudaMemcpyAsync(out, d, sizeof(double) * 3 * ns, cudaMemcpyDeviceToHost, b->stream);
    cudaStreamSynchronize(b->stream);
    cudaFree(d);
    return e == cudaSuccess ? SGB_OK : bfail(b, SGB_ERR_CUDA, "noise export failed");
}

int sgb_batch_energy(sgb_batch* b, double* E) {
    if (!b || !E) return bfail(b, SGB_ERR_ARG, "invalid arguments");
    if (!b->coup_set) return bfail(b, SGB_ERR_STATE, "couplings must be set first");
    if (!b->grp.empty()) return group_energy(b, E);
    int rc = b->fp32 ? enqueue_energy<float>(b) : enqueue_energy<double>(b);
    if (rc) return rc;
    BCK(cudaMemcpyAsync(E, b->E, sizeof(double) * b->nrep, cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    return SGB_OK;
}

int sgb_batch_exchange(sgb_batch* b, int32_t exch_start, uint64_t seed, uint64_t round, const double* uniforms,
                       int64_t* n_accept) {
    if (!b || (exch_start != 1 && exch_start != 2)) return bfail(b, SGB_ERR_ARG, "exch_start must be 1 or 2");
    if (!b->grp.empty()) return bfail(b, SGB_ERR_ARG, "replica exchange over systems runs through ParallelTempering(system, sampler, kT_sched)");
    if (!b->coup_set) return bfail(b, SGB_ERR_STATE, "couplings must be set first");
    int rc = b->fp32 ? enqueue_energy<float>(b) : enqueue_energy<double>(b);
    if (rc) return rc;
    double* u = nullptr;
    if (uniforms) {
        if (bmalloc(b, (void**)&u, sizeof(double) * b->nrep)) return SGB_ERR_NOMEM;
        BCK(cudaMemcpyAsync(u, uniforms, sizeof(double) * b->nrep, cudaMemcpyHostToDevice, b->stream));
    }
    rc = enqueue_exchange(b, exch_start, seed, round, u);
    cudaStreamSynchronize(b->stream);
    if (u) cudaFree(u);
    if (rc) return rc;
    if (n_accept) {
        std::vector<long long> na(b->nrep);
        BCK(cudaMemcpy(na.data(), b->n_accept, sizeof(long long) * b->nrep, cudaMemcpyDeviceToHost));
        for (int i = 0; i < b->nrep; i++) n_accept[i] = na[i];
    }
    return SGB_OK;
}

int sgb_batch_step_ensemble(sgb_batch* b, double dt, double damping, uint64_t seed, int32_t nsteps, int32_t exch_interval,
                            int64_t* n_accept) {
    if (!b || exch_interval < 1 || nsteps < 0) return bfail(b, SGB_ERR_ARG, "invalid arguments");
    if (!b->grp.empty()) return bfail(b, SGB_ERR_ARG, "replica exchange over systems runs through ParallelTempering(system, sampler, kT_sched)");
    if (damping <= 0 || !(dt > 0)) return bfail(b, SGB_ERR_ARG, "Select positive dt and damping");
    if (!b->coup_set || !b->state_set) return bfail(b, SGB_ERR_STATE, "couplings and states must be set first");
    const int n_exch = (nsteps + exch_interval - 1) / exch_interval;
    int rc = b->fp32 ? tune_langevin<float>(b, dt, damping, seed) : tune_langevin<double>(b, dt, damping, seed);
    if (rc) return rc;
    BCK(cudaMemsetAsync(b->ctrl, 0, sgb_ctrl_clear_bytes(), b->stream));
    BCK(cudaMemsetAsync(b->counters + 1, 0, sizeof(unsigned long long), b->stream));
    const bool reuse = b->graph && b->graph_interval == exch_interval && b->graph_dt == dt && b->graph_damping == damping &&
                       b->graph_seed == seed;
    if (!reuse) {
        if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
        // capture one round: exch_interval Langevin steps, energies, one exchange
        cudaGraph_t g = nullptr;
        bool captured = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
        if (captured) {
            rc = b->fp32 ? enqueue_langevin<float>(b, dt, damping, seed, exch_interval)
                         : enqueue_langevin<double>(b, dt, damping, seed, exch_interval);
            if (!rc) rc = b->fp32 ? enqueue_energy<float>(b) : enqueue_energy<double>(b);
            if (!rc) rc = enqueue_exchange(b, 0, seed, 0, nullptr);
            cudaError_t e = cudaStreamEndCapture(b->stream, &g);
            if (rc || e != cudaSuccess || !g || cudaGraphInstantiate(&b->graph, g, 0) != cudaSuccess) {
                b->graph = nullptr;
                cudaGetLastError();
            }
            if (g) cudaGraphDestroy(g);
        }
        b->graph_interval = exch_interval;
        b->graph_dt = dt;
        b->graph_damping = damping;
        b->graph_seed = seed;
    }
    for (int i = 0; i < n_exch; i++) {
        if (b->graph) {
            if (cudaGraphLaunch(b->graph, b->stream) != cudaSuccess) return bfail(b, SGB_ERR_CUDA, "cudaGraphLaunch failed");
            b->launches += 4;
        } else {
            rc = b->fp32 ? enqueue_langevin<float>(b, dt, damping, seed, exch_interval)
                         : enqueue_langevin<double>(b, dt, damping, seed, exch_interval);
            if (!rc) rc = b->fp32 ? enqueue_energy<float>(b) : enqueue_energy<double>(b);
            if (!rc) rc = enqueue_exchange(b, 0, seed, 0, nullptr);
            if (rc) return rc;
        }
    }
    Ctrl st;
    if ((rc = read_status(b, &st))) return rc;
    if (st.status != 0) return bfail(b, st.status, "step_ensemble kernel reported an error");
    if (n_accept) {
        std::vector<long long> na(b->nrep);
        BCK(cudaMemcpy(na.data(), b->n_accept, sizeof(long long) * b->nrep, cudaMemcpyDeviceToHost));
        for (int i = 0; i < b->nrep; i++) n_accept[i] = na[i];
    }
    return SGB_OK;
}

int sgb_batch_graph_active(const sgb_batch* b) { return b && b->graph ? 1 : 0; }

int sgb_batch_set_midpoint_predictor(sgb_batch* b, int32_t order) {
    if (!b) return bfail(nullptr, SGB_ERR_ARG, "null handle");
    if (order < 0 || order > 4) return bfail(b, SGB_ERR_ARG, "predictor order must be in 0..4");
    b->mid_order = order;
    for (sgb_system* s : b->grp) s->mid_order = order;
    return SGB_OK;
}

int sgb_batch_midpoint_shapes(const sgb_batch* b, int32_t cap, int32_t* shapes, float* ms, int32_t* chosen) {
    if (!b) return SGB_ERR_ARG;
    const int n = (int)b->mid_shapes.size();
    for (int k = 0; k < n && k < cap; k++) {
        const MidShape& m = b->mid_shapes[k];
        if (shapes) {
            int32_t* r = shapes + 7 * k;
            r[0] = m.idx; r[1] = m.G; r[2] = m.bps; r[3] = m.grid; r[4] = (int32_t)m.smem;
            r[5] = m.kind;
            r[6] = m.kind ? (1 << m.lbx) | ((1 << m.lby) << 8) | ((1 << m.lbz) << 16) | ((m.nt / 32) << 24) : 0;
        }
        if (ms) ms[k] = m.ms;
    }
    if (chosen) *chosen = b->mid_choice;
    return n;
}

int sgb_batch_langevin_shapes(const sgb_batch* b, float* ms3, int32_t* chosen_bps) {
    if (!b) return SGB_ERR_ARG;
    if (ms3)
        for (int k = 0; k < 3; k++) ms3[k] = b->heun_ms[k];
    if (chosen_bps) *chosen_bps = b->heun_bps;
    return 3;
}

int sgb_batch_set_midpoint_first_accept(sgb_batch* b, int32_t on) {
    if (!b) return bfail(nullptr, SGB_ERR_ARG, "null handle");
    b->mid_accept0 = on ? 1 : 0;
    return SGB_OK;
}

int sgb_batch_set_midpoint_chunk(sgb_batch* b, int32_t replicas) {
    if (!b) return bfail(nullptr, SGB_ERR_ARG, "null handle");
    if (replicas < 0 || replicas > 64) return bfail(b, SGB_ERR_ARG, "replicas per midpoint launch must be in [0, 64] (0: sized for L2)");
    b->mid_chunk = replicas;
    return SGB_OK;
}

int sgb_batch_select_midpoint_shape(sgb_batch* b, int32_t row) {
    if (!b) return SGB_ERR_ARG;
    if (row < -1 || row >= (int)b->mid_shapes.size()) {
        b->err = "no such midpoint launch shape (run a batched add_sample first)";
        return SGB_ERR_ARG;
    }
    b->mid_choice = row;
    return SGB_OK;
}

int sgb_batch_set_wait_limit(sgb_batch* b, double seconds) {
    if (!b) return SGB_ERR_ARG;
    if (!(seconds >= 0) || seconds > 3600) {
        b->err = "wait limit must be in [0, 3600] s (0: the 4 s default)";
        return SGB_ERR_ARG;
    }
    if (!b->grp.empty()) {
        for (sgb_system* s : b->grp) {
            const int rc = sgb_set_wait_limit(s, seconds);
            if (rc) return bfail(b, rc, s->err);
        }
        return SGB_OK;
    }
    const unsigned long long ns = (unsigned long long)(seconds * 1e9);
    BCK(cudaMemcpyAsync(&b->ctrl->wait_ns, &ns, sizeof(ns), cudaMemcpyHostToDevice, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    return SGB_OK;
}

int sgb_batch_event_record(sgb_batch* b, int32_t slot) {
    if (!b || slot < 0 || slot >= 8) return bfail(b, SGB_ERR_ARG, "bad event slot");
    BCK(cudaEventRecord(b->ev[slot], b->stream));
    return SGB_OK;
}

int sgb_batch_event_elapsed(sgb_batch* b, int32_t a, int32_t c, float* ms) {
    if (!b || !ms || a < 0 || a >= 8 || c < 0 || c >= 8) return bfail(b, SGB_ERR_ARG, "bad event slot");
    BCK(cudaEventSynchronize(b->ev[c]));
    BCK(cudaEventElapsedTime(ms, b->ev[a], b->ev[c]));
    return SGB_OK;
}

int64_t sgb_batch_kernel_launches(const sgb_batch* b) {
    if (!b) return 0;
    int64_t n = b->launches;
    for (const sgb_system* s : b->grp) n += s->launches;
    return n;
}

}  // extern "C"
