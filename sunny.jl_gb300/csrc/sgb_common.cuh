// sgb_common.cuh -- device-side building blocks shared by the sm_103a kernels of
// libsunnygb300: precision traits, the coupling tables staged in shared memory, the
// bounded inter-CTA barrier used by the persistent kernels, and the Philox-4x32-10
// counter-based Gaussian source for Langevin noise.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>
#include <cuda/atomic>
#include "../../include/sunny_gb300.h"

#define SGB_MAX_SUBLAT 64
#define SGB_MAX_N 5

// ---------------------------------------------------------------------------------
// Coupling tables. One DBond is a directed bond seen from its first atom; the library
// stores both directions of every Sunny PairCoupling so that the gradient is a gather
// (each site sums over its own bond list), which equals Sunny's scatter over non-culled
// bonds (src/System/Interactions.jl:554-591).
// ---------------------------------------------------------------------------------
template <class R>
struct DBond {
    R J[9];          // column-major 3x3 (already transposed for reverse copies)
    R scalar;        // constant shift (energy only)
    R bq;            // isotropic biquadratic strength (kind 1)
    int j;           // target atom
    int n[3];        // cell offset, reduced mod dims into [0, L) for single systems
    int jkind;       // 0: J = J[0] * identity, 1: full 3x3
    int bqkind;      // 0 none, 1 isotropic, 2 matrix (index bqidx)
    int bqidx;       // row in the 5x5 biquadratic table
    int fwd;         // 1 for the non-culled copy (counted in the energy)
    int pk;          // raw offsets and target packed as bytes: (n0+128) | (n1+128)<<8 | (n2+128)<<16 | j<<24
    int gref;        // SU(N) general terms: first row in the general-term table | rows << 20 (0: none)
};

// First row and number of rows of a bond's SU(N) general terms (DBond::gref).
template <class B>
__host__ __device__ __forceinline__ int dbond_gidx(const B& b) { return b.gref & 0xfffff; }
template <class B>
__host__ __device__ __forceinline__ int dbond_gcnt(const B& b) { return (int)((unsigned)b.gref >> 20); }

// Sunny's scalar_biquad_metric (src/System/Types.jl:40)
__host__ __device__ inline double biquad_metric(int q) {
    return q == 0 ? 0.5 : q == 1 ? 2.0 : q == 2 ? (1.0 / 6.0) : q == 3 ? 2.0 : 0.5;
}

// ---------------------------------------------------------------------------------
// Status word and bounded waits. Every wait has a wall-clock limit read from
// %globaltimer; on expiry the kernel records SGB_ERR_TIMEOUT and returns, so that a
// stuck barrier never hangs the GPU.
// ---------------------------------------------------------------------------------
// Control words of one persistent launch. The barrier word, the convergence sums and
// the status live on separate 128-byte lines so that spinning, atomics and flag reads
// do not contend for one L2 line.
//
// The barrier word packs an arrival count (bits 0-31), a generation (bits 32-62) and an
// abort flag (bit 63) that sgb_set_status raises, so that an arrival returns its place in
// the episode and a waiter sees an error in the word it polls: no extra loads on the
// barrier's critical path. The last arrival of an episode folds nblocks counts into one
// generation; arrivals so far = generation * nblocks + count is unchanged by the fold.
#define SGB_BAR_GEN 0x100000000ull
#define SGB_BAR_ABORT 0x8000000000000000ull
struct alignas(128) Ctrl {
    unsigned long long bar;
    unsigned int pad0[30];
    unsigned int pad1[32];
    double acc[3];       // rotating FP64 convergence accumulators
    double pad2[13];
    int status;
    int steps_done;
    long long iters;
    int final_buf;
    int pad3[27];
    // Wall-clock limit of every bounded wait of the launch, in ns (0: SGB_BARRIER_TIMEOUT_NS).
    // It sits after the words that each launch clears (sgb_ctrl_clear_bytes), so a limit set
    // on a handle (sgb_set_wait_limit) holds for all of its later launches.
    unsigned long long wait_ns;
    unsigned long long pad4[15];
};

// Bytes of Ctrl that are zeroed before a launch: everything up to the wait limit.
constexpr size_t sgb_ctrl_clear_bytes() { return offsetof(Ctrl, wait_ns); }

__device__ __forceinline__ uint64_t sgb_globaltimer() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void sgb_set_status(Ctrl* c, int code) {
    atomicCAS(&c->status, 0, code);
    __threadfence();
    atomicOr(&c->bar, SGB_BAR_ABORT);   // waiters at a barrier leave at once
}

__device__ __forceinline__ int sgb_read_status(Ctrl* c) {
    return cuda::atomic_ref<int, cuda::thread_scope_device>(c->status).load(cuda::memory_order_relaxed);
}

// Default limit of a bounded wait (4 s).
#define SGB_BARRIER_TIMEOUT_NS 4000000000ull

__device__ __forceinline__ uint64_t sgb_wait_limit(const Ctrl* c) {
    const unsigned long long w = *(volatile const unsigned long long*)&c->wait_ns;
    return w ? w : SGB_BARRIER_TIMEOUT_NS;
}

// Barrier across `nblocks` co-resident CTAs (cooperative launch guarantees residency).
// Memory written before the barrier by any CTA is visible to plain loads of every CTA
// after it: each CTA's bar.sync orders its writes before its leader's release arrival,
// and a waiter's acquire fence follows its last read of the word.
// A waiter leaves once the arrivals reach the end of its episode, so the last arrival's
// own add releases everyone and its fold of the count travels behind it, off the
// critical path. At the start of a launch the count field is zero (every episode of an
// earlier launch has folded, and launches clear the word), so the arrivals so far are a
// multiple of any nblocks.
// Returns false if the wait timed out or some CTA raised an error (sgb_set_status).
__device__ __forceinline__ bool sgb_grid_barrier(Ctrl* c, unsigned int nblocks) {
    __shared__ int ok_s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        if (nblocks > 1) {
            cuda::atomic_ref<unsigned long long, cuda::thread_scope_device> bar(c->bar);
            const unsigned long long prev = bar.fetch_add(1ull, cuda::memory_order_acq_rel);
            if (prev & SGB_BAR_ABORT) {
                ok = 0;
            } else {
                // the count is below 2 * nblocks: at or above nblocks, the previous
                // episode's fold has not landed yet and this arrival opens the next one
                const unsigned long long gen = (prev >> 32) & 0x7fffffffull;
                const unsigned int cnt = (unsigned int)prev;
                const bool late = cnt >= nblocks;
                const unsigned int pos = late ? cnt - nblocks : cnt;
                const unsigned long long target = (gen + (late ? 2ull : 1ull)) * nblocks;
                if (pos == nblocks - 1) {
                    bar.fetch_add(SGB_BAR_GEN - nblocks, cuda::memory_order_relaxed);
                } else {
                    uint64_t t0 = 0, lim = 0;
                    unsigned int spins = 0;
                    for (;;) {
                        const unsigned long long now = bar.load(cuda::memory_order_relaxed);
                        if (now & SGB_BAR_ABORT) {
                            ok = 0;
                            break;
                        }
                        if (((now >> 32) & 0x7fffffffull) * nblocks + (unsigned int)now >= target) break;
                        if ((++spins & 255u) == 0) {
                            uint64_t t = sgb_globaltimer();
                            if (t0 == 0) {
                                t0 = t;
                                lim = sgb_wait_limit(c);
                            } else if (t - t0 > lim) {
                                sgb_set_status(c, SGB_ERR_TIMEOUT);
                                ok = 0;
                                break;
                            }
                        }
                    }
                    cuda::atomic_thread_fence(cuda::memory_order_acquire, cuda::thread_scope_device);
                }
            }
        } else if (cuda::atomic_ref<unsigned long long, cuda::thread_scope_device>(c->bar).load(
                       cuda::memory_order_relaxed) & SGB_BAR_ABORT) {
            ok = 0;
        }
        ok_s = ok;
    }
    __syncthreads();
    return ok_s != 0;
}

// ---------------------------------------------------------------------------------
// Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) and Box-Muller.
// ---------------------------------------------------------------------------------
struct Philox4 { uint32_t x, y, z, w; };

__host__ __device__ inline uint32_t sgb_mulhi32(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
    return __umulhi(a, b);
#else
    return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}

__host__ __device__ inline Philox4 sgb_philox(Philox4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
        uint32_t hi0 = sgb_mulhi32(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        uint32_t hi1 = sgb_mulhi32(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
        Philox4 n;
        n.x = hi1 ^ c.y ^ k0;
        n.y = lo1;
        n.z = hi0 ^ c.w ^ k1;
        n.w = lo0;
        c = n;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

// Four standard normals for (seed, stream, step, site, block of 4 components).
template <class R>
__device__ inline void sgb_normals4(uint64_t seed, uint32_t stream, uint64_t step, uint32_t site,
                                    uint32_t blk, R out[4]) {
    Philox4 c;
    c.x = site;
    c.y = (uint32_t)step;
    c.z = (uint32_t)(step >> 32) ^ (blk << 24);
    c.w = stream;
    Philox4 r = sgb_philox(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    if constexpr (sizeof(R) == 8) {
        const double s = 2.3283064365386963e-10;  // 2^-32
        double u1 = ((double)r.x + 1.0) * s, u2 = (double)r.y * s;
        double u3 = ((double)r.z + 1.0) * s, u4 = (double)r.w * s;
        double a = sqrt(-2.0 * log(u1)), b = sqrt(-2.0 * log(u3));
        double s1, c1, s2, c2;
        sincospi(2.0 * u2, &s1, &c1);
        sincospi(2.0 * u4, &s2, &c2);
        out[0] = a * c1; out[1] = a * s1; out[2] = b * c2; out[3] = b * s2;
    } else {
        const float s = 2.3283064365386963e-10f;
        float u1 = ((float)r.x + 1.0f) * s, u2 = (float)r.y * s;
        float u3 = ((float)r.z + 1.0f) * s, u4 = (float)r.w * s;
        u1 = fminf(u1, 1.0f); u3 = fminf(u3, 1.0f);
        float a = sqrtf(-2.0f * logf(u1)), b = sqrtf(-2.0f * logf(u3));
        float s1, c1, s2, c2;
        sincospif(2.0f * u2, &s1, &c1);
        sincospif(2.0f * u4, &s2, &c2);
        out[0] = a * c1; out[1] = a * s1; out[2] = b * c2; out[3] = b * s2;
    }
}

// Four uniforms in (0, 1) for the LocalSampler's Metropolis draws of (seed, sweep, site),
// on a Philox stream of their own.
#define SGB_MC_STREAM 0x80000001u
__device__ inline void sgb_mc_uniforms4(uint64_t seed, uint64_t sweep, uint32_t site, double u[4]) {
    Philox4 c;
    c.x = site;
    c.y = (uint32_t)sweep;
    c.z = (uint32_t)(sweep >> 32) ^ (1u << 24);
    c.w = SGB_MC_STREAM;
    Philox4 r = sgb_philox(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    const double s = 2.3283064365386963e-10;   // 2^-32
    u[0] = ((double)r.x + 0.5) * s;
    u[1] = ((double)r.y + 0.5) * s;
    u[2] = ((double)r.z + 0.5) * s;
    u[3] = ((double)r.w + 0.5) * s;
}

// ---------------------------------------------------------------------------------
// Small helpers
// ---------------------------------------------------------------------------------
// Loads of state that other CTAs wrote before the last grid barrier: plain (L1-cacheable)
// loads, made coherent by the barrier's fences. Never the read-only (.nc) path.
template <class R> __device__ __forceinline__ R sgb_ld(const R* p) { return *p; }

template <class R> __device__ __forceinline__ R sgb_rsqrt(R x);
template <> __device__ __forceinline__ float sgb_rsqrt<float>(float x) { return rsqrtf(x); }
template <> __device__ __forceinline__ double sgb_rsqrt<double>(double x) { return 1.0 / sqrt(x); }

template <class R> __device__ __forceinline__ R sgb_sqrt(R x);
template <> __device__ __forceinline__ float sgb_sqrt<float>(float x) { return sqrtf(x); }
template <> __device__ __forceinline__ double sgb_sqrt<double>(double x) { return sqrt(x); }

// wrap x = c + n with c in [0, L) and n already reduced into [0, L)
__device__ __forceinline__ int sgb_wrap_pos(int x, int L) { return x >= L ? x - L : x; }
// wrap for |n| <= L (replica batches, where n is not pre-reduced)
__device__ __forceinline__ int sgb_wrap_any(int x, int L) {
    x = x < 0 ? x + L : x;
    return x >= L ? x - L : x;
}

// block-wide FP64 sum (any blockDim up to 1024); result valid in thread 0
__device__ inline double sgb_block_sum(double v) {
    __shared__ double red[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    const int nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x < 32) {
        r = threadIdx.x < nw ? red[threadIdx.x] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
    }
    return r;
}

// Block-wide sum of per-thread terms given in the working precision R: warps reduce in R
// (32 terms), the per-warp partials are summed in FP64. Result valid in thread 0.
template <class R>
__device__ inline double sgb_block_sum_r(R v) {
    __shared__ double redr[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    const int nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if (l == 0) redr[w] = (double)v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0)
        for (int k = 0; k < nw; k++) r += redr[k];
    return r;
}
