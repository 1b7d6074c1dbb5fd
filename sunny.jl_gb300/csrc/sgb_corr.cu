// sgb_corr.cu -- SampledCorrelations accumulation kernels for sm_103a.
//
// Reference: src/SampledCorrelations/CorrelationSampling.jl:48-139 (accum_sample!) and
// src/SampledCorrelations/SampledCorrelations.jl:128-142 (merge_correlations).
//
// Sunny computes, per sample and per (c, i, j):
//     C(q, ω) = FFT_t[ w(t)/n(t) * IFFT_t[ conj(A_αi(q, ω)) A_βj(q, ω) ] ]
// and folds C into a running mean. Every operation after the product is linear and
// identical for every sample, so the mean of C equals the same transform applied to the
// mean of the products. The library therefore streams only
//     P(c,i,j,q,ω) += conj(A_αi(q,ω)) A_βj(q,ω)          (FP64 sum, one pass per sample)
// over the accumulator, which makes add_sample! a single coalesced read+write of the
// accumulator, and applies IFFT -> window/n(t) -> FFT once, when the data are read.
//
// Layouts:
//   sample spectra  A[n_all_omega][nobs][npos][ncell]  complex R
//   accumulator     P[n_all_omega][ncell][npos(j)][npos(i)][ncorr]  complex double
//                   (identical to Sunny's column-major data[c, i, j, q1, q2, q3, ω])
#include "sgb_corr.h"
#include <cufft.h>
#include <stdint.h>

namespace {

// ---- bulk-copy (TMA) primitives: 1-D cp.async.bulk with mbarrier completion ---------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* m, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(m)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t* m, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(m)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* m) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(m)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* m, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(m)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// wait for phase `parity` of m to complete; false after a 2 s limit
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* m, uint32_t parity) {
    if (mbar_try_wait(m, parity)) return true;
    const uint64_t t0 = globaltimer_ns();
    while (!mbar_try_wait(m, parity))
        if (globaltimer_ns() - t0 > 2000000000ull) return false;
    return true;
}
// global -> shared, completion counted on mbarrier m (bytes: multiple of 16, 16-byte aligned)
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* m) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(m))
                 : "memory");
}
// shared -> global, tracked by bulk groups
__device__ __forceinline__ void bulk_store(void* dst, const void* src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_u32(src)), "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
__device__ __forceinline__ void bulk_wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

template <class R> struct C2 { R x, y; };

// One CTA handles one ω and QT consecutive wave vectors: it stages the QT x nobs x npos
// complex spectra of every replica in shared memory and then streams the contiguous
// QT*B accumulator entries (B = ncorr*npos*npos), coalesced, with streaming cache hints.
// With nrep replicas the products of all of them are summed before the single FP64
// read-modify-write, so the accumulator traffic per sample falls as 1/nrep.
template <class R, int QT>
__global__ void __launch_bounds__(256) k_corr_accum(const R* __restrict__ A, double* __restrict__ P,
                                                  const int* __restrict__ pairs, int ncorr, int nobs, int npos,
                                                  int ncell, int nomega, int nrep, size_t rep_stride) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int nrow = nobs * npos;
    // Shared layout [rep][ql][obs][pos], each observable block padded by one element: the
    // threads of a warp read different (obs, pos) at one ql, which then fall in distinct
    // banks instead of a 256-byte stride on one bank.
    const int rowpad = nobs * (npos + 1);
    C2<R>* As = reinterpret_cast<C2<R>*>(smem_raw);          // [nrep][QT][rowpad]
    int* pr = reinterpret_cast<int*>(As + (size_t)nrep * QT * rowpad);
    const int w = blockIdx.y;
    const int q0 = blockIdx.x * QT;
    const int nq = min(QT, ncell - q0);
    for (int e = threadIdx.x; e < nrep * nrow * QT; e += blockDim.x) {
        int r = e / (nrow * QT), rem = e - r * nrow * QT;
        int row = rem / QT, ql = rem % QT;
        C2<R> v = {0, 0};
        if (ql < nq) {
            size_t idx = (size_t)r * rep_stride + ((size_t)w * nrow + row) * ncell + q0 + ql;
            v.x = A[2 * idx];
            v.y = A[2 * idx + 1];
        }
        const int o = row / npos, p = row - o * npos;
        As[((size_t)r * QT + ql) * rowpad + o * (npos + 1) + p] = v;
    }
    for (int e = threadIdx.x; e < 2 * ncorr; e += blockDim.x) pr[e] = pairs[e];
    __syncthreads();
    const int B = ncorr * npos * npos;
    const size_t base = ((size_t)w * ncell + q0) * B;
    double2* out = reinterpret_cast<double2*>(P) + base;
    // Element (ql, r) of the tile is out[ql*B + r] with r = c + ncorr*(i + npos*j). A thread
    // owns the r values threadIdx.x + k*blockDim.x for every ql, so their shared-memory
    // offsets are computed once, outside the streaming loop (no divisions per element).
    constexpr int KMAX = 8;
    int ia[KMAX], ib[KMAX];
    const int nk = (B + blockDim.x - 1) / blockDim.x;
#pragma unroll
    for (int k = 0; k < KMAX; k++) {
        int r = threadIdx.x + k * blockDim.x;
        ia[k] = -1; ib[k] = -1;
        if (k < nk && r < B) {
            int c = r % ncorr, t = r / ncorr;
            int i = t % npos, j = t / npos;
            ia[k] = pr[2 * c] * (npos + 1) + i;
            ib[k] = pr[2 * c + 1] * (npos + 1) + j;
        }
    }
    for (int ql = 0; ql < nq; ql++) {
        double2* row = out + (size_t)ql * B;
        double2 acc[KMAX];
#pragma unroll
        for (int k = 0; k < KMAX; k++)
            if (ia[k] >= 0) acc[k] = __ldcs(row + threadIdx.x + k * blockDim.x);
#pragma unroll
        for (int k = 0; k < KMAX; k++) {
            if (ia[k] < 0) continue;
            R sre = 0, sim = 0;
            for (int rr = 0; rr < nrep; rr++) {
                const C2<R>* Ar = As + ((size_t)rr * QT + ql) * rowpad;
                C2<R> a = Ar[ia[k]];
                C2<R> b = Ar[ib[k]];
                // conj(a) * b
                sre += a.x * b.x + a.y * b.y;
                sim += a.x * b.y - a.y * b.x;
            }
            acc[k].x += (double)sre;
            acc[k].y += (double)sim;
            __stcs(row + threadIdx.x + k * blockDim.x, acc[k]);
        }
    }
}

// The same accumulation with the accumulator rows moved by bulk copies, warp-specialised.
// A CTA owns one ω and QT consecutive wave vectors: one contiguous block of QT rows of B
// complex doubles. Warp NCW (the producer) streams the rows through a ring of NST
// shared-memory buffers with bulk loads (mbarrier `full`) and writes each finished row
// back with a bulk store once the NCW compute warps have released it (mbarrier `done`);
// the compute warps add the replicas' products in shared memory and never wait for a
// store. Every wait is bounded (2 s): on expiry the CTA records err = 1 and stops.
// conj(a) b added to (re, im)
template <class R>
__device__ __forceinline__ void cmul_conj_acc(const C2<R>& a, const C2<R>& b, R& re, R& im) {
    re += a.x * b.x + a.y * b.y;
    im += a.x * b.y - a.y * b.x;
}

template <class R, int QT, int NST>
__global__ void __launch_bounds__(288) k_corr_accum_bulk(const R* __restrict__ A, double* __restrict__ P,
                                                       const int* __restrict__ pairs, int ncorr, int nobs, int npos,
                                                       int ncell, int nomega, int nrep, size_t rep_stride,
                                                       int* __restrict__ err) {
    constexpr int NCW = 8;   // compute warps
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int B = ncorr * npos * npos;
    const uint32_t rowbytes = (uint32_t)B * 16u;
    double2* rows = reinterpret_cast<double2*>(smem_raw);                       // [NST][B]
    uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw + (size_t)NST * rowbytes);
    uint64_t* done = full + NST;
    constexpr int MBYTES = (16 * NST + 15) / 16 * 16;
    const int nrow = nobs * npos;
    const int rowpad = nobs * (npos + 1);
    C2<R>* As = reinterpret_cast<C2<R>*>(smem_raw + (size_t)NST * rowbytes + MBYTES);   // [nrep][QT][rowpad]
    int* pr = reinterpret_cast<int*>(As + (size_t)nrep * QT * rowpad);
    __shared__ int bad;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int w = blockIdx.y;
    const int q0 = blockIdx.x * QT;
    const int nq = min(QT, ncell - q0);
    double2* out = reinterpret_cast<double2*>(P) + ((size_t)w * ncell + q0) * B;
    if (warp == NCW && lane == 0) {
        bad = 0;
        for (int s = 0; s < NST; s++) { mbar_init(&full[s], 1); mbar_init(&done[s], NCW); }
        mbar_fence_init();
        for (int s = 0; s < NST && s < nq; s++) {
            mbar_expect_tx(&full[s], rowbytes);
            bulk_load(rows + (size_t)s * B, out + (size_t)s * B, rowbytes, &full[s]);
        }
    }
    for (int e = threadIdx.x; e < nrep * nrow * QT; e += blockDim.x) {
        int r = e / (nrow * QT), rem = e - r * nrow * QT;
        int row = rem / QT, ql = rem % QT;
        C2<R> v = {0, 0};
        if (ql < nq) {
            size_t idx = (size_t)r * rep_stride + ((size_t)w * nrow + row) * ncell + q0 + ql;
            v.x = A[2 * idx];
            v.y = A[2 * idx + 1];
        }
        const int o = row / npos, p = row - o * npos;
        As[((size_t)r * QT + ql) * rowpad + o * (npos + 1) + p] = v;
    }
    for (int e = threadIdx.x; e < 2 * ncorr; e += blockDim.x) pr[e] = pairs[e];
    __syncthreads();
    if (warp == NCW) {
        // producer: store finished rows, refill their buffers
        if (lane == 0) {
            for (int ql = 0; ql < nq; ql++) {
                const int s = ql % NST;
                if (!mbar_wait_bounded(&done[s], (uint32_t)((ql / NST) & 1))) { bad = 1; break; }
                bulk_store(out + (size_t)ql * B, rows + (size_t)s * B, rowbytes);
                if (ql + NST < nq) {
                    bulk_wait_read_all();   // the store has read the buffer
                    mbar_expect_tx(&full[s], rowbytes);
                    bulk_load(rows + (size_t)s * B, out + (size_t)(ql + NST) * B, rowbytes, &full[s]);
                }
            }
            bulk_wait_all();
            if (bad) atomicExch(err, 1);
        }
        return;
    }
    constexpr int KMAX = 8;
    int ia[KMAX], ib[KMAX];
    const int nthr = NCW * 32;
    const int nk = (B + nthr - 1) / nthr;
#pragma unroll
    for (int k = 0; k < KMAX; k++) {
        int r = threadIdx.x + k * nthr;
        ia[k] = -1; ib[k] = -1;
        if (k < nk && r < B) {
            int c = r % ncorr, t = r / ncorr;
            int i = t % npos, j = t / npos;
            ia[k] = pr[2 * c] * (npos + 1) + i;
            ib[k] = pr[2 * c + 1] * (npos + 1) + j;
        }
    }
    // Three observables with the canonical six pairs (every ssf_* measure): a thread owns
    // whole (i, j) sublattice pairs, loads the 3 + 3 spectra of a replica once and forms
    // the six products from them, half the shared-memory loads of one entry per thread.
    const bool canon = nobs == 3 && ncorr == 6 && pr[0] == 2 && pr[1] == 2 && pr[2] == 1 && pr[3] == 2 &&
                       pr[4] == 0 && pr[5] == 2 && pr[6] == 1 && pr[7] == 1 && pr[8] == 0 && pr[9] == 1 &&
                       pr[10] == 0 && pr[11] == 0;
    for (int ql = 0; ql < nq; ql++) {
        const int s = ql % NST;
        if (!mbar_wait_bounded(&full[s], (uint32_t)((ql / NST) & 1))) { bad = 1; break; }
        if (bad) break;
        double2* row = rows + (size_t)s * B;
        if (canon) {
            for (int pidx = threadIdx.x; pidx < npos * npos; pidx += nthr) {
                const int i = pidx % npos, j = pidx / npos;
                R tr[6], ti[6];
#pragma unroll
                for (int c = 0; c < 6; c++) { tr[c] = 0; ti[c] = 0; }
                for (int rr = 0; rr < nrep; rr++) {
                    const C2<R>* Ar = As + ((size_t)rr * QT + ql) * rowpad;
                    const C2<R> a0 = Ar[i], a1 = Ar[(npos + 1) + i], a2 = Ar[2 * (npos + 1) + i];
                    const C2<R> b0 = Ar[j], b1 = Ar[(npos + 1) + j], b2 = Ar[2 * (npos + 1) + j];
                    cmul_conj_acc(a2, b2, tr[0], ti[0]);
                    cmul_conj_acc(a1, b2, tr[1], ti[1]);
                    cmul_conj_acc(a0, b2, tr[2], ti[2]);
                    cmul_conj_acc(a1, b1, tr[3], ti[3]);
                    cmul_conj_acc(a0, b1, tr[4], ti[4]);
                    cmul_conj_acc(a0, b0, tr[5], ti[5]);
                }
                double2* e = row + (size_t)6 * pidx;
#pragma unroll
                for (int c = 0; c < 6; c++) {
                    double2 acc = e[c];
                    acc.x += (double)tr[c];
                    acc.y += (double)ti[c];
                    e[c] = acc;
                }
            }
            fence_proxy_async();
            __syncwarp();
            if (lane == 0) mbar_arrive(&done[s]);
            continue;
        }
#pragma unroll
        for (int k = 0; k < KMAX; k++) {
            if (ia[k] < 0) continue;
            R sre = 0, sim = 0;
            for (int rr = 0; rr < nrep; rr++) {
                const C2<R>* Ar = As + ((size_t)rr * QT + ql) * rowpad;
                C2<R> a = Ar[ia[k]];
                C2<R> b = Ar[ib[k]];
                sre += a.x * b.x + a.y * b.y;
                sim += a.x * b.y - a.y * b.x;
            }
            double2 acc = row[threadIdx.x + k * nthr];
            acc.x += (double)sre;
            acc.y += (double)sim;
            row[threadIdx.x + k * nthr] = acc;
        }
        fence_proxy_async();   // the generic-proxy writes become visible to the bulk store
        __syncwarp();
        if (lane == 0) mbar_arrive(&done[s]);
    }
}

// Gather `ncol` accumulator columns (stride `ld` along ω) starting at column col0 into
// tmp[ncol][n] and scale by 1/nsamples.
__global__ void k_gather_cols(const double2* __restrict__ P, size_t ld, size_t col0, int ncol, int n, double scale,
                              double2* __restrict__ tmp) {
    size_t total = (size_t)ncol * n;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        int w = (int)(e / ncol), c = (int)(e % ncol);
        double2 v = P[(size_t)w * ld + col0 + c];
        v.x *= scale; v.y *= scale;
        tmp[(size_t)c * n + w] = v;
    }
}

// tmp[c][t] *= g[t]   (g = window(t) / n_contrib(t) / n, CorrelationSampling.jl:74-107)
__global__ void k_apply_window(double2* tmp, int ncol, int n, const double* __restrict__ g) {
    size_t total = (size_t)ncol * n;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        double s = g[e % n];
        tmp[e].x *= s;
        tmp[e].y *= s;
    }
}

// Transpose tmp[ncol][n] back to out[n][ncol] (ω-major, as Sunny's data layout).
__global__ void k_scatter_cols(const double2* __restrict__ tmp, int ncol, int n, double2* __restrict__ out) {
    size_t total = (size_t)ncol * n;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        int w = (int)(e / ncol), c = (int)(e % ncol);
        out[e] = tmp[(size_t)c * n + w];
    }
}

__global__ void k_add_inplace(double* __restrict__ dst, const double* __restrict__ src, size_t n) {
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
        dst[e] += src[e];
}

// Per-sample products of columns [col0, col0 + ncol) of one replica's spectra, in the
// read-out layout tmp[col - col0][ω] (col = c + ncorr (i + npos (j + npos q))):
//     conj(A_{α,i}(q, ω)) A_{β,j}(q, ω).
template <class R>
__global__ void k_product_cols(const R* __restrict__ A, const int* __restrict__ pairs, int ncorr, int nobs, int npos,
                               int ncell, int n, size_t col0, int ncol, double2* __restrict__ tmp) {
    const size_t total = (size_t)ncol * n;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int w = (int)(e % n);
        const size_t col = col0 + e / n;
        const int c = (int)(col % ncorr);
        size_t t = col / ncorr;
        const int i = (int)(t % npos);
        t /= npos;
        const int j = (int)(t % npos);
        const int q = (int)(t / npos);
        const size_t ia = (((size_t)w * nobs + pairs[2 * c]) * npos + i) * ncell + q;
        const size_t ib = (((size_t)w * nobs + pairs[2 * c + 1]) * npos + j) * ncell + q;
        const double ax = A[2 * ia], ay = A[2 * ia + 1], bx = A[2 * ib], by = A[2 * ib + 1];
        tmp[e] = make_double2(ax * bx + ay * by, ax * by - ay * bx);
    }
}

// Welford update of the running mean and M with one transformed sample x (read-out
// layout, columns [col0, col0 + ncol)), CorrelationSampling.jl:117-134:
//   μ_old = mean; mean += (x - mean) / count; M += Re((x - μ_old) conj(x - mean)).
// mean and M use Sunny's layout, index ω * ld + col.
__global__ void k_welford_cols(const double2* __restrict__ tmp, int ncol, int n, size_t col0, size_t ld, double count,
                               double2* __restrict__ mean, double* __restrict__ M) {
    const size_t total = (size_t)ncol * n;
    const double inv = 1.0 / count;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int w = (int)(e / ncol), cl = (int)(e % ncol);
        const double2 x = tmp[(size_t)cl * n + w];
        const size_t idx = (size_t)w * ld + col0 + cl;
        const double2 m0 = mean[idx];
        const double2 m1 = make_double2(m0.x + (x.x - m0.x) * inv, m0.y + (x.y - m0.y) * inv);
        mean[idx] = m1;
        const double dx0 = x.x - m0.x, dy0 = x.y - m0.y, dx1 = x.x - m1.x, dy1 = x.y - m1.y;
        M[idx] += dx0 * dx1 + dy0 * dy1;
    }
}

// merge_correlations with errors (SampledCorrelations.jl:128-142):
//   μ = n/(n+m) d1 + m/(n+m) d2; M1 = (M1 + n|μ - d1|²) + (M2 + m|μ - d2|²); d1 = μ.
__global__ void k_merge_welford(double2* __restrict__ d1, double* __restrict__ M1, const double2* __restrict__ d2,
                                const double* __restrict__ M2, double n, double m, size_t len) {
    const double a = n / (n + m), b = m / (n + m);
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < len; e += (size_t)gridDim.x * blockDim.x) {
        const double2 x = d1[e], y = d2[e];
        const double2 mu = make_double2(a * x.x + b * y.x, a * x.y + b * y.y);
        const double ex = mu.x - x.x, ey = mu.y - x.y, fx = mu.x - y.x, fy = mu.y - y.y;
        M1[e] = (M1[e] + n * (ex * ex + ey * ey)) + (M2[e] + m * (fx * fx + fy * fy));
        d1[e] = mu;
    }
}

// Statistical comparison of two calculate_errors accumulators of one layout. Per bin k,
// Δ = μa − μb and s = Ma/(na(na−1)) + Mb/(nb(nb−1)), the variance of Δ if both means
// estimate one S(q,ω). Each block writes 7 FP64 partial sums: Σ|Δ|², Σs, Σs², Σ|μb|²,
// Σ|μa|², #(|Δ|² > 9s), #(s > 0). Launched with 256 threads.
__global__ void k_compare_welford(const double2* __restrict__ ma, const double* __restrict__ Ma,
                                  const double2* __restrict__ mb, const double* __restrict__ Mb, double fa, double fb,
                                  size_t len, double* __restrict__ part) {
    double acc[7] = {0, 0, 0, 0, 0, 0, 0};
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < len; e += (size_t)gridDim.x * blockDim.x) {
        const double2 x = ma[e], y = mb[e];
        const double dx = x.x - y.x, dy = x.y - y.y;
        const double d2 = dx * dx + dy * dy;
        const double sv = fa * Ma[e] + fb * Mb[e];
        acc[0] += d2;
        acc[1] += sv;
        acc[2] += sv * sv;
        acc[3] += y.x * y.x + y.y * y.y;
        acc[4] += x.x * x.x + x.y * x.y;
        acc[5] += d2 > 9.0 * sv ? 1.0 : 0.0;
        acc[6] += sv > 0.0 ? 1.0 : 0.0;
    }
    __shared__ double red[8][7];
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < 7; k++) {
        double v = acc[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (l == 0) red[w][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < 7) {
        double t = 0;
        for (int q = 0; q < 8; q++) t += red[q][threadIdx.x];
        part[(size_t)blockIdx.x * 7 + threadIdx.x] = t;
    }
}

// Cross term of two independent paired differences, bin by bin: Δ1 = a1 − b1 and Δ2 = a2 − b2
// from disjoint sets of paired samples have independent noise, so E[Re Δ1·conj(Δ2)] is the
// squared systematic difference alone. Each block writes 2 partial sums: Σ Re Δ1·conj(Δ2)
// and Σ|(b1 + b2)/2|². Launched with 256 threads.
__global__ void k_cross_diff(const double2* __restrict__ a1, const double2* __restrict__ b1, const double2* __restrict__ a2,
                             const double2* __restrict__ b2, size_t len, double* __restrict__ part) {
    double acc0 = 0, acc1 = 0;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < len; e += (size_t)gridDim.x * blockDim.x) {
        const double2 x1 = a1[e], y1 = b1[e], x2 = a2[e], y2 = b2[e];
        const double d1x = x1.x - y1.x, d1y = x1.y - y1.y, d2x = x2.x - y2.x, d2y = x2.y - y2.y;
        acc0 += d1x * d2x + d1y * d2y;
        const double mx = 0.5 * (y1.x + y2.x), my = 0.5 * (y1.y + y2.y);
        acc1 += mx * mx + my * my;
    }
    __shared__ double red[8][2];
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        acc0 += __shfl_down_sync(0xffffffffu, acc0, o);
        acc1 += __shfl_down_sync(0xffffffffu, acc1, o);
    }
    if (l == 0) { red[w][0] = acc0; red[w][1] = acc1; }
    __syncthreads();
    if (threadIdx.x < 2) {
        double t = 0;
        for (int q = 0; q < 8; q++) t += red[q][threadIdx.x];
        part[(size_t)blockIdx.x * 2 + threadIdx.x] = t;
    }
}

// Columns of the accumulator belonging to the wave vectors qidx[0..nq): the B = ncorr*npos^2
// columns of wave vector q are [q*B, (q+1)*B). tmp[k*B + b][ω] = scale * P[ω][qidx[k]*B + b].
__global__ void k_gather_qcols(const double2* __restrict__ P, size_t ld, const int* __restrict__ qidx, int nq, int B,
                               int n, double scale, double2* __restrict__ tmp) {
    const size_t total = (size_t)nq * B * n;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int w = (int)(e % n);
        const size_t col = e / n;
        const int k = (int)(col / B), b = (int)(col % B);
        double2 v = P[(size_t)w * ld + (size_t)qidx[k] * B + b];
        v.x *= scale; v.y *= scale;
        tmp[e] = v;
    }
}

// Phase averaging and the S(q,ω) combiner (DataRetrieval.jl:147-171, PhaseAveraging.jl):
// elems[c] = Σ_{i,j} p_i conj(p_j) data[c,i,j,q,ω] with p_i = ff_i(|q|) exp(-2πi q·r_i);
// combiner 0 = trace of the 3x3 correlation matrix, 1 = its component perpendicular to q
// (ssf_trace / ssf_perp, MeasureSpec.jl:115-224, corr_pairs (3,3),(2,3),(1,3),(2,2),(1,2),(1,1)),
// 2 = the ncorr raw elements. One CTA per wave vector, threads over the requested ω.
__global__ void k_intensity(const double2* __restrict__ tmp, int ncorr, int npos, int n, const double2* __restrict__ pref,
                            const double* __restrict__ qcart, const int* __restrict__ widx, int nw, int combiner,
                            double* __restrict__ out) {
    const int k = blockIdx.x;
    const int B = ncorr * npos * npos;
    const double2* col0 = tmp + (size_t)k * B * n;
    const double2* p = pref + (size_t)k * npos;
    for (int t = threadIdx.x; t < nw; t += blockDim.x) {
        const int w = widx[t];
        double er[8], ei[8];
        for (int c = 0; c < ncorr && c < 8; c++) { er[c] = 0; ei[c] = 0; }
        for (int j = 0; j < npos; j++) {
            const double2 pj = p[j];
            for (int i = 0; i < npos; i++) {
                const double2 pi = p[i];
                // f = p_i conj(p_j)
                const double fr = pi.x * pj.x + pi.y * pj.y, fi = pi.y * pj.x - pi.x * pj.y;
                for (int c = 0; c < ncorr && c < 8; c++) {
                    const double2 d = col0[(size_t)(c + ncorr * (i + npos * j)) * n + w];
                    er[c] += fr * d.x - fi * d.y;
                    ei[c] += fr * d.y + fi * d.x;
                }
            }
        }
        if (combiner == 2) {
            for (int c = 0; c < ncorr; c++) {
                out[(((size_t)k * nw + t) * ncorr + c) * 2] = er[c];
                out[(((size_t)k * nw + t) * ncorr + c) * 2 + 1] = ei[c];
            }
            continue;
        }
        // real 3x3 matrix from (3,3),(2,3),(1,3),(2,2),(1,2),(1,1): m11 = e5, m12 = e4, m13 = e2,
        // m22 = e3, m23 = e1, m33 = e0 (real parts; the matrix is Hermitian)
        const double tr = er[5] + er[3] + er[0];
        double v = tr;
        if (combiner == 1) {
            const double qx = qcart[3 * k], qy = qcart[3 * k + 1], qz = qcart[3 * k + 2];
            const double q2 = qx * qx + qy * qy + qz * qz;
            if (q2 == 0.0) {
                v = (2.0 / 3.0) * tr;
            } else {
                const double qmq = qx * qx * er[5] + qy * qy * er[3] + qz * qz * er[0] + 2 * qx * qy * er[4] +
                                   2 * qx * qz * er[2] + 2 * qy * qz * er[1];
                v = tr - qmq / q2;
            }
        }
        out[(size_t)k * nw + t] = v;
    }
}

int grid_for(size_t n) {
    size_t g = (n + 255) / 256;
    if (g > 65535) g = 65535;
    if (g < 1) g = 1;
    return (int)g;
}

}  // namespace

int corr_launch_compare_welford(const double* ma, const double* Ma, const double* mb, const double* Mb, double fa, double fb,
                                size_t len, double* part, cudaStream_t st) {
    k_compare_welford<<<SGB_CMP_BLOCKS, 256, 0, st>>>(reinterpret_cast<const double2*>(ma), Ma,
                                                       reinterpret_cast<const double2*>(mb), Mb, fa, fb, len, part);
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

int corr_launch_cross_diff(const double* a1, const double* b1, const double* a2, const double* b2, size_t len, double* part,
                           cudaStream_t st) {
    k_cross_diff<<<SGB_CMP_BLOCKS, 256, 0, st>>>(reinterpret_cast<const double2*>(a1), reinterpret_cast<const double2*>(b1),
                                                  reinterpret_cast<const double2*>(a2), reinterpret_cast<const double2*>(b2), len,
                                                  part);
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

int corr_launch_gather_q(const double* P, size_t ld, const int* qidx, int nq, int B, int n, double scale, double* tmp,
                         cudaStream_t st) {
    k_gather_qcols<<<grid_for((size_t)nq * B * n), 256, 0, st>>>(reinterpret_cast<const double2*>(P), ld, qidx, nq, B, n,
                                                                  scale, reinterpret_cast<double2*>(tmp));
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

int corr_launch_intensity(const double* tmp, int ncorr, int npos, int n, const double* pref, const double* qcart,
                          const int* widx, int nw, int combiner, int nq, double* out, cudaStream_t st) {
    if (ncorr > 8) return SGB_ERR_ARG;
    k_intensity<<<nq, 128, 0, st>>>(reinterpret_cast<const double2*>(tmp), ncorr, npos, n,
                                     reinterpret_cast<const double2*>(pref), qcart, widx, nw, combiner, out);
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

template <class R>
int corr_launch_product(const R* A, const int* pairs, int ncorr, int nobs, int npos, int ncell, int n, size_t col0,
                        int ncol, double* tmp, cudaStream_t st) {
    k_product_cols<R><<<grid_for((size_t)ncol * n), 256, 0, st>>>(A, pairs, ncorr, nobs, npos, ncell, n, col0, ncol,
                                                                   reinterpret_cast<double2*>(tmp));
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}
template int corr_launch_product<float>(const float*, const int*, int, int, int, int, int, size_t, int, double*, cudaStream_t);
template int corr_launch_product<double>(const double*, const int*, int, int, int, int, int, size_t, int, double*, cudaStream_t);

int corr_launch_welford(const double* tmp, int ncol, int n, size_t col0, size_t ld, double count, double* mean, double* M,
                        cudaStream_t st) {
    k_welford_cols<<<grid_for((size_t)ncol * n), 256, 0, st>>>(reinterpret_cast<const double2*>(tmp), ncol, n, col0, ld,
                                                                count, reinterpret_cast<double2*>(mean), M);
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

int corr_launch_merge_welford(double* d1, double* M1, const double* d2, const double* M2, double n, double m, size_t len,
                              cudaStream_t st) {
    k_merge_welford<<<grid_for(len), 256, 0, st>>>(reinterpret_cast<double2*>(d1), M1, reinterpret_cast<const double2*>(d2),
                                                   M2, n, m, len);
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

template <class R, int QT, int NST>
static int accum_bulk(const R* A, double* P, const int* pairs, int ncorr, int nobs, int npos, int ncell, int nomega,
                      int nrep, size_t rep_stride, int* err, cudaStream_t st) {
    const size_t B = (size_t)ncorr * npos * npos;
    const size_t smem = (size_t)NST * B * 16 + (16 * NST + 15) / 16 * 16 +
                        (size_t)nrep * nobs * (npos + 1) * QT * sizeof(C2<R>) + 2 * ncorr * sizeof(int) + 16;
    if (smem > 220 * 1024) return SGB_ERR_ARG;
    if (cudaFuncSetAttribute(k_corr_accum_bulk<R, QT, NST>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return SGB_ERR_CUDA;
    dim3 grid((ncell + QT - 1) / QT, nomega);
    k_corr_accum_bulk<R, QT, NST><<<grid, 288, smem, st>>>(A, P, pairs, ncorr, nobs, npos, ncell, nomega, nrep, rep_stride, err);
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

template <class R, int QT>
static int accum_qt(const R* A, double* P, const int* pairs, int ncorr, int nobs, int npos, int ncell, int nomega,
                    int nrep, size_t rep_stride, size_t smem, cudaStream_t st) {
    if (smem > 48 * 1024) {
        if (cudaFuncSetAttribute(k_corr_accum<R, QT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
            return SGB_ERR_CUDA;
    }
    dim3 grid((ncell + QT - 1) / QT, nomega);
    k_corr_accum<R, QT><<<grid, 256, smem, st>>>(A, P, pairs, ncorr, nobs, npos, ncell, nomega, nrep, rep_stride);
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

// The q tile shrinks (32 -> 16 -> 8 wave vectors per CTA) when many replicas' spectra
// would not fit in shared memory.
template <class R>
int corr_launch_accum(const R* A, double* P, const int* pairs, int ncorr, int nobs, int npos, int ncell, int nomega,
                      int nrep, size_t rep_stride, cudaStream_t st, int variant, int* err) {
    if (ncorr * npos * npos > 8 * 256) return SGB_ERR_ARG;   // at most 8 accumulator entries per thread and row
    if (variant > 0 && err) {
        // 8 wave vectors per CTA and a 2-row ring: 2-3 CTAs per SM (measured fastest of
        // tiles 4/8/16 x rings 2/3/4 on the 16^3 x 16 pyrochlore with 8 replicas)
        const int rc = accum_bulk<R, 8, 2>(A, P, pairs, ncorr, nobs, npos, ncell, nomega, nrep, rep_stride, err, st);
        if (rc != SGB_ERR_ARG) return rc;
    }
    auto bytes = [&](int qt) { return (size_t)nrep * nobs * (npos + 1) * qt * sizeof(C2<R>) + 2 * ncorr * sizeof(int) + 16; };
    const size_t lim = 200 * 1024;
    if (bytes(32) <= lim) return accum_qt<R, 32>(A, P, pairs, ncorr, nobs, npos, ncell, nomega, nrep, rep_stride, bytes(32), st);
    if (bytes(16) <= lim) return accum_qt<R, 16>(A, P, pairs, ncorr, nobs, npos, ncell, nomega, nrep, rep_stride, bytes(16), st);
    if (bytes(8) <= lim) return accum_qt<R, 8>(A, P, pairs, ncorr, nobs, npos, ncell, nomega, nrep, rep_stride, bytes(8), st);
    return SGB_ERR_ARG;
}

int corr_launch_gather(const double* P, size_t ld, size_t col0, int ncol, int n, double scale, double* tmp, cudaStream_t st) {
    k_gather_cols<<<grid_for((size_t)ncol * n), 256, 0, st>>>(reinterpret_cast<const double2*>(P), ld, col0, ncol, n,
                                                                scale, reinterpret_cast<double2*>(tmp));
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

int corr_launch_window(double* tmp, int ncol, int n, const double* g, cudaStream_t st) {
    k_apply_window<<<grid_for((size_t)ncol * n), 256, 0, st>>>(reinterpret_cast<double2*>(tmp), ncol, n, g);
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

int corr_launch_scatter(const double* tmp, int ncol, int n, double* out, cudaStream_t st) {
    k_scatter_cols<<<grid_for((size_t)ncol * n), 256, 0, st>>>(reinterpret_cast<const double2*>(tmp), ncol, n,
                                                                 reinterpret_cast<double2*>(out));
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

int corr_launch_add(double* dst, const double* src, size_t n, cudaStream_t st) {
    k_add_inplace<<<grid_for(n), 256, 0, st>>>(dst, src, n);
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

template int corr_launch_accum<float>(const float*, double*, const int*, int, int, int, int, int, int, size_t, cudaStream_t,
                                      int, int*);
template int corr_launch_accum<double>(const double*, double*, const int*, int, int, int, int, int, int, size_t,
                                       cudaStream_t, int, int*);
