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

namespace {

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
                      int nrep, size_t rep_stride, cudaStream_t st) {
    if (ncorr * npos * npos > 8 * 256) return SGB_ERR_ARG;   // at most 8 accumulator entries per thread and row
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

template int corr_launch_accum<float>(const float*, double*, const int*, int, int, int, int, int, int, size_t, cudaStream_t);
template int corr_launch_accum<double>(const double*, double*, const int*, int, int, int, int, int, int, size_t, cudaStream_t);
