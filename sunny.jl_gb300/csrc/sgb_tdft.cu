// sgb_tdft.cu -- the time transform of add_sample! (CorrelationSampling.jl:65-69) for FP32
// accumulators: the FFT along time of every (observable, position, cell) series of every
// replica, n = n_all_ω points of which the first m = n/2 + 1 are snapshots and the rest
// zero padding (CorrelationSampling.jl:36-39), into the spectrum buffer.
//
// n = 2(nω − 1) is rarely a product of small primes (398 = 2·199 for nω = 200), so the
// transform is Bluestein's chirp z-transform (Bluestein 1970; Rabiner, Schafer & Rader
// 1969). With w_j = exp(−πi j²/n), jk = (j² + k² − (k−j)²)/2 gives
//   X_k = Σ_{t<m} x_t e^{−2πi tk/n} = w_k Σ_{t<m} (x_t w_t) conj(w_{k−t}),
// a linear convolution of the m weighted samples with the chirp conj(w_j), j in
// [−(m−1), n−1], computed cyclically with length M = 1024 ≥ n + m − 1 as
// IFFT(FFT(a) · FFT(b)). FFT(b)/M is precomputed on the host in FP64 (rounded to FP32 once),
// as is the chirp (its phase reduced exactly as j² mod 2n).
//
// One warp transforms one series; its 1024 points are 32 per lane in registers. Each
// 1024-point FFT is the four-step factorisation 1024 = 32 × 32: 32-point DFTs in registers
// (radix-2 decimation in frequency, output order fixed by register renaming at compile
// time), the twiddles exp(∓2πi·lane·k/1024) from a shared table laid out [k][lane] (conflict
// free), a transpose through the warp's shared 32 × 33 tile (padded against bank
// conflicts), and 32-point DFTs again. The zero padding is never loaded and only the
// n wanted outputs are stored. A CTA of 8 warps takes 8 adjacent series of one replica;
// its samples come in and its spectra go out through shared memory row by row, so each
// warp-wide load or store moves 4 time rows of 64 contiguous bytes. Since n + m − 1 <= 1024
// bounds m by 342, only registers j <= 10 of the first DFT hold samples; its first stage
// is written for that.
#include <cuda_runtime.h>

#include <cmath>
#include <complex>
#include <vector>

#include "sgb_common.cuh"
#include "sgb_corr.h"

namespace {

constexpr int TD_M = 1024;
constexpr int TD_WARPS = 8;

// exp(−2πi k/32), k = 0..15, set by the host (FP64 values rounded once)
__constant__ float2 c_w32[16];

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ float2 cmulcf(float2 a, float2 b) {   // a · conj(b)
    return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}

__host__ __device__ constexpr int bitrev5(int k) {
    return ((k & 1) << 4) | ((k & 2) << 2) | (k & 4) | ((k & 8) >> 2) | ((k & 16) >> 4);
}

// In-register 32-point DFT, X_k = Σ_j v_j exp(∓2πi jk/32) (INV: +), radix-2 decimation in
// frequency; the result is left in bit-reversed register order (X_k in v[bitrev5(k)]).
template <bool INV>
__device__ __forceinline__ void dft32_dif(float2* v) {
#pragma unroll
    for (int half = 16; half >= 1; half >>= 1) {
#pragma unroll
        for (int blk = 0; blk < 32; blk += 2 * half) {
#pragma unroll
            for (int i = 0; i < half; i++) {
                const float2 a = v[blk + i], b = v[blk + i + half];
                v[blk + i] = make_float2(a.x + b.x, a.y + b.y);
                const float2 d = make_float2(a.x - b.x, a.y - b.y);
                const int e = i * (16 / half);   // twiddle exp(∓2πi e/32)
                if (e == 0) {
                    v[blk + i + half] = d;
                } else if (e == 8) {             // ∓i
                    v[blk + i + half] = INV ? make_float2(-d.y, d.x) : make_float2(d.y, -d.x);
                } else {
                    v[blk + i + half] = INV ? cmulcf(d, c_w32[e]) : cmulf(d, c_w32[e]);
                }
            }
        }
    }
}

// The first DFT of the forward transform, whose registers j >= 11 are zero: its first
// stage (pairs j, j + 16) reduces to v[j + 16] = v[j] w^j.
__device__ __forceinline__ void dft32_dif_first(float2* v) {
#pragma unroll
    for (int i = 0; i < 16; i++) {
        const float2 a = v[i];
        v[i + 16] = i == 0 ? a : (i == 8 ? make_float2(a.y, -a.x) : cmulf(a, c_w32[i]));
    }
#pragma unroll
    for (int half = 8; half >= 1; half >>= 1) {
#pragma unroll
        for (int blk = 0; blk < 32; blk += 2 * half) {
#pragma unroll
            for (int i = 0; i < half; i++) {
                const float2 a = v[blk + i], b = v[blk + i + half];
                v[blk + i] = make_float2(a.x + b.x, a.y + b.y);
                const float2 d = make_float2(a.x - b.x, a.y - b.y);
                const int e = i * (16 / half);
                v[blk + i + half] = e == 0 ? d : (e == 8 ? make_float2(d.y, -d.x) : cmulf(d, c_w32[e]));
            }
        }
    }
}

constexpr int TD_JMAX = 11;            // registers that can hold samples (m <= 342)
constexpr int TD_ROWS_IN = 32 * TD_JMAX;
constexpr int TD_LD = TD_WARPS + 1;    // staging row stride: lanes 32 rows apart hit distinct banks

__global__ void __launch_bounds__(32 * TD_WARPS, 2)
k_time_dft(const float2* __restrict__ A, float2* __restrict__ Ahat, long long ncols, long long stride, long long rep_stride,
           int n, int m, const float2* __restrict__ chirp, const float2* __restrict__ fb, const float2* __restrict__ tw) {
    __shared__ float2 s_tw[TD_M];                  // [k][lane] = exp(−2πi lane k / 1024)
    __shared__ float2 s_t[TD_WARPS][32 * 33];      // per-warp transpose tile
    __shared__ float2 s_io[TD_ROWS_IN * TD_LD];    // staged samples [t][series], later spectra [k][series]
    for (int i = threadIdx.x; i < TD_M; i += blockDim.x) s_tw[i] = tw[i];
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    const long long col0 = (long long)blockIdx.x * TD_WARPS;
    const long long col = col0 + wp;
    // the CTA's series are adjacent in memory when all eight lie in one replica
    const bool rowwise = col0 + TD_WARPS <= ncols && (col0 / stride) == ((col0 + TD_WARPS - 1) / stride);
    const long long base0 = (col0 / stride) * rep_stride + (col0 % stride);
    if (rowwise) {
        for (int e = threadIdx.x; e < m * TD_WARPS; e += blockDim.x) {
            const int t = e / TD_WARPS, c = e % TD_WARPS;
            s_io[t * TD_LD + c] = __ldg(A + base0 + (long long)t * stride + c);
        }
    }
    __syncthreads();
    if (col >= ncols) return;
    const long long base = (col / stride) * rep_stride + (col % stride);
    float2* T = s_t[wp];
    float2 v[32];
    // a_t = x_t w_t at t = 32 j + lane (zero beyond the snapshots)
#pragma unroll
    for (int j = 0; j < 32; j++) {
        const int t = 32 * j + lane;
        if (j < TD_JMAX && t < m)
            v[j] = cmulf(rowwise ? s_io[t * TD_LD + wp] : __ldg(A + base + (long long)t * stride), __ldg(chirp + t));
        else v[j] = make_float2(0.f, 0.f);
    }
    // forward FFT: DFT over j (index 32 j + lane), twiddle exp(−2πi lane k1/1024), transpose,
    // DFT over the former lanes; lane then holds frequency lane + 32 k2 in v[bitrev5(k2)]
    dft32_dif_first(v);
#pragma unroll
    for (int k1 = 0; k1 < 32; k1++) T[lane * 33 + k1] = cmulf(v[bitrev5(k1)], s_tw[k1 * 32 + lane]);
    __syncwarp();
#pragma unroll
    for (int j2 = 0; j2 < 32; j2++) v[j2] = T[j2 * 33 + lane];
    __syncwarp();
    dft32_dif<false>(v);
    // multiply by FFT(b)/M at frequency lane + 32 k2
#pragma unroll
    for (int k2 = 0; k2 < 32; k2++) v[bitrev5(k2)] = cmulf(v[bitrev5(k2)], __ldg(fb + lane + 32 * k2));
    // inverse FFT from index lane + 32 k2: DFT over k2, twiddle exp(+2πi lane j1/1024),
    // transpose, DFT over the former lanes; lane then holds point lane + 32 j2 in v[bitrev5(j2)]
    {
        float2 u[32];
#pragma unroll
        for (int k2 = 0; k2 < 32; k2++) u[k2] = v[bitrev5(k2)];
        dft32_dif<true>(u);
#pragma unroll
        for (int j1 = 0; j1 < 32; j1++) T[lane * 33 + j1] = cmulcf(u[bitrev5(j1)], s_tw[j1 * 32 + lane]);
    }
    __syncwarp();
#pragma unroll
    for (int k1 = 0; k1 < 32; k1++) v[k1] = T[k1 * 33 + lane];
    dft32_dif<true>(v);
    // X_k = w_k y_k for the n wanted points
    if (!rowwise) {
#pragma unroll
        for (int j2 = 0; j2 < 32; j2++) {
            const int k = lane + 32 * j2;
            if (k < n) Ahat[base + (long long)k * stride] = cmulf(v[bitrev5(j2)], __ldg(chirp + k));
        }
        return;
    }
    // row-wise stores in two halves of the spectrum through the staging buffer (its
    // samples were consumed before the first transpose)
    __syncthreads();
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int k0 = h * TD_ROWS_IN, k1 = min(n, k0 + TD_ROWS_IN);
#pragma unroll
        for (int j2 = 0; j2 < 32; j2++) {
            const int k = lane + 32 * j2;
            if (k >= k0 && k < k1) s_io[(k - k0) * TD_LD + wp] = cmulf(v[bitrev5(j2)], __ldg(chirp + k));
        }
        __syncthreads();
        for (int e = threadIdx.x; e < (k1 - k0) * TD_WARPS; e += blockDim.x) {
            const int k = k0 + e / TD_WARPS, c = e % TD_WARPS;
            Ahat[base0 + (long long)k * stride + c] = s_io[(k - k0) * TD_LD + c];
        }
        __syncthreads();
    }
}

}  // namespace

// The fixed 1024-point convolution pays off when the linear convolution needs more than
// 512 points; shorter series stay with cuFFT.
bool tdft_supported(int n, int m) {
    return n >= 2 && m >= 1 && n + m - 1 > TD_M / 2 && n + m - 1 <= TD_M && m <= TD_ROWS_IN && n <= 2 * TD_ROWS_IN;
}

// Tables of one transform length: chirp[max(n, m)], FFT(b)/M [1024], twiddles [1024].
int tdft_tables(int n, int m, void** chirp_out, void** fb_out, void** tw_out) {
    if (!tdft_supported(n, m)) return SGB_ERR_ARG;
    typedef std::complex<double> cd;
    const double pi = 3.14159265358979323846;
    const int nc = n > m ? n : m;
    std::vector<cd> w(nc);
    for (int j = 0; j < nc; j++) {
        const long long r = ((long long)j * j) % (2LL * n);   // exp(−πi j²/n) depends on j² mod 2n
        w[j] = std::polar(1.0, -pi * (double)r / n);
    }
    std::vector<cd> b(TD_M, cd(0, 0));
    for (int j = 0; j < n; j++) b[j] = std::conj(w[j]);
    for (int j = 1; j < m; j++) b[TD_M - j] = std::conj(w[j]);
    std::vector<float2> fb(TD_M), chirp(nc), tw(TD_M);
    std::vector<cd> root(TD_M);   // exp(−2πi r/M)
    for (int r = 0; r < TD_M; r++) root[r] = std::polar(1.0, -2 * pi * (double)r / TD_M);
    for (int k = 0; k < TD_M; k++) {   // direct FP64 DFT of b, scaled by 1/M
        cd acc(0, 0);
        for (int j = 0; j < TD_M; j++) acc += b[j] * root[(j * k) % TD_M];
        acc /= (double)TD_M;
        fb[k] = make_float2((float)acc.real(), (float)acc.imag());
    }
    for (int j = 0; j < nc; j++) chirp[j] = make_float2((float)w[j].real(), (float)w[j].imag());
    for (int k = 0; k < 32; k++)
        for (int l = 0; l < 32; l++) {
            const cd z = std::polar(1.0, -2 * pi * (double)(l * k) / TD_M);
            tw[k * 32 + l] = make_float2((float)z.real(), (float)z.imag());
        }
    float2 w32[16];
    for (int k = 0; k < 16; k++) {
        const cd z = std::polar(1.0, -2 * pi * k / 32.0);
        w32[k] = make_float2((float)z.real(), (float)z.imag());
    }
    if (cudaMemcpyToSymbol(c_w32, w32, sizeof(w32)) != cudaSuccess) return SGB_ERR_CUDA;
    void *dc = nullptr, *df = nullptr, *dt = nullptr;
    if (cudaMalloc(&dc, sizeof(float2) * nc) != cudaSuccess || cudaMalloc(&df, sizeof(float2) * TD_M) != cudaSuccess ||
        cudaMalloc(&dt, sizeof(float2) * TD_M) != cudaSuccess) {
        cudaFree(dc); cudaFree(df); cudaFree(dt);
        return SGB_ERR_NOMEM;
    }
    cudaMemcpy(dc, chirp.data(), sizeof(float2) * nc, cudaMemcpyHostToDevice);
    cudaMemcpy(df, fb.data(), sizeof(float2) * TD_M, cudaMemcpyHostToDevice);
    cudaMemcpy(dt, tw.data(), sizeof(float2) * TD_M, cudaMemcpyHostToDevice);
    *chirp_out = dc;
    *fb_out = df;
    *tw_out = dt;
    return SGB_OK;
}

int tdft_launch(const float* A, float* Ahat, long long ncols, long long stride, long long rep_stride, int n, int m,
                const void* chirp, const void* fb, const void* tw, cudaStream_t st) {
    const long long grid = (ncols + TD_WARPS - 1) / TD_WARPS;
    if (grid < 1 || grid > 0x7fffffffLL) return SGB_ERR_ARG;
    k_time_dft<<<(unsigned)grid, 32 * TD_WARPS, 0, st>>>(reinterpret_cast<const float2*>(A), reinterpret_cast<float2*>(Ahat), ncols,
                                                         stride, rep_stride, n, m, reinterpret_cast<const float2*>(chirp),
                                                         reinterpret_cast<const float2*>(fb), reinterpret_cast<const float2*>(tw));
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}
