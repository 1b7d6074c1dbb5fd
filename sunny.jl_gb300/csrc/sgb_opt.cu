// sgb_opt.cu -- device vector kernels of minimize_energy! (dipole modes, FP64).
//
// Reference algorithm (Sunny.jl v0.9.2): src/Optimization.jl:31-166 -- nonlinear
// conjugate gradient on the product of unit spheres (retraction x -> x/|x|, gradient and
// direction projected onto the tangent space), gradient scaled by |S| = κ, convergence on
// the largest gradient component (g_abstol) or the largest step component (x_abstol).
// The optimiser itself (Optim.jl's ConjugateGradient with a Hager-Zhang line search) is
// a third-party dependency; the host side in sgb_api.cu restates its published method.
//
// Layout: unit spins x, projected gradient g and direction d are FP64 SoA [3][ns]; the
// spin state S of the system is refreshed as κ·x before every energy/gradient call.
// Reductions: each kernel writes per-block partials [block][K] that the host adds in a
// fixed order (sums) or maximises.
#include <algorithm>

#include "sgb_internal.h"

#include "sgb_device.cuh"

namespace {
using namespace sgbdev;

constexpr int kOptGrid = 256;

__device__ inline void block_reduce_store(double* part, int K, const double* v, const bool* is_max) {
    __shared__ double red[32][10];
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = (blockDim.x + 31) >> 5;
    for (int k = 0; k < K; k++) {
        double a = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            double b = __shfl_down_sync(0xffffffffu, a, o);
            a = is_max[k] ? fmax(a, b) : a + b;
        }
        if (l == 0) red[w][k] = a;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 0; k < K; k++) {
            double a = 0.0;   // maxima are of absolute values
            for (int q = 0; q < nw; q++) a = is_max[k] ? fmax(a, red[q][k]) : a + red[q][k];
            part[blockIdx.x * K + k] = a;
        }
    }
}

// Tangent projection at the unit point u: real (dipoles) g - u (u·g), or complex (kets)
// g - u (uᴴ g), which also removes the phase direction as Optimization.jl:49-57 does.
template <int K, bool CPLX>
__device__ __forceinline__ void project(const double* u, double* g) {
    if (!CPLX) {
        double c = 0;
#pragma unroll
        for (int q = 0; q < K; q++) c += u[q] * g[q];
#pragma unroll
        for (int q = 0; q < K; q++) g[q] -= u[q] * c;
    } else {
        double cr = 0, ci = 0;
#pragma unroll
        for (int q = 0; q < K / 2; q++) {
            cr += u[2 * q] * g[2 * q] + u[2 * q + 1] * g[2 * q + 1];
            ci += u[2 * q] * g[2 * q + 1] - u[2 * q + 1] * g[2 * q];
        }
#pragma unroll
        for (int q = 0; q < K / 2; q++) {
            const double ur = u[2 * q], ui = u[2 * q + 1];
            g[2 * q] -= ur * cr - ui * ci;
            g[2 * q + 1] -= ur * ci + ui * cr;
        }
    }
}

// Gradient of E with respect to the unit variables: κ ∇E for dipoles; 2 √κ HZ for kets,
// the real gradient of E(√κ u) in R^2N (HZ = dE/dZ̄), so that φ' = Σ G·d / |x + α d|.
template <bool CPLX>
__device__ __forceinline__ double grad_scale(double kappa) { return CPLX ? 2.0 * sqrt(kappa) : kappa; }

// perturb_spins! (System.jl:519-524; perturbed_spin :454-468) with Philox normals, then
// x = normalize(S), or (1, 1, ...)/√K' for a vacancy (Optimization.jl:115-117). The state
// is SoA [K][ns]: dipoles (K = 3) or kets as (re, im) (K = 2N, normals of E|ξ|² = 1).
template <int K, bool CPLX>
__global__ void k_opt_init(double* S, const double* kappa, int ns, double jitter, uint64_t seed, double* x) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
        double v[K];
#pragma unroll
        for (int q = 0; q < K; q++) v[q] = S[(size_t)q * ns + i];
        const double k = kappa[i];
        const double amp = CPLX ? sqrt(k) : k;
        if (jitter != 0.0) {
            double g[12];
#pragma unroll
            for (int blk = 0; blk < (K + 3) / 4; blk++) sgb_normals4<double>(seed, 0x80000002u, 0, (uint32_t)i, (uint32_t)blk, g + 4 * blk);
            double n2 = 0;
#pragma unroll
            for (int q = 0; q < K; q++) {
                v[q] += jitter * amp * g[q] * (CPLX ? 0.70710678118654752 : 1.0);
                n2 += v[q] * v[q];
            }
            const double f = k == 0.0 ? 0.0 : amp / sqrt(n2);
#pragma unroll
            for (int q = 0; q < K; q++) { v[q] *= f; S[(size_t)q * ns + i] = v[q]; }
        }
        double n2 = 0;
#pragma unroll
        for (int q = 0; q < K; q++) n2 += v[q] * v[q];
        if (n2 == 0.0) {
            const double r = 1.0 / sqrt((double)(CPLX ? K / 2 : K));
#pragma unroll
            for (int q = 0; q < K; q++) x[(size_t)q * ns + i] = (CPLX && (q & 1)) ? 0.0 : r;
        } else {
            const double f = 1.0 / sqrt(n2);
#pragma unroll
            for (int q = 0; q < K; q++) x[(size_t)q * ns + i] = v[q] * f;
        }
    }
}

// state = amp·normalize(x + α d), amp = κ (dipole) or √κ (ket) (retraction, then
// set_dipole! / set_coherent!)
template <int K, bool CPLX>
__global__ void k_opt_point(const double* x, const double* d, double alpha, const double* kappa, int ns, double* S) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
        double y[K], n2 = 0;
#pragma unroll
        for (int q = 0; q < K; q++) { y[q] = x[(size_t)q * ns + i] + alpha * d[(size_t)q * ns + i]; n2 += y[q] * y[q]; }
        const double f = (CPLX ? sqrt(kappa[i]) : kappa[i]) / sqrt(n2);
#pragma unroll
        for (int q = 0; q < K; q++) S[(size_t)q * ns + i] = y[q] * f;
    }
}

// φ'(α) = Σ_i G_i(α)·d_i / |x_i + α d_i| with G_i(α) the projected gradient at the
// retracted point (grad: AoS [ns][K]).
template <int K, bool CPLX>
__global__ void k_opt_dphi(const double* x, const double* d, double alpha, const double* grad, const double* kappa,
                           int ns, double* part) {
    double acc = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
        double u[K], g[K], n2 = 0;
#pragma unroll
        for (int q = 0; q < K; q++) { u[q] = x[(size_t)q * ns + i] + alpha * d[(size_t)q * ns + i]; n2 += u[q] * u[q]; }
        const double r = sqrt(n2);
        const double sc = grad_scale<CPLX>(kappa[i]);
#pragma unroll
        for (int q = 0; q < K; q++) { u[q] /= r; g[q] = sc * grad[(size_t)i * K + q]; }
        project<K, CPLX>(u, g);
        double t = 0;
#pragma unroll
        for (int q = 0; q < K; q++) t += g[q] * d[(size_t)q * ns + i];
        acc += t / r;
    }
    const bool mx[1] = {false};
    block_reduce_store(part, 1, &acc, mx);
}

// Accept the step: x <- normalize(x + α d); g <- projected gradient there; d <- d
// transported (projected onto the new tangent space); old g transported for y = g - g_old.
// Partials: [0] d·y [1] y·y [2] g·y [3] g·d [4] d·d [5] g_old·g_old [6] g·g
//           [7] max |g| component [8] max |Δx| component [9] Σ |G|² (unprojected)
template <int K, bool CPLX>
__global__ void k_opt_accept(double* x, double* d, double alpha, const double* grad, const double* kappa, int ns,
                             double* g, double* part) {
    double v[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
        double xo[K], dd[K], u[K], gn[K], go[K], n2 = 0;
#pragma unroll
        for (int q = 0; q < K; q++) {
            xo[q] = x[(size_t)q * ns + i];
            dd[q] = d[(size_t)q * ns + i];
            go[q] = g[(size_t)q * ns + i];
            u[q] = xo[q] + alpha * dd[q];
            n2 += u[q] * u[q];
        }
        const double r = sqrt(n2);
        const double sc = grad_scale<CPLX>(kappa[i]);
#pragma unroll
        for (int q = 0; q < K; q++) {
            u[q] /= r;
            gn[q] = sc * grad[(size_t)i * K + q];
            v[9] += gn[q] * gn[q];
            v[5] += go[q] * go[q];
        }
        project<K, CPLX>(u, gn);
        project<K, CPLX>(u, dd);
        project<K, CPLX>(u, go);
#pragma unroll
        for (int q = 0; q < K; q++) {
            const double yv = gn[q] - go[q];
            v[0] += dd[q] * yv;
            v[1] += yv * yv;
            v[2] += gn[q] * yv;
            v[3] += gn[q] * dd[q];
            v[4] += dd[q] * dd[q];
            v[6] += gn[q] * gn[q];
            v[7] = fmax(v[7], fabs(gn[q]));
            v[8] = fmax(v[8], fabs(u[q] - xo[q]));
            g[(size_t)q * ns + i] = gn[q];
            d[(size_t)q * ns + i] = dd[q];
            x[(size_t)q * ns + i] = u[q];
        }
    }
    const bool mx[10] = {false, false, false, false, false, false, false, true, true, false};
    block_reduce_store(part, 10, v, mx);
}

// d <- -g + β d over K·ns elements; partial [0] = g·d (the new φ'(0)), [1] = max |d|
__global__ void k_opt_dir(const double* g, double* d, double beta, long long n, double* part) {
    double v[2] = {0, 0};
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const double dn = -g[e] + beta * d[e];
        d[e] = dn;
        v[0] += g[e] * dn;
        v[1] = fmax(v[1], fabs(dn));
    }
    const bool mx[2] = {false, true};
    block_reduce_store(part, 2, v, mx);
}

int grid_for(int n) { return std::max(1, std::min(kOptGrid, (n + SGB_BLOCK - 1) / SGB_BLOCK)); }

}  // namespace

int opt_grid(int ns) { return grid_for(10 * ns); }

// K = 3 (dipoles) or 2N (kets, N = 2..5)
#define OPT_DISPATCH(KER, ...)                                                                  \
    switch (K) {                                                                                \
        case 3: KER<3, false><<<grid_for(10 * ns), SGB_BLOCK, 0, st>>>(__VA_ARGS__); break;     \
        case 4: KER<4, true><<<grid_for(10 * ns), SGB_BLOCK, 0, st>>>(__VA_ARGS__); break;      \
        case 6: KER<6, true><<<grid_for(10 * ns), SGB_BLOCK, 0, st>>>(__VA_ARGS__); break;      \
        case 8: KER<8, true><<<grid_for(10 * ns), SGB_BLOCK, 0, st>>>(__VA_ARGS__); break;      \
        case 10: KER<10, true><<<grid_for(10 * ns), SGB_BLOCK, 0, st>>>(__VA_ARGS__); break;    \
        default: return SGB_ERR_ARG;                                                            \
    }                                                                                           \
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;

int opt_launch_init(int K, double* S, const double* kappa, int ns, double jitter, uint64_t seed, double* x, cudaStream_t st) {
    OPT_DISPATCH(k_opt_init, S, kappa, ns, jitter, seed, x)
}
int opt_launch_point(int K, const double* x, const double* d, double alpha, const double* kappa, int ns, double* S,
                     cudaStream_t st) {
    OPT_DISPATCH(k_opt_point, x, d, alpha, kappa, ns, S)
}
int opt_launch_dphi(int K, const double* x, const double* d, double alpha, const double* grad, const double* kappa, int ns,
                    double* part, cudaStream_t st) {
    OPT_DISPATCH(k_opt_dphi, x, d, alpha, grad, kappa, ns, part)
}
int opt_launch_accept(int K, double* x, double* d, double alpha, const double* grad, const double* kappa, int ns, double* g,
                      double* part, cudaStream_t st) {
    OPT_DISPATCH(k_opt_accept, x, d, alpha, grad, kappa, ns, g, part)
}
int opt_launch_dir(int K, const double* g, double* d, double beta, int ns, double* part, cudaStream_t st) {
    k_opt_dir<<<grid_for(10 * ns), SGB_BLOCK, 0, st>>>(g, d, beta, (long long)K * ns, part);
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}
