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

// perturb_spins! (System.jl:519-524, perturbed_spin :454-460) with Philox normals, then
// x = normalize(S), or (1,1,1)/√3 for a vacancy (Optimization.jl:115-117).
__global__ void k_opt_init(double* S, const double* kappa, int ns, double jitter, uint64_t seed, double* x) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
        double sx = S[i], sy = S[ns + i], sz = S[2 * ns + i];
        const double k = kappa[i];
        if (jitter != 0.0) {
            double g[4];
            sgb_normals4<double>(seed, 0x80000002u, 0, (uint32_t)i, 0u, g);
            sx += jitter * k * g[0]; sy += jitter * k * g[1]; sz += jitter * k * g[2];
            normalize_dip<double>(sx, sy, sz, k);
            S[i] = sx; S[ns + i] = sy; S[2 * ns + i] = sz;
        }
        double n2 = sx * sx + sy * sy + sz * sz;
        if (n2 == 0.0) {
            const double r = 0.57735026918962576;   // 1/sqrt(3)
            x[i] = r; x[ns + i] = r; x[2 * ns + i] = r;
        } else {
            const double f = 1.0 / sqrt(n2);
            x[i] = sx * f; x[ns + i] = sy * f; x[2 * ns + i] = sz * f;
        }
    }
}

// S = κ·normalize(x + α d) (retraction, then set_dipole!)
__global__ void k_opt_point(const double* x, const double* d, double alpha, const double* kappa, int ns, double* S) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
        double yx = x[i] + alpha * d[i], yy = x[ns + i] + alpha * d[ns + i], yz = x[2 * ns + i] + alpha * d[2 * ns + i];
        const double f = kappa[i] / sqrt(yx * yx + yy * yy + yz * yz);
        S[i] = yx * f; S[ns + i] = yy * f; S[2 * ns + i] = yz * f;
    }
}

// φ'(α) = Σ_i g_i(α)·d_i / |x_i + α d_i| with g_i(α) the projected, κ-scaled gradient at
// the retracted point (grad: AoS [ns][3]).
__global__ void k_opt_dphi(const double* x, const double* d, double alpha, const double* grad, const double* kappa,
                           int ns, double* part) {
    double acc = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
        double yx = x[i] + alpha * d[i], yy = x[ns + i] + alpha * d[ns + i], yz = x[2 * ns + i] + alpha * d[2 * ns + i];
        const double r = sqrt(yx * yx + yy * yy + yz * yz);
        const double ux = yx / r, uy = yy / r, uz = yz / r;
        const double k = kappa[i];
        double gx = k * grad[3 * i], gy = k * grad[3 * i + 1], gz = k * grad[3 * i + 2];
        const double ug = ux * gx + uy * gy + uz * gz;
        gx -= ux * ug; gy -= uy * ug; gz -= uz * ug;
        acc += (gx * d[i] + gy * d[ns + i] + gz * d[2 * ns + i]) / r;
    }
    const bool mx[1] = {false};
    block_reduce_store(part, 1, &acc, mx);
}

// Accept the step: x <- normalize(x + α d); g <- projected gradient there; d <- d
// transported (projected onto the new tangent space); old g transported for y = g - g_old.
// Partials: [0] d·y [1] y·y [2] g·y [3] g·d [4] d·d [5] g_old·g_old [6] g·g
//           [7] max |g| component [8] max |Δx| component [9] Σ |κ ∇E|² (unprojected)
__global__ void k_opt_accept(double* x, double* d, double alpha, const double* grad, const double* kappa, int ns,
                             double* g, double* part) {
    double v[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
        double xo[3] = {x[i], x[ns + i], x[2 * ns + i]};
        double dd[3] = {d[i], d[ns + i], d[2 * ns + i]};
        double y[3] = {xo[0] + alpha * dd[0], xo[1] + alpha * dd[1], xo[2] + alpha * dd[2]};
        const double r = sqrt(y[0] * y[0] + y[1] * y[1] + y[2] * y[2]);
        double u[3] = {y[0] / r, y[1] / r, y[2] / r};
        const double k = kappa[i];
        double gk[3] = {k * grad[3 * i], k * grad[3 * i + 1], k * grad[3 * i + 2]};
        v[9] += gk[0] * gk[0] + gk[1] * gk[1] + gk[2] * gk[2];
        const double ug = u[0] * gk[0] + u[1] * gk[1] + u[2] * gk[2];
        const double ud = u[0] * dd[0] + u[1] * dd[1] + u[2] * dd[2];
        double go[3] = {g[i], g[ns + i], g[2 * ns + i]};
        const double uo = u[0] * go[0] + u[1] * go[1] + u[2] * go[2];
        v[5] += go[0] * go[0] + go[1] * go[1] + go[2] * go[2];
        for (int c = 0; c < 3; c++) {
            const double gn = gk[c] - u[c] * ug;
            const double dt = dd[c] - u[c] * ud;
            const double yv = gn - (go[c] - u[c] * uo);
            v[0] += dt * yv;
            v[1] += yv * yv;
            v[2] += gn * yv;
            v[3] += gn * dt;
            v[4] += dt * dt;
            v[6] += gn * gn;
            v[7] = fmax(v[7], fabs(gn));
            v[8] = fmax(v[8], fabs(u[c] - xo[c]));
            g[(size_t)c * ns + i] = gn;
            d[(size_t)c * ns + i] = dt;
            x[(size_t)c * ns + i] = u[c];
        }
    }
    const bool mx[10] = {false, false, false, false, false, false, false, true, true, false};
    block_reduce_store(part, 10, v, mx);
}

// d <- -g + β d; partial [0] = g·d (the new φ'(0)), [1] = max |d| component
__global__ void k_opt_dir(const double* g, double* d, double beta, int ns, double* part) {
    double v[2] = {0, 0};
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < 3 * ns; e += gridDim.x * blockDim.x) {
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

int opt_grid(int ns) { return grid_for(3 * ns); }

int opt_launch_init(double* S, const double* kappa, int ns, double jitter, uint64_t seed, double* x, cudaStream_t st) {
    k_opt_init<<<grid_for(3 * ns), SGB_BLOCK, 0, st>>>(S, kappa, ns, jitter, seed, x);
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}
int opt_launch_point(const double* x, const double* d, double alpha, const double* kappa, int ns, double* S,
                     cudaStream_t st) {
    k_opt_point<<<grid_for(3 * ns), SGB_BLOCK, 0, st>>>(x, d, alpha, kappa, ns, S);
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}
int opt_launch_dphi(const double* x, const double* d, double alpha, const double* grad, const double* kappa, int ns,
                    double* part, cudaStream_t st) {
    k_opt_dphi<<<grid_for(3 * ns), SGB_BLOCK, 0, st>>>(x, d, alpha, grad, kappa, ns, part);
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}
int opt_launch_accept(double* x, double* d, double alpha, const double* grad, const double* kappa, int ns, double* g,
                      double* part, cudaStream_t st) {
    k_opt_accept<<<grid_for(3 * ns), SGB_BLOCK, 0, st>>>(x, d, alpha, grad, kappa, ns, g, part);
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}
int opt_launch_dir(const double* g, double* d, double beta, int ns, double* part, cudaStream_t st) {
    k_opt_dir<<<grid_for(3 * ns), SGB_BLOCK, 0, st>>>(g, d, beta, ns, part);
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}
