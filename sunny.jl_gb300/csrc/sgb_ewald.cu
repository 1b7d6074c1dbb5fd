// sgb_ewald.cu -- long-range dipole-dipole interactions (Ewald summation) for sm_103a.
//
// Reference algorithm (Sunny.jl v0.9.2): src/System/Ewald.jl
//   precompute_dipole_ewald      :40-146  pair matrices A[offset, i, j] from real-space
//                                         and reciprocal sums (σ = V^(1/3)/3, 6√2 cut-offs)
//   ewald_energy                 :149-176 E = μ (A ⋆ μ) / 2 with μ = -g S
//   accum_ewald_grad!            :180-207 ∇E -= gᵀ ϕ, ϕ = A ⋆ μ by FFT over cells
//
// Design: the matrices are computed on the device, one thread per (offset cell, i, j),
// in FP64, and transformed once (cuFFT D2Z over the cell grid, one batch member per
// matrix element and atom pair). A gradient evaluation is four launches: μ = -g S into a
// [atom][component][cell] grid, a batched D2Z, the per-wave-vector product with the
// conjugated matrices (correlation over cell offsets), a batched Z2D, and a fused pass
// that adds -gᵀϕ/ncell to the gradient and ½ μ·ϕ/ncell to the energy partials.
#include <cufft.h>

#include <vector>

#include "sgb_internal.h"

#include "sgb_device.cuh"

namespace {
using namespace sgbdev;

__device__ inline void m3v(const double* M, const double* v, double* o) {   // column-major
    o[0] = M[0] * v[0] + M[3] * v[1] + M[6] * v[2];
    o[1] = M[1] * v[0] + M[4] * v[1] + M[7] * v[2];
    o[2] = M[2] * v[0] + M[5] * v[1] + M[8] * v[2];
}

// A[comp][cell], comp = ((i*na + j)*9 + row + 3*col)
__global__ void k_ewald_A(EwaldGeom G, const double* pos, double* A) {
    const int ncell = G.L[0] * G.L[1] * G.L[2];
    const long long nitem = (long long)ncell * G.na * G.na;
    const double pi = 3.14159265358979323846;
    for (long long it = blockIdx.x * (long long)blockDim.x + threadIdx.x; it < nitem; it += (long long)gridDim.x * blockDim.x) {
        const int cell = (int)(it % ncell);
        const int ij = (int)(it / ncell);
        const int i = ij / G.na, j = ij % G.na;
        const int c1 = cell % G.L[0], c2 = (cell / G.L[0]) % G.L[1], c3 = cell / (G.L[0] * G.L[1]);
        double fr[3] = {c1 + pos[3 * j] - pos[3 * i], c2 + pos[3 * j + 1] - pos[3 * i + 1], c3 + pos[3 * j + 2] - pos[3 * i + 2]};
        double dr[3];
        m3v(G.lat, fr, dr);
        double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        const double s2 = G.sig * G.sig;
        for (int n1 = -G.nmax[0]; n1 <= G.nmax[0]; n1++)
            for (int n2 = -G.nmax[1]; n2 <= G.nmax[1]; n2++)
                for (int n3 = -G.nmax[2]; n3 <= G.nmax[2]; n3++) {
                    double nn[3] = {(double)n1, (double)n2, (double)n3}, sh[3];
                    m3v(G.sup, nn, sh);
                    const double rx = dr[0] + sh[0], ry = dr[1] + sh[1], rz = dr[2] + sh[2];
                    const double r2 = rx * rx + ry * ry + rz * rz;
                    if (!(r2 > 0 && r2 <= G.rmax * G.rmax)) continue;
                    const double r = sqrt(r2), r3 = r2 * r;
                    const double ec = erfc(r / (sqrt(2.0) * G.sig));
                    const double ga = sqrt(2 / pi) * (r / G.sig) * exp(-r2 / (2 * s2));
                    const double ci = (ec + ga) / r3 / (4 * pi);
                    const double cr = 3 * (ec + (1 + r2 / (3 * s2)) * ga) / r3 / (4 * pi) / r2;
                    const double rv[3] = {rx, ry, rz};
#pragma unroll
                    for (int q = 0; q < 3; q++)
#pragma unroll
                        for (int p = 0; p < 3; p++) acc[p + 3 * q] += (p == q ? ci : 0.0) - cr * rv[p] * rv[q];
                }
        for (int m1 = -G.mmax[0]; m1 <= G.mmax[0]; m1++)
            for (int m2 = -G.mmax[1]; m2 <= G.mmax[1]; m2++)
                for (int m3 = -G.mmax[2]; m3 <= G.mmax[2]; m3++) {
                    double mm[3] = {(double)m1, (double)m2, (double)m3}, k[3];
                    m3v(G.rec, mm, k);
                    const double k2 = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
                    if (k2 <= 1e-16) {
#pragma unroll
                        for (int q = 0; q < 9; q++) acc[q] += G.demag[q] / G.V;   // surface (demagnetisation) term
                    } else if (k2 <= G.kmax * G.kmax) {
                        const double w = cos(k[0] * dr[0] + k[1] * dr[1] + k[2] * dr[2]) * exp(-s2 * k2 / 2) / k2 / G.V;
#pragma unroll
                        for (int q = 0; q < 3; q++)
#pragma unroll
                            for (int p = 0; p < 3; p++) acc[p + 3 * q] += w * k[p] * k[q];
                    }
                }
        if (dr[0] == 0 && dr[1] == 0 && dr[2] == 0) {
            const double self = 1.0 / (3 * pow(2 * pi, 1.5) * s2 * G.sig);
            acc[0] -= self; acc[4] -= self; acc[8] -= self;
        }
#pragma unroll
        for (int q = 0; q < 9; q++) A[((size_t)ij * 9 + q) * ncell + cell] = acc[q] * G.mu0;
    }
}

// μ[a][α][cell] = -(g S)_α at site (cell, a); g: [ns][9] column-major
template <class R>
__global__ void k_ewald_mu(const R* S, const double* g, int ns, int ncell, double* mu) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += gridDim.x * blockDim.x) {
        const int a = s / ncell, c = s % ncell;
        const double v[3] = {(double)S[s], (double)S[ns + s], (double)S[2 * ns + s]};
        double o[3];
        m3v(g + 9 * (size_t)s, v, o);
        for (int al = 0; al < 3; al++) mu[((size_t)a * 3 + al) * ncell + c] = -o[al];
    }
}

// Fϕ[i][α][m] = Σ_j Σ_β conj(FA[(i,j,α,β)][m]) Fμ[j][β][m]
__global__ void k_ewald_conv(const cufftDoubleComplex* FA, const cufftDoubleComplex* Fmu, int na, int nm,
                             cufftDoubleComplex* Fphi) {
    const long long n = (long long)nm * na * 3;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const int m = (int)(t % nm);
        const int ia = (int)(t / nm);
        const int i = ia / 3, al = ia % 3;
        double re = 0, im = 0;
        for (int j = 0; j < na; j++)
            for (int be = 0; be < 3; be++) {
                const cufftDoubleComplex A = FA[((size_t)(i * na + j) * 9 + al + 3 * be) * nm + m];
                const cufftDoubleComplex u = Fmu[((size_t)j * 3 + be) * nm + m];
                re += A.x * u.x + A.y * u.y;   // conj(A) u
                im += A.x * u.y - A.y * u.x;
            }
        Fphi[(size_t)ia * nm + m] = make_cuDoubleComplex(re, im);
    }
}

// grad[s][c] -= (gᵀ ϕ)_c / ncell (AoS [ns][3]); energy partials ½ μ·ϕ / ncell per block
template <class R>
__global__ void k_ewald_finish(const R* S, const double* g, const double* phi, int ns, int ncell, double* grad,
                               double* part) {
    double e = 0;
    const double inv = 1.0 / ncell;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += gridDim.x * blockDim.x) {
        const int a = s / ncell, c = s % ncell;
        const double p[3] = {phi[((size_t)a * 3 + 0) * ncell + c] * inv, phi[((size_t)a * 3 + 1) * ncell + c] * inv,
                             phi[((size_t)a * 3 + 2) * ncell + c] * inv};
        const double* G = g + 9 * (size_t)s;
        const double v[3] = {(double)S[s], (double)S[ns + s], (double)S[2 * ns + s]};
        double mu[3];
        m3v(G, v, mu);
        e += -0.5 * (mu[0] * p[0] + mu[1] * p[1] + mu[2] * p[2]);
        if (grad) {
            for (int cc = 0; cc < 3; cc++) grad[3 * (size_t)s + cc] -= G[3 * cc] * p[0] + G[3 * cc + 1] * p[1] + G[3 * cc + 2] * p[2];
        }
    }
    if (part) {
        const double t = sgb_block_sum(e);
        if (threadIdx.x == 0) part[blockIdx.x] = t;
    }
}

// ---- integrator stages for systems with long-range terms (one launch per stage) -----
// Heun stage 1 (Integrators.jl:313-326): ξ, Δ1 = rhs(S, ξ, ∇E(S)), P = normalize(S + Δ1)
template <class R, bool INJECT>
__global__ void k_lr_heun_a(const R* S, const double* grad, R* P, R* D1, R* XI, const R* kappa, int ns, R dt, R lam,
                            R nscale, uint64_t seed, uint64_t step, const double* noise) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
        R x0 = 0, x1 = 0, x2 = 0;
        if (nscale != (R)0) {
            if (INJECT) {
                x0 = (R)noise[3 * (size_t)i] * nscale; x1 = (R)noise[3 * (size_t)i + 1] * nscale; x2 = (R)noise[3 * (size_t)i + 2] * nscale;
            } else {
                R g4[4];
                sgb_normals4<R>(seed, 0u, step, (uint32_t)i, 0u, g4);
                x0 = g4[0] * nscale; x1 = g4[1] * nscale; x2 = g4[2] * nscale;
            }
        }
        const R sx = S[i], sy = S[ns + i], sz = S[2 * ns + i];
        R d0, d1, d2;
        rhs_dipole<R>(sx, sy, sz, x0, x1, x2, (R)grad[3 * (size_t)i], (R)grad[3 * (size_t)i + 1], (R)grad[3 * (size_t)i + 2], dt,
                      lam, d0, d1, d2);
        R px = sx + d0, py = sy + d1, pz = sz + d2;
        normalize_dip<R>(px, py, pz, kappa[i]);
        P[i] = px; P[ns + i] = py; P[2 * ns + i] = pz;
        D1[i] = d0; D1[ns + i] = d1; D1[2 * ns + i] = d2;
        XI[i] = x0; XI[ns + i] = x1; XI[2 * ns + i] = x2;
    }
}

// Heun stage 2 (Integrators.jl:327-331): S = normalize(S + (Δ1 + rhs(P, ξ, ∇E(P)))/2)
template <class R>
__global__ void k_lr_heun_b(R* S, const R* P, const double* grad, const R* D1, const R* XI, const R* kappa, int ns, R dt,
                            R lam) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
        R e0, e1, e2;
        rhs_dipole<R>(P[i], P[ns + i], P[2 * ns + i], XI[i], XI[ns + i], XI[2 * ns + i], (R)grad[3 * (size_t)i],
                      (R)grad[3 * (size_t)i + 1], (R)grad[3 * (size_t)i + 2], dt, lam, e0, e1, e2);
        R nx = S[i] + (D1[i] + e0) / 2, ny = S[ns + i] + (D1[ns + i] + e1) / 2, nz = S[2 * ns + i] + (D1[2 * ns + i] + e2) / 2;
        normalize_dip<R>(nx, ny, nz, kappa[i]);
        S[i] = nx; S[ns + i] = ny; S[2 * ns + i] = nz;
    }
}

// midpoint (Integrators.jl:379-413): Ŝ = normalize((S + S')/2)
template <class R>
__global__ void k_lr_mid_half(const R* S, const R* Sp, R* H, const R* kappa, int ns) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
        R hx = (S[i] + Sp[i]) / 2, hy = (S[ns + i] + Sp[ns + i]) / 2, hz = (S[2 * ns + i] + Sp[2 * ns + i]) / 2;
        normalize_dip<R>(hx, hy, hz, kappa[i]);
        H[i] = hx; H[ns + i] = hy; H[2 * ns + i] = hz;
    }
}

// S'' = S + rhs(Ŝ, 0, ∇E(Ŝ)); partial sums of |S' - S''|²; S' <- S''
template <class R>
__global__ void k_lr_mid_update(const R* S, const R* H, const double* grad, R* Sp, int ns, R dt, R lam, double* part) {
    double acc = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
        R d0, d1, d2;
        rhs_dipole<R>(H[i], H[ns + i], H[2 * ns + i], (R)0, (R)0, (R)0, (R)grad[3 * (size_t)i], (R)grad[3 * (size_t)i + 1],
                      (R)grad[3 * (size_t)i + 2], dt, lam, d0, d1, d2);
        const R nx = S[i] + d0, ny = S[ns + i] + d1, nz = S[2 * ns + i] + d2;
        const double e0 = (double)Sp[i] - nx, e1 = (double)Sp[ns + i] - ny, e2 = (double)Sp[2 * ns + i] - nz;
        acc += e0 * e0 + e1 * e1 + e2 * e2;
        Sp[i] = nx; Sp[ns + i] = ny; Sp[2 * ns + i] = nz;
    }
    const double t = sgb_block_sum(acc);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// accepted: S = normalize(S'')
template <class R>
__global__ void k_lr_mid_accept(R* S, const R* Sp, const R* kappa, int ns) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
        R x = Sp[i], y = Sp[ns + i], z = Sp[2 * ns + i];
        normalize_dip<R>(x, y, z, kappa[i]);
        S[i] = x; S[ns + i] = y; S[2 * ns + i] = z;
    }
}

// Field at `site` from every dipole, f = Σ_j g_siteᵀ A[cell_j - cell_site, i, j] g_j S_j, then
// out[0] += dS·f + ½ Δμ·A[0, i, i]·Δμ with Δμ = -g_site dS (one block).
template <class R>
__global__ void k_ewald_delta(const R* S, const double* g, const double* A, int L1, int L2, int L3, int na, int site,
                              double d0, double d1, double d2, double* out) {
    const int ncell = L1 * L2 * L3, ns = ncell * na;
    const int ai = site / ncell, ci = site % ncell;
    const int x1 = ci % L1, y1 = (ci / L1) % L2, z1 = ci / (L1 * L2);
    double f0 = 0, f1 = 0, f2 = 0;
    for (int j = threadIdx.x; j < ns; j += blockDim.x) {
        const int aj = j / ncell, cj = j % ncell;
        const int x2 = cj % L1, y2 = (cj / L1) % L2, z2 = cj / (L1 * L2);
        const int off = sgb_wrap_any(x2 - x1, L1) + L1 * (sgb_wrap_any(y2 - y1, L2) + L2 * sgb_wrap_any(z2 - z1, L3));
        const double* gj = g + 9 * (size_t)j;
        const double sx = S[j], sy = S[ns + j], sz = S[2 * ns + j];
        double mu[3] = {gj[0] * sx + gj[3] * sy + gj[6] * sz, gj[1] * sx + gj[4] * sy + gj[7] * sz, gj[2] * sx + gj[5] * sy + gj[8] * sz};
        const size_t c0 = (size_t)((ai * na + aj) * 9) * ncell + off;
        double am[3];
        for (int r = 0; r < 3; r++)
            am[r] = A[c0 + (size_t)r * ncell] * mu[0] + A[c0 + (size_t)(r + 3) * ncell] * mu[1] + A[c0 + (size_t)(r + 6) * ncell] * mu[2];
        f0 += am[0]; f1 += am[1]; f2 += am[2];
    }
    f0 = sgb_block_sum(f0);
    f1 = sgb_block_sum(f1);
    f2 = sgb_block_sum(f2);
    if (threadIdx.x == 0) {
        const double* gi = g + 9 * (size_t)site;
        const double phi[3] = {f0, f1, f2};
        double f[3];
        for (int r = 0; r < 3; r++) f[r] = gi[3 * r] * phi[0] + gi[3 * r + 1] * phi[1] + gi[3 * r + 2] * phi[2];
        const double dS[3] = {d0, d1, d2};
        double dmu[3], ad[3];
        for (int r = 0; r < 3; r++) dmu[r] = -(gi[r] * dS[0] + gi[r + 3] * dS[1] + gi[r + 6] * dS[2]);
        const size_t c0 = (size_t)((ai * na + ai) * 9) * ncell;
        for (int r = 0; r < 3; r++)
            ad[r] = A[c0 + (size_t)r * ncell] * dmu[0] + A[c0 + (size_t)(r + 3) * ncell] * dmu[1] + A[c0 + (size_t)(r + 6) * ncell] * dmu[2];
        out[0] = dS[0] * f[0] + dS[1] * f[1] + dS[2] * f[2] + 0.5 * (dmu[0] * ad[0] + dmu[1] * ad[1] + dmu[2] * ad[2]);
    }
}

int grid_for(long long n) {
    long long g = (n + SGB_BLOCK - 1) / SGB_BLOCK;
    return (int)(g < 1 ? 1 : (g > 4096 ? 4096 : g));
}

}  // namespace

int ewald_precompute(const EwaldGeom& G, const double* pos_d, double* A, cudaStream_t st) {
    const long long n = (long long)G.L[0] * G.L[1] * G.L[2] * G.na * G.na;
    k_ewald_A<<<grid_for(n), SGB_BLOCK, 0, st>>>(G, pos_d, A);
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

template <class R>
int ewald_apply(const EwaldDev& E, const R* S, double* grad_aos, double* part, cudaStream_t st) {
    const int ncell = E.L[0] * E.L[1] * E.L[2];
    const int ns = ncell * E.na;
    k_ewald_mu<R><<<grid_for(ns), SGB_BLOCK, 0, st>>>(S, E.g, ns, ncell, E.mu);
    if (cudaGetLastError() != cudaSuccess) return SGB_ERR_CUDA;
    if (cufftSetStream(E.plan_f, st) != CUFFT_SUCCESS || cufftSetStream(E.plan_b, st) != CUFFT_SUCCESS) return SGB_ERR_CUDA;
    if (cufftExecD2Z(E.plan_f, E.mu, E.Fmu) != CUFFT_SUCCESS) return SGB_ERR_CUDA;
    k_ewald_conv<<<grid_for((long long)E.nm * E.na * 3), SGB_BLOCK, 0, st>>>(E.FA, E.Fmu, E.na, E.nm, E.Fphi);
    if (cudaGetLastError() != cudaSuccess) return SGB_ERR_CUDA;
    if (cufftExecZ2D(E.plan_b, E.Fphi, E.phi) != CUFFT_SUCCESS) return SGB_ERR_CUDA;
    k_ewald_finish<R><<<EWALD_PART_BLOCKS, SGB_BLOCK, 0, st>>>(S, E.g, E.phi, ns, ncell, grad_aos, part);
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

template <class R>
int ewald_launch_delta(const EwaldDev& E, const R* S, int site, const double* dS3, double* out, cudaStream_t st) {
    k_ewald_delta<R><<<1, 256, 0, st>>>(S, E.g, E.Areal, E.L[0], E.L[1], E.L[2], E.na, site, dS3[0], dS3[1], dS3[2], out);
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}
template int ewald_launch_delta<float>(const EwaldDev&, const float*, int, const double*, double*, cudaStream_t);
template int ewald_launch_delta<double>(const EwaldDev&, const double*, int, const double*, double*, cudaStream_t);

template int ewald_apply<float>(const EwaldDev&, const float*, double*, double*, cudaStream_t);
template int ewald_apply<double>(const EwaldDev&, const double*, double*, double*, cudaStream_t);

template <class R>
int lr_heun_a(const R* S, const double* grad, R* P, R* D1, R* XI, const R* kappa, int ns, double dt, double lam,
              double nscale, uint64_t seed, uint64_t step, const double* noise, cudaStream_t st) {
    if (noise)
        k_lr_heun_a<R, true><<<grid_for(ns), SGB_BLOCK, 0, st>>>(S, grad, P, D1, XI, kappa, ns, (R)dt, (R)lam, (R)nscale, seed,
                                                                step, noise);
    else
        k_lr_heun_a<R, false><<<grid_for(ns), SGB_BLOCK, 0, st>>>(S, grad, P, D1, XI, kappa, ns, (R)dt, (R)lam, (R)nscale, seed,
                                                                 step, noise);
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}
template <class R>
int lr_heun_b(R* S, const R* P, const double* grad, const R* D1, const R* XI, const R* kappa, int ns, double dt,
              double lam, cudaStream_t st) {
    k_lr_heun_b<R><<<grid_for(ns), SGB_BLOCK, 0, st>>>(S, P, grad, D1, XI, kappa, ns, (R)dt, (R)lam);
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}
template <class R>
int lr_mid_half(const R* S, const R* Sp, R* H, const R* kappa, int ns, cudaStream_t st) {
    k_lr_mid_half<R><<<grid_for(ns), SGB_BLOCK, 0, st>>>(S, Sp, H, kappa, ns);
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}
template <class R>
int lr_mid_update(const R* S, const R* H, const double* grad, R* Sp, int ns, double dt, double lam, double* part,
                  cudaStream_t st) {
    k_lr_mid_update<R><<<EWALD_PART_BLOCKS, SGB_BLOCK, 0, st>>>(S, H, grad, Sp, ns, (R)dt, (R)lam, part);
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}
template <class R>
int lr_mid_accept(R* S, const R* Sp, const R* kappa, int ns, cudaStream_t st) {
    k_lr_mid_accept<R><<<grid_for(ns), SGB_BLOCK, 0, st>>>(S, Sp, kappa, ns);
    return cudaGetLastError() == cudaSuccess ? SGB_OK : SGB_ERR_CUDA;
}

#define SGB_LR_INST(R)                                                                                           \
    template int lr_heun_a<R>(const R*, const double*, R*, R*, R*, const R*, int, double, double, double, uint64_t, \
                              uint64_t, const double*, cudaStream_t);                                          \
    template int lr_heun_b<R>(R*, const R*, const double*, const R*, const R*, const R*, int, double, double,      \
                              cudaStream_t);                                                                   \
    template int lr_mid_half<R>(const R*, const R*, R*, const R*, int, cudaStream_t);                            \
    template int lr_mid_update<R>(const R*, const R*, const double*, R*, int, double, double, double*, cudaStream_t); \
    template int lr_mid_accept<R>(R*, const R*, const R*, int, cudaStream_t);
SGB_LR_INST(float)
SGB_LR_INST(double)
