// sgb_adjoint.cu -- gradient of an S(q,ω) loss through a deterministic ImplicitMidpoint
// trajectory with respect to coupling parameters (discrete adjoint, FP64).
//
// Sunny.jl has no reverse rule for its dynamics; the parameter convention follows its
// fitting code (src/Fitting.jl:123-152, src/ModelParams.jl:140-150): the energy is linear
// in labelled parameters, E(θ) = E_rest + Σ_k θ_k E_k. The forward pass is exactly one
// add_sample! (src/SampledCorrelations/CorrelationSampling.jl:1-139) of a dipole-mode
// system integrated by the spherical midpoint method (src/Integrators.jl:379-413) with
// damping 0, followed by the loss L = mean over all complex bins of |data - target|².
//
// Reverse pass:
//   * loss -> spectra: data = W(conj(Â_α) Â_β) with W = F diag(g) F* (cuFFT transforms
//     along ω, g = window / n_contrib / n). W is self-adjoint, so the cotangent of the
//     product is W(dL/d data*); Â-cotangents follow from the bilinear product, then the
//     time transform (adjoint = inverse transform) and the space transform (adjoint =
//     forward transform) give dL/d(snapshot) for every recorded step.
//   * steps: the converged midpoint step solves G(X, S) = X - S + dt Ŝ × ∇E(Ŝ) = 0 with
//     Ŝ = κ (S + X) / |S + X| and S_next = κ X / |X|. With v the cotangent of X,
//     μ solves (∂G/∂X)ᵀ μ = v by the fixed-point iteration μ <- v - dt P Jhᵀ μ, where
//     P = ∂Ŝ/∂S = (κ/|S+X|)(I - ûûᵀ) and Jhᵀ y = ∇E(Ŝ) × y + H (y × Ŝ), H the Hessian of
//     E. Then the cotangent of S is 2μ - v and dL/dθ_k -= dt Σ μ · (Ŝ × ∇E_k(Ŝ)).
//     H z is the field-free gradient evaluated at z, exact because the supported energies
//     are quadratic forms (bilinear pair couplings, onsite anisotropy of rank <= 2).
//   * memory: the state is checkpointed every `checkpoint` steps on the forward pass;
//     each segment is recomputed forward, then swept backward.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>
#include "sgb_device.cuh"
#include "sgb_tables.h"
#include "sgb_handles.h"
#include "sgb_corr.h"

struct sgb_adjoint {
    sgb_system* sys = nullptr;
    sgb_corr* corr = nullptr;
    int np = 0;
    std::vector<void*> ptables;          // device tables of each parameter's unit couplings
    std::vector<Model<double>> pm;       // models of the parameter couplings
    Model<double> quad{};                // the system's couplings without the Zeeman field (H z)
    double* target = nullptr;            // [col][ω] complex
    double* data = nullptr;              // [col][ω] complex
    double* abar = nullptr;              // cotangent of the spectra, layout of corr->Ahat
    double* G = nullptr;                 // [nsnaps][3][ns] dL/dS at recorded steps
    double* ckpt = nullptr;              // [nseg + 1][3][ns]
    double* traj = nullptr;              // [checkpoint + 1][3][ns]
    double* w3 = nullptr;                // scratch [3][ns] x 6: Ŝ, lam, v, mu, mu2, w
    double* fac = nullptr;               // [ns]
    double* gbuf = nullptr;              // [ns][3] ∇E(Ŝ)
    double* hbuf = nullptr;              // [ns][3] H w
    double* gk = nullptr;                // [np][ns][3] ∇E_k(Ŝ)
    double* part = nullptr;              // reduction partials
    double* red = nullptr;               // [8 + np] reduction results
    double* gth = nullptr;               // [np] accumulated dL/dθ
    cufftHandle plan_w = 0;
    bool have_plan = false;
    int ncols = 0, cap_ckpt = 0, cap_seg = 0;
    bool have_target = false;
    std::string err;
};

namespace {

constexpr int ADJ_BLOCK = 256;
constexpr int ADJ_MAXGRID = 1024;

int grid_of(size_t n) { return (int)std::min<size_t>(ADJ_MAXGRID, std::max<size_t>(1, (n + ADJ_BLOCK - 1) / ADJ_BLOCK)); }

// Ŝ = κ (S + X) / |S + X| and fac = κ / |S + X| per site (SoA [3][ns]).
__global__ void k_adj_mid(const double* __restrict__ S, const double* __restrict__ X, const double* __restrict__ kap,
                          int ns, double* __restrict__ Sh, double* __restrict__ fac) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
        const double x = S[i] + X[i], y = S[ns + i] + X[ns + i], z = S[2 * ns + i] + X[2 * ns + i];
        const double r = sqrt(x * x + y * y + z * z);
        const double f = (kap[i] == 0.0 || r == 0.0) ? 0.0 : kap[i] / r;
        Sh[i] = f * x; Sh[ns + i] = f * y; Sh[2 * ns + i] = f * z;
        fac[i] = f;
    }
}

// v = λ - x̂ (x̂ · λ), x̂ = X / |X| (cotangent through S_next = κ X / |X| with |X| = κ).
__global__ void k_adj_proj(const double* __restrict__ X, const double* __restrict__ lam, int ns, double* __restrict__ v) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
        const double x = X[i], y = X[ns + i], z = X[2 * ns + i];
        const double r2 = x * x + y * y + z * z;
        const double lx = lam[i], ly = lam[ns + i], lz = lam[2 * ns + i];
        const double d = r2 > 0 ? (x * lx + y * ly + z * lz) / r2 : 0.0;
        v[i] = lx - d * x; v[ns + i] = ly - d * y; v[2 * ns + i] = lz - d * z;
    }
}

// w = μ × Ŝ
__global__ void k_adj_cross(const double* __restrict__ mu, const double* __restrict__ Sh, int ns, double* __restrict__ w) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
        const double a = mu[i], b = mu[ns + i], c = mu[2 * ns + i];
        const double x = Sh[i], y = Sh[ns + i], z = Sh[2 * ns + i];
        w[i] = b * z - c * y; w[ns + i] = c * x - a * z; w[2 * ns + i] = a * y - b * x;
    }
}

// μ' = v - dt P (g × μ + H w); partials of |μ' - μ|² and |v|² (grad buffers are [ns][3]).
__global__ void k_adj_iter(const double* __restrict__ mu, const double* __restrict__ v, const double* __restrict__ g,
                           const double* __restrict__ Hw, const double* __restrict__ Sh, const double* __restrict__ fac,
                           const double* __restrict__ kap, int ns, double dt, double* __restrict__ mu2,
                           double* __restrict__ part) {
    double dd = 0, vv = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
        const double a = mu[i], b = mu[ns + i], c = mu[2 * ns + i];
        const double gx = g[3 * i], gy = g[3 * i + 1], gz = g[3 * i + 2];
        double yx = gy * c - gz * b + Hw[3 * i];
        double yy = gz * a - gx * c + Hw[3 * i + 1];
        double yz = gx * b - gy * a + Hw[3 * i + 2];
        const double f = fac[i];
        double ux = 0, uy = 0, uz = 0;
        if (kap[i] != 0.0) { ux = Sh[i] / kap[i]; uy = Sh[ns + i] / kap[i]; uz = Sh[2 * ns + i] / kap[i]; }
        const double d = ux * yx + uy * yy + uz * yz;
        const double px = f * (yx - d * ux), py = f * (yy - d * uy), pz = f * (yz - d * uz);
        const double nx = v[i] - dt * px, ny = v[ns + i] - dt * py, nz = v[2 * ns + i] - dt * pz;
        mu2[i] = nx; mu2[ns + i] = ny; mu2[2 * ns + i] = nz;
        dd += (nx - a) * (nx - a) + (ny - b) * (ny - b) + (nz - c) * (nz - c);
        vv += v[i] * v[i] + v[ns + i] * v[ns + i] + v[2 * ns + i] * v[2 * ns + i];
    }
    const double s0 = sgb_block_sum(dd);
    const double s1 = sgb_block_sum(vv);
    if (threadIdx.x == 0) { part[2 * blockIdx.x] = s0; part[2 * blockIdx.x + 1] = s1; }
}

// λ = 2μ - v (+ G, the direct cotangent of a recorded state); partials of
// -dt μ · (Ŝ × ∇E_k(Ŝ)) for every parameter k.
__global__ void k_adj_finish(const double* __restrict__ mu, const double* __restrict__ v, const double* __restrict__ Gs,
                             const double* __restrict__ Sh, const double* __restrict__ gk, int np, int ns, double dt,
                             double* __restrict__ lam, double* __restrict__ part) {
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
        const double a = mu[i], b = mu[ns + i], c = mu[2 * ns + i];
        for (int q = 0; q < 3; q++) {
            double l = 2.0 * mu[q * ns + i] - v[q * ns + i];
            if (Gs) l += Gs[q * ns + i];
            lam[q * ns + i] = l;
        }
        const double x = Sh[i], y = Sh[ns + i], z = Sh[2 * ns + i];
        for (int k = 0; k < np; k++) {
            const double* e = gk + (size_t)k * 3 * ns + 3 * (size_t)i;
            const double cx = y * e[2] - z * e[1], cy = z * e[0] - x * e[2], cz = x * e[1] - y * e[0];
            acc[k] += -dt * (a * cx + b * cy + c * cz);
        }
    }
    for (int k = 0; k < np; k++) {
        const double s = sgb_block_sum(acc[k]);
        if (threadIdx.x == 0) part[(size_t)k * gridDim.x + blockIdx.x] = s;
    }
}

// out[k] (+)= Σ_b part[k * nb + b], in block order (deterministic).
__global__ void k_adj_reduce(const double* __restrict__ part, int nb, int ncomp, int stride_k, int stride_b,
                             double* __restrict__ out, int accumulate) {
    const int k = blockIdx.x;
    if (k >= ncomp) return;
    double s = 0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) s += part[(size_t)k * stride_k + (size_t)b * stride_b];
    const double t = sgb_block_sum(s);
    if (threadIdx.x == 0) out[k] = accumulate ? out[k] + t : t;
}

// Loss partials Σ |D - T|² and the cotangent dbar = (D - T) / Nb (complex, same layout).
__global__ void k_adj_loss(const double2* __restrict__ D, const double2* __restrict__ T, size_t n, double inv,
                           double2* __restrict__ dbar, double* __restrict__ part) {
    double s = 0;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const double2 d = D[e], t = T[e];
        const double x = d.x - t.x, y = d.y - t.y;
        s += x * x + y * y;
        dbar[e] = make_double2(x * inv, y * inv);
    }
    const double r = sgb_block_sum(s);
    if (threadIdx.x == 0) part[blockIdx.x] = r;
}

// Cotangents of the spectra: for P_{c,i,j} = conj(Â_{α,i}) Â_{β,j} with cotangent P̄,
// Â̄_{α,i} += conj(P̄) Â_{β,j} and Â̄_{β,j} += P̄ Â_{α,i}. Â and Â̄ in the accumulator's
// spectrum layout [ω][o][a][cell]; P̄ in the read-out layout [col][ω] with
// col = c + ncorr (i + npos (j + npos cell)).
__global__ void k_adj_spec(const double2* __restrict__ Pb, const double2* __restrict__ Ah, const int* __restrict__ pairs,
                           int ncorr, int nobs, int npos, int ncell, int n, double2* __restrict__ Ab) {
    const size_t total = (size_t)n * nobs * npos * ncell;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int cell = (int)(e % ncell);
        size_t r = e / ncell;
        const int a = (int)(r % npos); r /= npos;
        const int o = (int)(r % nobs);
        const int w = (int)(r / nobs);
        const size_t row = (size_t)w * nobs;
        double ax = 0, ay = 0;
        for (int c = 0; c < ncorr; c++) {
            const int al = pairs[2 * c], be = pairs[2 * c + 1];
            if (al == o) {
                for (int j = 0; j < npos; j++) {
                    const double2 p = Pb[((size_t)c + (size_t)ncorr * (a + (size_t)npos * (j + (size_t)npos * cell))) * n + w];
                    const double2 h = Ah[((row + be) * npos + j) * ncell + cell];
                    // conj(p) * h
                    ax += p.x * h.x + p.y * h.y;
                    ay += p.x * h.y - p.y * h.x;
                }
            }
            if (be == o) {
                for (int i = 0; i < npos; i++) {
                    const double2 p = Pb[((size_t)c + (size_t)ncorr * (i + (size_t)npos * (a + (size_t)npos * cell))) * n + w];
                    const double2 h = Ah[((row + al) * npos + i) * ncell + cell];
                    // p * h
                    ax += p.x * h.x - p.y * h.y;
                    ay += p.x * h.y + p.y * h.x;
                }
            }
        }
        Ab[e] = make_double2(ax, ay);
    }
}

// dL/dS at recorded step t: 2 scale Σ_o ops[o][q][site] Re(Ā[t][o][a][cell]).
__global__ void k_adj_snapgrad(const double2* __restrict__ Ab, const double* __restrict__ ops, int nobs, int npos,
                               int ncell, int nsnaps, double scale, double* __restrict__ G) {
    const int ns = npos * ncell;
    const size_t total = (size_t)nsnaps * ns;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int site = (int)(e % ns);
        const int t = (int)(e / ns);
        const int a = site / ncell, cell = site % ncell;
        double g0 = 0, g1 = 0, g2 = 0;
        for (int o = 0; o < nobs; o++) {
            const double re = Ab[(((size_t)t * nobs + o) * npos + a) * ncell + cell].x;
            const double* op = ops + (size_t)o * 3 * ns;
            g0 += op[site] * re; g1 += op[ns + site] * re; g2 += op[2 * ns + site] * re;
        }
        double* out = G + (size_t)t * 3 * ns;
        out[site] = 2 * scale * g0; out[ns + site] = 2 * scale * g1; out[2 * ns + site] = 2 * scale * g2;
    }
}

int afail(sgb_adjoint* a, int code, const std::string& msg) {
    if (a) {
        a->err = msg;
        if (a->sys) a->sys->err = msg;
    }
    sgb_int_set_error(msg);
    return code;
}

#define ACK(call)                                                                                         \
    do {                                                                                                  \
        cudaError_t _e = (call);                                                                          \
        if (_e != cudaSuccess) return afail(a, SGB_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
    } while (0)

bool onsite_rank_le2(const double* c28) {
    for (int k = 6; k < 28; k++)
        if (c28[k] != 0.0) return false;
    return true;
}

int amalloc(sgb_adjoint* a, void** p, size_t bytes) {
    if (cudaMalloc(p, bytes ? bytes : 16) != cudaSuccess) {
        *p = nullptr;
        return afail(a, SGB_ERR_NOMEM, "device allocation failed (adjoint buffers)");
    }
    return SGB_OK;
}

// W = F diag(g) F* along ω on `buf` ([ncols][n] complex), in place.
int apply_w(sgb_adjoint* a, double* buf) {
    sgb_corr* c = a->corr;
    cudaStream_t st = a->sys->stream;
    if (cufftExecZ2Z(a->plan_w, (cufftDoubleComplex*)buf, (cufftDoubleComplex*)buf, CUFFT_INVERSE) != CUFFT_SUCCESS)
        return afail(a, SGB_ERR_CUDA, "cuFFT (adjoint read-out inverse) failed");
    if (corr_launch_window(buf, a->ncols, c->nomega, c->g, st)) return afail(a, SGB_ERR_CUDA, "window launch");
    if (cufftExecZ2Z(a->plan_w, (cufftDoubleComplex*)buf, (cufftDoubleComplex*)buf, CUFFT_FORWARD) != CUFFT_SUCCESS)
        return afail(a, SGB_ERR_CUDA, "cuFFT (adjoint read-out forward) failed");
    a->sys->launches++;
    return SGB_OK;
}

int grad_into(sgb_adjoint* a, const Model<double>& M, const double* S, double* out) {
    if (dip_launch_grad<double>(M, S, out, a->sys->stream) != SGB_OK)
        return afail(a, SGB_ERR_CUDA, std::string("gradient launch: ") + cudaGetErrorString(cudaGetLastError()));
    a->sys->launches++;
    return SGB_OK;
}

// The system's coupling tables are rebuilt (and reallocated) whenever its couplings
// change: take the current model before every pass and re-check what the adjoint supports.
int refresh_models(sgb_adjoint* a) {
    sgb_system* s = a->sys;
    int rc = sgb_int_ensure_tables(s);
    if (rc) return rc;
    if (s->has_biquad) return afail(a, SGB_ERR_ARG, "the adjoint supports bilinear pair couplings only (no biquadratic terms)");
    for (int at = 0; at < s->d.natoms; at++)
        if (!onsite_rank_le2(s->onsite_h.data() + 28 * at))
            return afail(a, SGB_ERR_ARG, "the adjoint supports onsite anisotropy of rank <= 2");
    a->quad = s->md;
    a->quad.h = nullptr;
    for (Model<double>& M : a->pm) M.kappa = s->md.kappa;
    return SGB_OK;
}

}  // namespace

extern "C" {

void sgb_adjoint_destroy(sgb_adjoint* a) {
    if (!a) return;
    if (a->sys && a->sys->stream) cudaStreamSynchronize(a->sys->stream);
    for (void*& p : a->ptables)
        if (p) cudaFree(p);
    void* bufs[] = {a->target, a->data, a->abar, a->G, a->ckpt, a->traj, a->w3, a->fac, a->gbuf, a->hbuf,
                    a->gk, a->part, a->red, a->gth};
    for (void* p : bufs)
        if (p) cudaFree(p);
    if (a->have_plan) cufftDestroy(a->plan_w);
    if (a->corr) sgb_corr_destroy(a->corr);
    delete a;
}

int sgb_adjoint_create(sgb_system* s, const sgb_corr_desc* d, int32_t nparams, const sgb_bond* bonds,
                       const int32_t* nbonds, const double* onsite, sgb_adjoint** out) {
    if (!s || !d || !out || nparams < 1 || nparams > 8 || !nbonds) return afail(nullptr, SGB_ERR_ARG, "invalid arguments");
    *out = nullptr;
    if (s->sun || s->fp32) return afail(nullptr, SGB_ERR_ARG, "the adjoint supports FP64 dipole-mode systems");
    if (s->ewald_on) return afail(nullptr, SGB_ERR_ARG, "the adjoint does not support dipole-dipole interactions");
    if (s->inh_bonds || s->inh_onsite) return afail(nullptr, SGB_ERR_ARG, "the adjoint supports homogeneous systems only");
    if (d->damping != 0.0) return afail(nullptr, SGB_ERR_ARG, "the adjoint differentiates the undamped midpoint method (damping = 0)");
    if (d->n_all_omega < 2) return afail(nullptr, SGB_ERR_ARG, "the adjoint needs a dynamical S(q,ω) (n_all_omega > 1)");
    int rc = sgb_int_ensure_tables(s);
    if (rc) return rc;
    if (s->has_biquad) return afail(nullptr, SGB_ERR_ARG, "the adjoint supports bilinear pair couplings only (no biquadratic terms)");
    const int na = s->d.natoms;
    for (int at = 0; at < na; at++)
        if (!onsite_rank_le2(s->onsite_h.data() + 28 * at))
            return afail(nullptr, SGB_ERR_ARG, "the adjoint supports onsite anisotropy of rank <= 2");
    sgb_adjoint* a = new sgb_adjoint();
    a->sys = s;
    a->np = nparams;
    auto bad = [&](int code) { sgb_adjoint_destroy(a); return code; };
    // the accumulator that records and transforms the sample
    if ((rc = sgb_corr_create(s, d, &a->corr))) return bad(rc);
    sgb_corr* c = a->corr;
    std::vector<double> g;
    sgb_int_window_weights(c->nomega, 0, g);
    ACK(cudaMemcpy(c->g, g.data(), sizeof(double) * c->nomega, cudaMemcpyHostToDevice));
    c->window = 0;
    // parameter models
    const sgb_bond* b = bonds;
    for (int k = 0; k < nparams; k++) {
        if (nbonds[k] < 0) return bad(afail(a, SGB_ERR_ARG, "negative bond count"));
        std::vector<sgb_bond> bk(b, b + nbonds[k]);
        b += nbonds[k];
        for (const sgb_bond& e : bk)
            if (e.biquad_kind != 0) return bad(afail(a, SGB_ERR_ARG, "parameter couplings must be bilinear"));
        std::vector<double> on(28 * (size_t)na, 0.0);
        if (onsite) {
            on.assign(onsite + (size_t)k * 28 * na, onsite + (size_t)(k + 1) * 28 * na);
            for (int at = 0; at < na; at++)
                if (!onsite_rank_le2(on.data() + 28 * at))
                    return bad(afail(a, SGB_ERR_ARG, "parameter anisotropy must have rank <= 2"));
        }
        Model<double> M{};
        std::vector<unsigned char> buf;
        bool any_bq = false;
        std::string e = sgbhost::pack_tables<double>(na, 0, false, s->d.dims, bk, on, M, buf, any_bq);
        if (!e.empty()) return bad(afail(a, SGB_ERR_ARG, e));
        void* t = nullptr;
        if ((rc = amalloc(a, &t, buf.size()))) return bad(rc);
        a->ptables.push_back(t);
        ACK(cudaMemcpy(t, buf.data(), buf.size(), cudaMemcpyHostToDevice));
        M.L1 = s->d.dims[0]; M.L2 = s->d.dims[1]; M.L3 = s->d.dims[2];
        M.ns = s->ns; M.ncell = s->ncell;
        M.kappa = s->md.kappa;
        M.h = nullptr;
        M.nbr = nullptr;
        M.tables = (const unsigned char*)t;
        a->pm.push_back(M);
    }
    a->quad = s->md;
    a->quad.h = nullptr;
    const size_t ns = s->ns;
    a->ncols = (int)(c->plen / c->nomega);
    const size_t plen = c->plen;
    const size_t nA = (size_t)c->nomega * c->nobs * c->npos * c->ncell;
    if ((rc = amalloc(a, (void**)&a->target, 16 * plen)) || (rc = amalloc(a, (void**)&a->data, 16 * plen)) ||
        (rc = amalloc(a, (void**)&a->abar, 16 * nA)) ||
        (rc = amalloc(a, (void**)&a->G, sizeof(double) * 3 * ns * c->nsnaps)) ||
        (rc = amalloc(a, (void**)&a->w3, sizeof(double) * 3 * ns * 6)) ||
        (rc = amalloc(a, (void**)&a->fac, sizeof(double) * ns)) ||
        (rc = amalloc(a, (void**)&a->gbuf, sizeof(double) * 3 * ns)) ||
        (rc = amalloc(a, (void**)&a->hbuf, sizeof(double) * 3 * ns)) ||
        (rc = amalloc(a, (void**)&a->gk, sizeof(double) * 3 * ns * nparams)) ||
        (rc = amalloc(a, (void**)&a->part, sizeof(double) * 2 * ADJ_MAXGRID * (nparams + 2))) ||
        (rc = amalloc(a, (void**)&a->red, sizeof(double) * (8 + nparams))) ||
        (rc = amalloc(a, (void**)&a->gth, sizeof(double) * nparams)))
        return bad(rc);
    ACK(cudaMemset(a->target, 0, 16 * plen));
    int n1[1] = {c->nomega};
    if (cufftPlanMany(&a->plan_w, 1, n1, nullptr, 1, c->nomega, nullptr, 1, c->nomega, CUFFT_Z2Z, a->ncols) != CUFFT_SUCCESS)
        return bad(afail(a, SGB_ERR_CUDA, "cufftPlanMany (adjoint read-out) failed"));
    a->have_plan = true;
    cufftSetStream(a->plan_w, s->stream);
    *out = a;
    return SGB_OK;
}

const char* sgb_adjoint_last_error(const sgb_adjoint* a) { return a ? a->err.c_str() : ""; }

int sgb_adjoint_set_target(sgb_adjoint* a, const double* target) {
    if (!a || !target) return afail(a, SGB_ERR_ARG, "null argument");
    sgb_corr* c = a->corr;
    sgb_system* s = a->sys;
    // host Sunny layout [c,i,j,q,ω] -> device read-out layout [col][ω]
    double* tmp = nullptr;
    int rc = amalloc(a, (void**)&tmp, 16 * c->plen);
    if (rc) return rc;
    cudaError_t e = cudaMemcpyAsync(tmp, target, 16 * c->plen, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess && corr_launch_gather(tmp, a->ncols, 0, a->ncols, c->nomega, 1.0, a->target, s->stream))
        e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    cudaFree(tmp);
    if (e != cudaSuccess) return afail(a, SGB_ERR_CUDA, std::string("target upload: ") + cudaGetErrorString(e));
    a->have_target = true;
    return SGB_OK;
}

int sgb_adjoint_loss_grad(sgb_adjoint* a, const double* S0, int32_t checkpoint, double* loss, double* grad,
                          double* grad_S0, double* data_out) {
    if (!a || !S0) return afail(a, SGB_ERR_ARG, "null argument");
    sgb_system* s = a->sys;
    sgb_corr* c = a->corr;
    if (!s) return afail(a, SGB_ERR_STATE, "the System of this adjoint was destroyed");
    const int mp = c->measperiod;
    const int nsteps = mp * (c->nsnaps - 1);
    if (checkpoint < 1) checkpoint = nsteps;
    checkpoint = std::max(mp, (checkpoint / mp) * mp);   // segments hold whole measurement periods
    const int nseg = (nsteps + checkpoint - 1) / checkpoint;
    const size_t ns = s->ns, st3 = 3 * ns;
    cudaStream_t st = s->stream;
    int rc;
    if (a->cap_ckpt < nseg + 1) {
        if (a->ckpt) cudaFree(a->ckpt);
        a->ckpt = nullptr;
        if ((rc = amalloc(a, (void**)&a->ckpt, sizeof(double) * st3 * (nseg + 1)))) return rc;
        a->cap_ckpt = nseg + 1;
    }
    if (a->cap_seg < checkpoint + 1) {
        if (a->traj) cudaFree(a->traj);
        a->traj = nullptr;
        if ((rc = amalloc(a, (void**)&a->traj, sizeof(double) * st3 * (checkpoint + 1)))) return rc;
        a->cap_seg = checkpoint + 1;
    }
    // ---- forward: trajectory with snapshots and checkpoints -------------------------------
    if ((rc = sgb_set_state(s, S0, nullptr))) return rc;
    if ((rc = refresh_models(a))) return rc;
    const double scale = 1.0 / std::sqrt((double)c->ncell);
    const size_t nA = (size_t)c->nomega * c->nobs * c->npos * c->ncell;
    ACK(cudaMemsetAsync(c->A, 0, 16 * nA, st));
    for (int sg = 0; sg < nseg; sg++) {
        const int s0 = sg * checkpoint, len = std::min(checkpoint, nsteps - s0);
        ACK(cudaMemcpyAsync(a->ckpt + (size_t)sg * st3, s->S, sizeof(double) * st3, cudaMemcpyDeviceToDevice, st));
        SnapArgs<double> sn{1, c->nobs, mp, s0 / mp, (const double*)c->ops, (double*)c->A, scale};
        if ((rc = sgb_int_midpoint_snap(s, c->dt, c->tol, c->max_iters, len, sn, nullptr))) return rc;
    }
    ACK(cudaMemcpyAsync(a->ckpt + (size_t)nseg * st3, s->S, sizeof(double) * st3, cudaMemcpyDeviceToDevice, st));
    // ---- loss: space and time transforms, product, read-out transform ---------------------------
    if (cufftExecZ2Z(c->plan_space, (cufftDoubleComplex*)c->A, (cufftDoubleComplex*)c->A, CUFFT_INVERSE) != CUFFT_SUCCESS)
        return afail(a, SGB_ERR_CUDA, "space FFT failed");
    if (cufftExecZ2Z(c->plan_time, (cufftDoubleComplex*)c->A, (cufftDoubleComplex*)c->Ahat, CUFFT_FORWARD) != CUFFT_SUCCESS)
        return afail(a, SGB_ERR_CUDA, "time FFT failed");
    ACK(cudaMemsetAsync(c->P, 0, 16 * c->plen, st));
    if (corr_launch_accum<double>((const double*)c->Ahat, c->P, c->pairs, c->ncorr, c->nobs, c->npos, c->ncell, c->nomega,
                                  1, nA, st))
        return afail(a, SGB_ERR_CUDA, "accumulate launch");
    if (corr_launch_gather(c->P, a->ncols, 0, a->ncols, c->nomega, 1.0, a->data, st)) return afail(a, SGB_ERR_CUDA, "gather launch");
    s->launches += 2;
    if ((rc = apply_w(a, a->data))) return rc;
    if (data_out) {
        // read-out layout -> Sunny layout, through the accumulator's P buffer
        if (corr_launch_scatter(a->data, a->ncols, c->nomega, c->P, st)) return afail(a, SGB_ERR_CUDA, "scatter launch");
        ACK(cudaMemcpyAsync(data_out, c->P, 16 * c->plen, cudaMemcpyDeviceToHost, st));
    }
    const double Nb = (double)c->plen;
    double* dbar = (double*)c->P;   // P is free from here on
    {
        const int gb = grid_of(c->plen);
        k_adj_loss<<<gb, ADJ_BLOCK, 0, st>>>((const double2*)a->data, (const double2*)a->target, c->plen, 1.0 / Nb,
                                             (double2*)dbar, a->part);
        k_adj_reduce<<<1, ADJ_BLOCK, 0, st>>>(a->part, gb, 1, 0, 1, a->red, 0);
        s->launches += 2;
    }
    double Lsum = 0;
    ACK(cudaMemcpyAsync(&Lsum, a->red, sizeof(double), cudaMemcpyDeviceToHost, st));
    // ---- reverse through the transforms ------------------------------------------------------
    if ((rc = apply_w(a, dbar))) return rc;                                    // P̄ = W(D̄)
    k_adj_spec<<<grid_of(nA), ADJ_BLOCK, 0, st>>>((const double2*)dbar, (const double2*)c->Ahat, c->pairs, c->ncorr,
                                                  c->nobs, c->npos, c->ncell, c->nomega, (double2*)a->abar);
    s->launches++;
    if (cufftExecZ2Z(c->plan_time, (cufftDoubleComplex*)a->abar, (cufftDoubleComplex*)c->A, CUFFT_INVERSE) != CUFFT_SUCCESS)
        return afail(a, SGB_ERR_CUDA, "time FFT (adjoint) failed");
    if (cufftExecZ2Z(c->plan_space, (cufftDoubleComplex*)c->A, (cufftDoubleComplex*)c->A, CUFFT_FORWARD) != CUFFT_SUCCESS)
        return afail(a, SGB_ERR_CUDA, "space FFT (adjoint) failed");
    k_adj_snapgrad<<<grid_of((size_t)c->nsnaps * ns), ADJ_BLOCK, 0, st>>>((const double2*)c->A, (const double*)c->ops,
                                                                          c->nobs, c->npos, c->ncell, c->nsnaps, scale, a->G);
    s->launches++;
    ACK(cudaGetLastError());
    // ---- reverse through the steps, segment by segment -----------------------------------------
    double* Sh = a->w3;
    double* lam = a->w3 + st3;
    double* v = a->w3 + 2 * st3;
    double* mu = a->w3 + 3 * st3;
    double* mu2 = a->w3 + 4 * st3;
    double* w = a->w3 + 5 * st3;
    ACK(cudaMemcpyAsync(lam, a->G + (size_t)(c->nsnaps - 1) * st3, sizeof(double) * st3, cudaMemcpyDeviceToDevice, st));
    ACK(cudaMemsetAsync(a->gth, 0, sizeof(double) * a->np, st));
    const int gb = grid_of(ns);
    const double dt = c->dt;
    const double* kap = s->md.kappa;
    SnapArgs<double> nosnap{0, 0, 1, 0, nullptr, nullptr, 0.0};
    const double adj_tol2 = 1e-28;   // |Δμ|² <= 1e-28 |v|², i.e. 1e-14 relative
    for (int sg = nseg - 1; sg >= 0; sg--) {
        const int s0 = sg * checkpoint, len = std::min(checkpoint, nsteps - s0);
        // recompute the segment's states
        ACK(cudaMemcpyAsync(s->S, a->ckpt + (size_t)sg * st3, sizeof(double) * st3, cudaMemcpyDeviceToDevice, st));
        ACK(cudaMemcpyAsync(a->traj, s->S, sizeof(double) * st3, cudaMemcpyDeviceToDevice, st));
        for (int j = 1; j <= len; j++) {
            if ((rc = sgb_int_midpoint_snap(s, dt, c->tol, c->max_iters, 1, nosnap, nullptr))) return rc;
            ACK(cudaMemcpyAsync(a->traj + (size_t)j * st3, s->S, sizeof(double) * st3, cudaMemcpyDeviceToDevice, st));
        }
        for (int j = len - 1; j >= 0; j--) {
            const double* Sn = a->traj + (size_t)j * st3;
            const double* Sx = a->traj + (size_t)(j + 1) * st3;
            const int n = s0 + j;   // step n -> n + 1
            k_adj_mid<<<gb, ADJ_BLOCK, 0, st>>>(Sn, Sx, kap, (int)ns, Sh, a->fac);
            k_adj_proj<<<gb, ADJ_BLOCK, 0, st>>>(Sx, lam, (int)ns, v);
            s->launches += 2;
            if ((rc = grad_into(a, s->md, Sh, a->gbuf))) return rc;
            for (int k = 0; k < a->np; k++)
                if ((rc = grad_into(a, a->pm[k], Sh, a->gk + (size_t)k * st3))) return rc;
            ACK(cudaMemcpyAsync(mu, v, sizeof(double) * st3, cudaMemcpyDeviceToDevice, st));
            bool conv = false;
            for (int it = 0; it < 200 && !conv; it++) {
                k_adj_cross<<<gb, ADJ_BLOCK, 0, st>>>(mu, Sh, (int)ns, w);
                s->launches++;
                if ((rc = grad_into(a, a->quad, w, a->hbuf))) return rc;
                k_adj_iter<<<gb, ADJ_BLOCK, 0, st>>>(mu, v, a->gbuf, a->hbuf, Sh, a->fac, kap, (int)ns, dt, mu2, a->part);
                k_adj_reduce<<<2, ADJ_BLOCK, 0, st>>>(a->part, gb, 2, 1, 2, a->red, 0);
                s->launches += 2;
                std::swap(mu, mu2);
                double r[2];
                ACK(cudaMemcpyAsync(r, a->red, sizeof(r), cudaMemcpyDeviceToHost, st));
                ACK(cudaStreamSynchronize(st));
                conv = r[0] <= adj_tol2 * r[1] || r[1] == 0.0;
            }
            if (!conv) return afail(a, SGB_ERR_NOCONVERGE, "adjoint fixed-point iteration did not converge");
            const double* Gs = (n % mp == 0) ? a->G + (size_t)(n / mp) * st3 : nullptr;
            k_adj_finish<<<gb, ADJ_BLOCK, 0, st>>>(mu, v, Gs, Sh, a->gk, a->np, (int)ns, dt, lam, a->part);
            k_adj_reduce<<<a->np, ADJ_BLOCK, 0, st>>>(a->part, gb, a->np, gb, 1, a->gth, 1);
            s->launches += 2;
            ACK(cudaGetLastError());
        }
    }
    // leave the system in its final forward state, as add_sample! does
    ACK(cudaMemcpyAsync(s->S, a->ckpt + (size_t)nseg * st3, sizeof(double) * st3, cudaMemcpyDeviceToDevice, st));
    std::vector<double> gth(a->np);
    ACK(cudaMemcpyAsync(gth.data(), a->gth, sizeof(double) * a->np, cudaMemcpyDeviceToHost, st));
    std::vector<double> lh;
    if (grad_S0) {
        lh.resize(st3);
        ACK(cudaMemcpyAsync(lh.data(), lam, sizeof(double) * st3, cudaMemcpyDeviceToHost, st));
    }
    ACK(cudaStreamSynchronize(st));
    if (loss) *loss = Lsum / Nb;
    if (grad)
        for (int k = 0; k < a->np; k++) grad[k] = gth[k];
    if (grad_S0)
        for (size_t i = 0; i < ns; i++)
            for (int q = 0; q < 3; q++) grad_S0[3 * i + q] = lh[q * ns + i];
    return SGB_OK;
}

int sgb_adjoint_loss(sgb_adjoint* a, const double* S0, double* loss, double* data_out) {
    if (!a || !S0) return afail(a, SGB_ERR_ARG, "null argument");
    sgb_system* s = a->sys;
    sgb_corr* c = a->corr;
    if (!s) return afail(a, SGB_ERR_STATE, "the System of this adjoint was destroyed");
    cudaStream_t st = s->stream;
    int rc;
    if ((rc = sgb_set_state(s, S0, nullptr))) return rc;
    if ((rc = refresh_models(a))) return rc;
    const double scale = 1.0 / std::sqrt((double)c->ncell);
    const size_t nA = (size_t)c->nomega * c->nobs * c->npos * c->ncell;
    ACK(cudaMemsetAsync(c->A, 0, 16 * nA, st));
    SnapArgs<double> sn{1, c->nobs, c->measperiod, 0, (const double*)c->ops, (double*)c->A, scale};
    if ((rc = sgb_int_midpoint_snap(s, c->dt, c->tol, c->max_iters, c->measperiod * (c->nsnaps - 1), sn, nullptr))) return rc;
    if (cufftExecZ2Z(c->plan_space, (cufftDoubleComplex*)c->A, (cufftDoubleComplex*)c->A, CUFFT_INVERSE) != CUFFT_SUCCESS)
        return afail(a, SGB_ERR_CUDA, "space FFT failed");
    if (cufftExecZ2Z(c->plan_time, (cufftDoubleComplex*)c->A, (cufftDoubleComplex*)c->Ahat, CUFFT_FORWARD) != CUFFT_SUCCESS)
        return afail(a, SGB_ERR_CUDA, "time FFT failed");
    ACK(cudaMemsetAsync(c->P, 0, 16 * c->plen, st));
    if (corr_launch_accum<double>((const double*)c->Ahat, c->P, c->pairs, c->ncorr, c->nobs, c->npos, c->ncell, c->nomega,
                                  1, nA, st))
        return afail(a, SGB_ERR_CUDA, "accumulate launch");
    if (corr_launch_gather(c->P, a->ncols, 0, a->ncols, c->nomega, 1.0, a->data, st)) return afail(a, SGB_ERR_CUDA, "gather launch");
    s->launches += 2;
    if ((rc = apply_w(a, a->data))) return rc;
    if (data_out) {
        if (corr_launch_scatter(a->data, a->ncols, c->nomega, c->P, st)) return afail(a, SGB_ERR_CUDA, "scatter launch");
        ACK(cudaMemcpyAsync(data_out, c->P, 16 * c->plen, cudaMemcpyDeviceToHost, st));
    }
    const int gb = grid_of(c->plen);
    k_adj_loss<<<gb, ADJ_BLOCK, 0, st>>>((const double2*)a->data, (const double2*)a->target, c->plen, 0.0,
                                         (double2*)c->P, a->part);
    k_adj_reduce<<<1, ADJ_BLOCK, 0, st>>>(a->part, gb, 1, 0, 1, a->red, 0);
    s->launches += 2;
    double Lsum = 0;
    ACK(cudaMemcpyAsync(&Lsum, a->red, sizeof(double), cudaMemcpyDeviceToHost, st));
    ACK(cudaStreamSynchronize(st));
    if (loss) *loss = Lsum / (double)c->plen;
    return SGB_OK;
}

}  // extern "C"
