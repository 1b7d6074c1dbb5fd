// sgb_internal.h -- host/device interface between the C ABI (sgb_api.cu) and the kernel
// translation units. Not installed; not part of the public ABI.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>
#include "sgb_common.cuh"

// Everything a kernel needs to evaluate couplings of one (homogeneous) system.
// The packed tables are copied into shared memory at kernel start.
template <class R>
struct Model {
    int L1, L2, L3, na;
    int ns;             // sites
    int ncell;          // L1*L2*L3
    int N;              // 0 in dipole modes
    int dipole_mode;    // 1 for :dipole / :dipole_uncorrected
    int has_biquad;     // any bond with a biquadratic coupling
    int general;        // any anisotropic (3x3) or biquadratic bond; 0 selects the isotropic fast path
    const R* kappa;     // [ns]
    const R* h;         // [3][ns] Zeeman g'B, or nullptr
    const unsigned char* tables;  // packed tables (device)
    const int* nbr;     // [kb][ns] neighbour table: site of the k-th bond of each site's sublattice
    int kb;             // rows of nbr: the most bonds of any sublattice
    int tables_bytes;
    // byte offsets inside the packed tables
    int off_stev;       // R[na][28]            (dipole)
    int off_kmax;       // int[na]              (dipole)
    int off_boff;       // int[na+1]
    int off_bonds;      // DBond<R>[nb]
    int off_bq;         // R[nbq][25]
    int off_lam;        // R[na][N*N][2]        (SU(N): Λ, column-major)
    int off_qmat;       // R[5][N*N][2]         (SU(N): Stevens quadrupoles)
    int nb, nbq;
    // Inhomogeneous systems (per-site couplings); nullptr where the per-sublattice tables
    // above apply. Bonds: site s owns entries ioff[s] .. ioff[s+1] of ient, each (neighbour
    // site, row of ctab); ctab rows hold both directions (the reversed copy has J^T and
    // fwd = 0) and cbq their 5x5 biquadratic matrices. Onsite: oidx[s] is a row of otab
    // (dipole: 28 Stevens coefficients, with highest rank okmax[row]; SU(N): N*N*2 Λ).
    const int* ioff;
    const int2* ient;
    const DBond<R>* ctab;
    const R* cbq;
    const int* oidx;
    const R* otab;
    const int* okmax;
    // SU(N) general pair couplings: term rows of 4 N^2 values, [a (N^2)][A (N*N complex)][b (N^2)],
    // where <A> = a·ρ and <B> = b·ρ over the packed density ρ of a ket (sun_rho); rows of a
    // bond are given by DBond::gref (dbond_gidx, dbond_gcnt). has_general: any such row.
    const R* gtab;
    int has_general;
    int qrows;          // rows per site of the SU(N) multipole buffers: 5 quadrupoles, then ρ (N^2)
};

// Observable recording for SampledCorrelations trajectories.
template <class R>
struct SnapArgs {
    int enabled;
    int nobs;
    int measperiod;
    int t0;              // row of the first snapshot written by this launch
    const R* ops;        // dipole: [nobs][3][ns]; SU(N): [nobs][N*N][2][ns]
    R* buf;              // complex [n_all_omega][nobs][npos][ncell] (interleaved re,im)
    R scale;             // 1/sqrt(ncell)
};

// Tensor maps of the three padded midpoint-spin buffers of the cell-block batched
// midpoint kernel (sgb_batch_blk.cu).
struct BlkMaps {
    CUtensorMap m[3];
};

struct LaunchInfo {
    int grid, block, spt;
    size_t smem;
};

// ---- dipole kernels (sgb_dipole.cu) ----
template <class R>
int dip_launch_heun(const Model<R>& M, R* S, R* P, Ctrl* ctrl, int nsteps, double dt, double lam,
                    double noise_scale, uint64_t seed, uint64_t step0, const double* noise,
                    const LaunchInfo& li, cudaStream_t st);
template <class R>
int dip_launch_midpoint(const Model<R>& M, R* S, R* H, Ctrl* ctrl, int nsteps, double dt, double lam,
                        double atol2, int max_iters, const SnapArgs<R>& snap, const LaunchInfo& li,
                        cudaStream_t st, int order = 0);
template <class R>
int dip_launch_grad(const Model<R>& M, const R* S, double* grad, cudaStream_t st);
template <class R>
int dip_launch_energy(const Model<R>& M, const R* S, double* partials, int nblocks, cudaStream_t st);
template <class R>
int dip_max_blocks(int spt, int block, size_t smem, int* blocks_per_sm);
// Langevin for small dipole lattices held by one thread-block cluster (cs CTAs); returns
// SGB_ERR_ARG when the cluster cannot be scheduled
#define SGB_CLUSTER_BLOCK 256
#define SGB_CLUSTER_MAX 16
template <class R>
int dip_launch_heun_cluster(const Model<R>& M, R* S, int cs, int nsteps, double dt, double lam, double noise_scale,
                            uint64_t seed, uint64_t step0, const double* noise, cudaStream_t st);
template <class R>
size_t dip_cluster_smem(const Model<R>& M, int nsl);
// one snapshot row t of the observables of dipoles S (SampledCorrelations trajectories
// outside the fused midpoint kernels)
template <class R>
int dip_launch_snapshot(const Model<R>& M, const R* S, const SnapArgs<R>& sn, int t, cudaStream_t st);
template <class R>
size_t sun_cluster_smem(const Model<R>& M, int nsl);
// hz ([ns][N][2]) += (f · S) Z for a per-site dipole field f ([ns][3], dE/dS)
template <class R>
int sun_launch_add_dipole_field(const Model<R>& M, const R* Z, const double* f, double* hz, cudaStream_t st);
// Stage kernels of SU(N) dynamics with dipole-dipole interactions (one launch per stage):
// 0 Heun predictor (Z, hz -> ZP, D1 increment, XI noise), 1 Heun corrector, 2 midpoint
// Zbar = (Z + ZP)/2 into D1, 3 midpoint update of ZP from hz with partial sums in part,
// 4 midpoint acceptance Z = normalize(ZP), 5 snapshot row t of Z.
template <class R>
int sun_launch_lr_stage(int stage, const Model<R>& M, R* Z, R* ZP, R* D1, R* XI, const double* hz, double dt, double lam,
                        double nscale, uint64_t seed, uint64_t step, const double* noise, double* part,
                        const SnapArgs<R>* sn, int t, cudaStream_t st);
template <class R>
int sun_launch_heun_cluster(const Model<R>& M, R* Z, R* D, R* Q, int cs, int nsteps, double dt, double lam, double nscale,
                            uint64_t seed, uint64_t step0, const double* noise, cudaStream_t st);

// ---- SU(N) kernels (sgb_sun.cu) ----
template <class R>
int sun_launch_heun(const Model<R>& M, R* Z, R* D, R* Q, R* P, R* QP, Ctrl* ctrl, int nsteps,
                    double dt, double lam, double noise_scale, uint64_t seed, uint64_t step0,
                    const double* noise, const LaunchInfo& li, cudaStream_t st);
template <class R>
int sun_launch_midpoint(const Model<R>& M, R* Z, R* D, R* Q, R* H, R* QH, Ctrl* ctrl, int nsteps,
                        double dt, double lam, double atol2, int max_iters, const SnapArgs<R>& snap,
                        const LaunchInfo& li, cudaStream_t st);
template <class R>
int sun_launch_refresh(const Model<R>& M, const R* Z, R* D, R* Q, cudaStream_t st);
template <class R>
int sun_launch_grad(const Model<R>& M, const R* Z, const R* D, const R* Q, double* grad, cudaStream_t st);
template <class R>
int sun_launch_energy(const Model<R>& M, const R* Z, const R* D, const R* Q, double* partials,
                      int nblocks, cudaStream_t st);
template <class R>
int sun_max_blocks(int N, int spt, int block, size_t smem, int* blocks_per_sm);

// ---- LocalSampler (sgb_mc.cu) ----
#define SGB_MC_MAXCOL 64       // colour classes of the bond-graph colouring
struct McArgs {
    const int* perm;             // [ns] sites ordered by colour class, ascending within a class
    int coff[SGB_MC_MAXCOL + 1]; // class c is perm[coff[c] .. coff[c+1])
    int ncol;
    int nsweeps;                 // sweeps, the last one partial when frac < 1
    double frac;                 // participation probability of the last sweep
    double kT;
    int nkind;                   // proposal mixture (sgb_proposal)
    int kind[4];
    double cum[4];               // cumulative probabilities
    double mag[4];
    uint64_t seed, sweep0;
    const double* rnd;           // injected randoms [nsweeps][ns][6] or nullptr
};
template <class R>
int mc_launch_sweeps(const Model<R>& M, R* S, Ctrl* ctrl, const McArgs& A, int grid, double* partials,
                     cudaStream_t st);
template <class R>
int mc_max_blocks(size_t smem, int* blocks_per_sm);
template <class R>
int mc_launch_local_dE(const Model<R>& M, const R* S, int site, double nx, double ny, double nz, double* out,
                       cudaStream_t st);
struct SunKet { double v[10]; };   // one coherent state, (re, im) per component, N <= 5
template <class R>
int sun_launch_local_sweeps(const Model<R>& M, R* Z, R* D, R* Q, Ctrl* ctrl, const McArgs& A, int grid, double* part,
                            cudaStream_t st);
template <class R>
int sun_mc_max_blocks(const Model<R>& M, int* bps);
template <class R>
int sun_launch_local_dE(const Model<R>& M, const R* Z, const R* D, const R* Q, int site, const SunKet& zk, double* out,
                        cudaStream_t st);

// ---- minimize_energy! vector kernels (sgb_opt.cu), FP64 state ----
// K reals per site: 3 (dipoles) or 2N (coherent states as (re, im)); vectors SoA [K][ns],
// gradients AoS [ns][K]
int opt_grid(int ns);   // blocks of every partial-writing kernel below
int opt_launch_init(int K, double* S, const double* kappa, int ns, double jitter, uint64_t seed, double* x, cudaStream_t st);
int opt_launch_point(int K, const double* x, const double* d, double alpha, const double* kappa, int ns, double* S,
                     cudaStream_t st);
int opt_launch_dphi(int K, const double* x, const double* d, double alpha, const double* grad, const double* kappa, int ns,
                    double* part, cudaStream_t st);
int opt_launch_accept(int K, double* x, double* d, double alpha, const double* grad, const double* kappa, int ns, double* g,
                      double* part, cudaStream_t st);
int opt_launch_dir(int K, const double* g, double* d, double beta, int ns, double* part, cudaStream_t st);

// ---- dipole-dipole Ewald summation (sgb_ewald.cu) ----
#include <cufft.h>
struct EwaldGeom {
    int L[3], na;
    double lat[9], sup[9], rec[9];   // column-major: unit cell, supercell, supercell reciprocals
    double demag[9];
    double V, sig, rmax, kmax, mu0;
    int nmax[3], mmax[3];
};
struct EwaldDev {
    int L[3], na, nm;                // nm = L3*L2*(L1/2+1) complex cells
    double* g = nullptr;             // [ns][9] column-major g tensors
    double* mu = nullptr;            // [na][3][ncell]
    double* phi = nullptr;           // [na][3][ncell]
    cufftDoubleComplex* FA = nullptr;    // [na*na*9][nm]
    cufftDoubleComplex* Fmu = nullptr;   // [na*3][nm]
    cufftDoubleComplex* Fphi = nullptr;  // [na*3][nm]
    cufftHandle plan_f = 0, plan_b = 0;
    bool have_f = false, have_b = false;
    double* Areal = nullptr;         // [na*na*9][ncell] pair matrices A (LocalSampler updates)
};
#define EWALD_PART_BLOCKS 256
// out[0] += ewald_energy_delta (Ewald.jl:230-241) for the dipole at `site` changing by dS;
// S: dipoles (expected dipoles in SU(N) mode) [3][ns]
template <class R>
int ewald_launch_delta(const EwaldDev& E, const R* S, int site, const double* dS3, double* out, cudaStream_t st);
// LocalSampler sweeps of a dipole system with dipole-dipole interactions: every update in
// sequence (the term couples every pair of sites), the Ewald field F ([ns][3], dE/dS of the
// term) kept current by a rank-one update after each accepted move; one CTA
template <class R>
int mc_launch_sweeps_ewald(const Model<R>& M, R* S, const McArgs& A, const EwaldDev& E, double* F, double* partials,
                           cudaStream_t st);
// SU(N) LocalSampler with dipole-dipole: sequential proposals in A.perm order in one CTA
template <class R>
int sun_launch_local_sweeps_ewald(const Model<R>& M, R* Z, R* D, R* Q, const McArgs& A, const EwaldDev& E, double* F,
                                  double* part, cudaStream_t st);
int ewald_precompute(const EwaldGeom& G, const double* pos_d, double* A, cudaStream_t st);
// adds the Ewald gradient into grad_aos ([ns][3], may be null) and writes EWALD_PART_BLOCKS
// energy partials into part (may be null)
template <class R>
int ewald_apply(const EwaldDev& E, const R* S, double* grad_aos, double* part, cudaStream_t st);

// integrator stages used when long-range terms need a global transform per gradient
template <class R>
int lr_heun_a(const R* S, const double* grad, R* P, R* D1, R* XI, const R* kappa, int ns, double dt, double lam,
              double nscale, uint64_t seed, uint64_t step, const double* noise, cudaStream_t st);
template <class R>
int lr_heun_b(R* S, const R* P, const double* grad, const R* D1, const R* XI, const R* kappa, int ns, double dt,
              double lam, cudaStream_t st);
template <class R>
int lr_mid_half(const R* S, const R* Sp, R* H, const R* kappa, int ns, cudaStream_t st);
template <class R>
int lr_mid_update(const R* S, const R* H, const double* grad, R* Sp, int ns, double dt, double lam, double* part,
                  cudaStream_t st);
template <class R>
int lr_mid_accept(R* S, const R* Sp, const R* kappa, int ns, cudaStream_t st);

// ---- shared utilities (sgb_dipole.cu) ----
int util_launch_reduce(const double* partials, int n, int ncomp, double* out, cudaStream_t st);
template <class R>
int util_launch_noise_export(int mode_sun, int N, int ns, uint64_t seed, uint64_t step, double* out,
                             cudaStream_t st);
int util_launch_fill(double* p, size_t n, double v, cudaStream_t st);
int util_launch_wait_probe(Ctrl* ctrl, int grid, cudaStream_t st);

#define SGB_ENERGY_BLOCKS 256
#define SGB_BLOCK 256          // block size of the non-persistent kernels
#define SGB_MAXBLOCK 512       // largest block of any persistent kernel

// Largest block of a persistent kernel: 512 threads (128 registers each) only where the
// kernel fits that budget without spilling (FP32 dipole, SPT <= 2), else 256.
constexpr int sgb_maxblock(bool dbl, bool sun, int spt) { return (!dbl && !sun && spt <= 2) ? 512 : 256; }
#define SGB_GATHER 8           // neighbour loads issued per gather chunk
