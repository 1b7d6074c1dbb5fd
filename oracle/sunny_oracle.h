/*
 * sunny_oracle.h -- TEST INFRASTRUCTURE ONLY. FP64 CPU restatement of Sunny.jl v0.9.2's
 * spin-dynamics hot path, used by tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline / reference arm as the checker. Nothing in the shipped library calls it.
 *
 * It follows the reference's own (scatter-form, per-sublattice) loop order so that it is
 * an independent check of the library's gather-form kernels. Parity is pinned against
 * the reference's RNG-independent known answers (sum rules, RCS factors, SU(N)/dipole
 * equivalence, energy conservation, kappa rescaling); the reference's one RNG-dependent
 * golden S(q,ω) vector needs Julia's Xoshiro stream and is not reproducible here.
 *
 * Data layout is that of include/sunny_gb300.h (Sunny's column-major arrays).
 */
#ifndef SUNNY_ORACLE_H
#define SUNNY_ORACLE_H
#include <stdint.h>
#include "../include/sunny_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int L[3];
    int na;
    int N;              /* 0 = dipole modes */
    int mode;           /* SGB_MODE_* */
    const double* kappa;   /* [ns]             */
    const double* g;       /* [ns][9] col-major */
    const double* field;   /* [ns][3] or NULL   */
    const double* onsite;  /* dipole: [na][28]; SU(N): [na][N*N][2] col-major */
    const sgb_bond* bonds; /* non-culled bonds  */
    int nbonds;
    /* Inhomogeneous systems (to_inhomogeneous, Interactions.jl:81-100), else NULL:
     * onsite couplings per site ([ns][28] or [ns][N*N][2]) and every site's non-culled
     * pair couplings, in the reference's site order (they replace `bonds`). */
    const double* onsite_site;
    const sgb_site_bond* site_bonds;
    int64_t nsite_bonds;
    /* SU(N) general pair couplings (Types.jl:23-30): term t = A[t] ⊗ B[t] on bonds[gen_bond[t]],
     * A, B [ngen][N][N] complex column-major (re, im). */
    const int* gen_bond;
    const double* gen_A;
    const double* gen_B;
    int ngen;
    /* Dipole-dipole matrices A[cell][i][j] (3x3 column-major, or_ewald_matrices) for the
     * Ewald term of local_energy_change (Ewald.jl:210-241), or NULL. */
    const double* ewA;
} or_sys;

int64_t or_nsites(const or_sys* s);

/* Interactions.jl:516-592 (dipole gradient, scatter form over non-culled bonds). */
void or_grad_dipoles(const or_sys* s, const double* S, double* grad);
/* Interactions.jl:596-669 (HZ = dE/dZbar). Z, HZ: [ns][N][2]. */
void or_grad_coherents(const or_sys* s, const double* Z, double* HZ);
/* Interactions.jl:401-508. S: dipoles [ns][3]; Z: coherents (SU(N) only, else NULL). */
double or_energy(const or_sys* s, const double* S, const double* Z);
/* OnsiteCoupling.jl:316-425 for one site: returns E, writes dE/dS. */
double or_classical_anisotropy(const double* c28, const double* S, double* grad3);
/* Spin.jl:72-87 */
void or_expected_spin(int N, const double* Z, double* S3);

/* Integrators.jl:313-332, one step. noise: [ns][3] standard normals or NULL (zero). */
void or_langevin_dipole(const or_sys* s, double* S, double dt, double damping, double kT,
                        const double* noise);
/* Integrators.jl:335-357, one step. Z [ns][N][2], S [ns][3] updated. noise: [ns][N][2]
 * complex normals with E|z|^2=1, or NULL. */
void or_langevin_sun(const or_sys* s, double* Z, double* S, double dt, double damping,
                     double kT, const double* noise);
/* Integrators.jl:379-413, one step; returns 0 or SGB_ERR_NOCONVERGE; *iters += count. */
int or_midpoint_dipole(const or_sys* s, double* S, double dt, double damping, double tol,
                       int max_iters, int64_t* iters);
/* Integrators.jl:422-452, one step. */
int or_midpoint_sun(const or_sys* s, double* Z, double* S, double dt, double damping,
                    double tol, int max_iters, int64_t* iters);

/* Multi-step drivers (noise: [nsteps][ns][...] or NULL). */
void or_langevin_steps(const or_sys* s, double* S, double* Z, double dt, double damping,
                       double kT, int nsteps, const double* noise);
int or_midpoint_steps(const or_sys* s, double* S, double* Z, double dt, double damping,
                      double tol, int max_iters, int nsteps, int64_t* iters);

/* Observables of one snapshot (CorrelationSampling.jl:1-19): out[nobs][ns] (real part;
 * the imaginary part is zero for Hermitian observables). obs as in sgb_corr_desc. */
void or_observables(const or_sys* s, const double* S, const double* Z, int nobs,
                    const double* obs, double* out);

/* local_energy_change (Interactions.jl:311-373), dipole modes: energy change if the dipole
 * at `site` became Snew. Pair terms of both bond directions: ΔS·J·S_j where the site is
 * the bond's first end, S_k·J·ΔS where it is the second. Returns NAN for a bond that
 * maps a site onto itself (the reference raises an error there). */
double or_local_energy_change(const or_sys* s, const double* S, int64_t site, const double* Snew);

/* LocalSampler updates (Samplers.jl:139-158, proposals System.jl:440-460, mixture
 * Samplers.jl:64-98) applied in a fixed order: for each of `nsweeps` sweeps, the sites
 * perm[0..ns) in turn; in the last sweep a site takes part only if its participation
 * uniform is below `frac` (frac >= 1: all). rand: [nsweeps][ns][6] = 3 standard normals,
 * mixture uniform, acceptance uniform, participation uniform, indexed by site. kind/cum/
 * mag: the mixture (cum = cumulative probabilities). dE, dS3 receive the sums of the
 * accepted changes. */
void or_local_sweeps(const or_sys* s, double* S, double kT, int nsweeps, double frac, const int* perm,
                     int nkind, const int* kind, const double* cum, const double* mag, const double* rand,
                     double* dE, double* dS3);

/* The same for SU(N) mode: Z [ns][N][2] kets, S [ns][3] their expected dipoles; Znew
 * [N][2]; rand [nsweeps][ns][2N+3] (N complex normals as (re, im), then the mixture,
 * acceptance and participation uniforms). Updates Z and S. */
double or_local_energy_change_sun(const or_sys* s, const double* S, const double* Z, int64_t site, const double* Znew);
void or_local_sweeps_sun(const or_sys* s, double* S, double* Z, double kT, int nsweeps, double frac, const int* perm,
                         int nkind, const int* kind, const double* cum, const double* mag, const double* rand,
                         double* dE, double* dS3);

/* Dipole-dipole Ewald matrices (Ewald.jl:40-146 precompute_dipole_ewald at q = 0):
 * A[cell][i][j] (3x3 column-major, cell = c1 + L1*(c2 + L2*c3) is the offset of atom j's
 * cell from atom i's), times mu0_muB2. latvecs: 3x3 column-major lattice vectors of the
 * unit cell; positions: [na][3] fractional; demag: 3x3 column-major. out: ncell*na*na*9. */
void or_ewald_matrices(int L1, int L2, int L3, int na, const double* latvecs, const double* positions,
                       const double* demag, double mu0_muB2, double* out);

/* Independent replicas stepped on a thread pool (OpenMP when compiled with it):
 * replica r has state S + r*ns*3 and temperature kT[r]; noise from the caller per
 * replica is not supported, the CPU path uses its own Gaussian source seeded by
 * (seed, r). Used only as the timed CPU baseline. Returns threads used. */
int or_langevin_replicas(const or_sys* s, int nrep, double* S, const double* kT, double dt,
                         double damping, int nsteps, uint64_t seed);

#ifdef __cplusplus
}
#endif
#endif
