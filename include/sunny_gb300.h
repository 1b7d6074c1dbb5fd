/*
 * sunny_gb300.h -- C ABI of libsunnygb300.so, the GB300 (sm_103a) spin-dynamics
 * library that a Sunny.jl package extension binds with `ccall`.
 *
 * The library replaces, for one `System`, the hot path of Sunny.jl v0.9.2:
 *   - the local energy gradient   src/System/Interactions.jl:516-669
 *   - the total energy            src/System/Interactions.jl:401-508
 *   - step!(sys, ::Langevin)      src/Integrators.jl:313-357
 *   - step!(sys, ::ImplicitMidpoint) src/Integrators.jl:379-452
 *   - add_sample!(sc, sys)        src/SampledCorrelations/CorrelationSampling.jl:1-180
 *   - merge_correlations          src/SampledCorrelations/SampledCorrelations.jl:128-142
 *   - replica exchange            src/MonteCarlo/ParallelTempering.jl:40-95
 *
 * Conventions (all chosen so that Julia arrays can be passed without copies):
 *   - Sites are ordered as Sunny's 4-D arrays (L1, L2, L3, natoms), column-major:
 *     site = c1 + L1*(c2 + L2*(c3 + L3*atom)), all indices 0-based here.
 *   - dipoles:   double[nsites][3]            (Array{Vec3,4})
 *   - coherents: double[nsites][N][2] (re,im) (Array{CVec{N},4})
 *   - 3x3, 5x5 and NxN matrices are COLUMN-MAJOR, as Julia stores Mat3/Mat5/Matrix.
 *   - Host buffers are owned by the caller; the library copies in and out and never
 *     keeps a host pointer. Device memory is owned by the handle.
 *   - Every entry point returns SGB_OK (0) or a negative SGB_ERR_* code; the message
 *     is available from sgb_last_error(handle) (or sgb_last_error(NULL) when no handle
 *     exists yet).
 *   - A handle is not thread safe (like a Sunny `System`): use one handle per thread.
 *     Each handle owns one CUDA stream.
 */
#ifndef SUNNY_GB300_H
#define SUNNY_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------- */
#define SGB_OK               0
#define SGB_ERR_ARG         -1  /* invalid argument (Julia: error(...) in constructors)   */
#define SGB_ERR_CUDA        -2  /* a CUDA runtime / cuFFT call failed                       */
#define SGB_ERR_NOCONVERGE  -3  /* implicit midpoint did not converge (Integrators.jl:412,451) */
#define SGB_ERR_TIMEOUT     -4  /* a bounded device-side wait gave up (no Julia analogue)     */
#define SGB_ERR_STATE       -5  /* call order violated (e.g. no couplings set)               */
#define SGB_ERR_NOMEM       -6  /* device allocation failed                                  */

/* ---- system modes and precisions ------------------------------------------ */
#define SGB_MODE_DIPOLE              0  /* :dipole              (System.jl:43-45) */
#define SGB_MODE_DIPOLE_UNCORRECTED  1  /* :dipole_uncorrected                   */
#define SGB_MODE_SUN                 2  /* :SUN                                   */

#define SGB_FP64  0  /* plain FP64 state and arithmetic                          */
#define SGB_FP32  1  /* FP32 state and arithmetic, FP64 reductions/accumulators   */

typedef struct sgb_system sgb_system;   /* one Sunny `System` resident on the GPU   */
typedef struct sgb_corr   sgb_corr;     /* one `SampledCorrelations` accumulator    */
typedef struct sgb_batch  sgb_batch;    /* many independent replicas (tempering)    */

typedef struct {
    int32_t dims[3];      /* supercell dimensions L1, L2, L3 (System.jl:33, `dims`)   */
    int32_t natoms;       /* atoms per cell                                          */
    int32_t N;            /* 0 in dipole modes; N = 2s+1 >= 2 in SU(N) mode            */
    int32_t mode;         /* SGB_MODE_*                                                */
    int32_t precision;    /* SGB_FP64 or SGB_FP32                                      */
    int32_t device;       /* CUDA ordinal                                              */
} sgb_desc;

/* One pair coupling, as Sunny's PairCoupling (src/System/Types.jl:46-66). Pass only the
 * non-culled couplings (isculled == false); the library adds the reversed copy with the
 * transposed coupling itself, as Sunny does when it propagates a bond
 * (src/System/PairExchange.jl:228-236, 466-467). */
typedef struct {
    int32_t i, j;         /* 0-based atom (sublattice) indices                         */
    int32_t n[3];         /* cell offset of atom j                                     */
    double  scalar;       /* constant shift (Types.jl:56)                              */
    double  bilin[9];     /* 3x3 column-major bilinear J: E += S_i' J S_j              */
    int32_t biquad_kind;  /* 0 none, 1 scalar (isotropic, uses scalar_biquad_metric),
                             2 full 5x5 in the Stevens quadrupole basis                */
    double  biquad[25];   /* kind 1: biquad[0]; kind 2: 5x5 column-major               */
} sgb_bond;

/* One pair coupling of an inhomogeneous system (to_inhomogeneous,
 * src/System/Interactions.jl:81-100): the non-culled PairCoupling held in the coupling
 * list of site (cell, bond.i). Couplings set with set_exchange_at! / set_pair_coupling_at!
 * (src/System/PairExchange.jl:447-534) are stored from both sites like every other bond,
 * so pass only the non-culled copy; the library adds the reversed copy itself. */
typedef struct {
    int32_t  cell[3];     /* 0-based cell of the bond's first site; its atom is bond.i  */
    int32_t  pad;
    sgb_bond bond;        /* the coupling as seen from that site (raw cell offset n)    */
} sgb_site_bond;

/* ---- system lifetime ------------------------------------------------------- */

/* Replaces System(...) construction of buffers (src/System/System.jl:33-93). */
int  sgb_create(const sgb_desc* desc, sgb_system** out);
void sgb_destroy(sgb_system* sys);
/* Last error message for `sys`, or the process-wide message when sys == NULL. */
const char* sgb_last_error(const sgb_system* sys);
/* Number of sites L1*L2*L3*natoms. */
int64_t sgb_nsites(const sgb_system* sys);

/* Per-site data: kappa[ns] (Types.jl:116 `κs`), g[ns][9] column-major (`gs`),
 * field[ns][3] (`extfield`, already scaled by the Bohr magneton,
 * Interactions.jl:210-229). `field` may be NULL (zero field). */
int sgb_set_sites(sgb_system* sys, const double* kappa, const double* g, const double* field);

/* Onsite coupling of one sublattice (src/System/OnsiteCoupling.jl:1-41).
 * Dipole modes: `coeffs` = 28 renormalised Stevens coefficients c0[1], c2[5], c4[9], c6[13],
 * each in descending q (Types.jl:4-10). SU(N) mode: `coeffs` = NxN Hermitian matrix,
 * column-major, interleaved (re,im). */
int sgb_set_onsite(sgb_system* sys, int32_t atom, const double* coeffs);

/* Replaces the whole pair-coupling table (Interactions.jl:1-42 `repopulate_couplings…`).
 * The per-sublattice table replaces any per-site table of sgb_set_bonds_at. */
int sgb_set_bonds(sgb_system* sys, const sgb_bond* bonds, int32_t nbonds);

/* General pair couplings of SU(N) mode: the tensor decomposition Σ_k A_k ⊗ B_k of a
 * PairCoupling (`general`, src/System/Types.jl:23-30), which adds Σ_k <A_k>_i <B_k>_j to the
 * energy (Interactions.jl:495-503) and (A_k Z_i) <B_k>_j, <A_k>_i (B_k Z_j) to HZ
 * (Interactions.jl:660-666). Term t belongs to bonds[bond[t]] of the last sgb_set_bonds
 * call (seen from its atom i; the library stores the reversed copy with A and B swapped,
 * as reverse(tensordec) does); A and B: [nterms][N][N] complex, column-major, (re, im)
 * interleaved, Hermitian. nterms = 0 removes every general term. Per-sublattice systems
 * only: a system with per-site couplings (sgb_set_bonds_at) returns SGB_ERR_ARG. */
int sgb_set_general(sgb_system* sys, const int32_t* bond, int32_t nterms, const double* A, const double* B);

/* Inhomogeneous pair couplings: every site's own list, as Sunny keeps it after
 * to_inhomogeneous (Interactions.jl:81-100) and edits it with set_exchange_at!,
 * set_pair_coupling_at! (PairExchange.jl:447-534), set_vacancy_at! (Interactions.jl:237-257)
 * and remove_periodicity!. `bonds` lists the non-culled couplings of all sites in any
 * order; neighbours are bonded_site(site, bond) with the periodic wrap (System.jl:204-212).
 * Replaces the per-sublattice table until the next sgb_set_bonds. Energy, gradient,
 * Langevin, the implicit midpoint, SampledCorrelations, LocalSampler and
 * minimize_energy use the per-site lists; replica batches and the adjoint return
 * SGB_ERR_ARG for such a system. */
int sgb_set_bonds_at(sgb_system* sys, const sgb_site_bond* bonds, int64_t nbonds);

/* Per-site onsite couplings (set_onsite_coupling_at!, OnsiteCoupling.jl:222-231):
 * coeffs[ns][28] renormalised Stevens coefficients (dipole modes) or [ns][N*N][2] Λ
 * (SU(N) mode), in site order. Replaces the per-sublattice onsite couplings until the
 * next sgb_set_onsite. */
int sgb_set_onsite_at(sgb_system* sys, const double* coeffs);

/* enable_dipole_dipole!(sys, μ0_μB²; demag) (Interactions.jl:180-188, Ewald.jl:1-207):
 * Ewald-summed dipole-dipole energy E = μ (A ⋆ μ)/2 with μ = -g S over the
 * periodic supercell. latvecs: unit-cell lattice vectors as the columns of a 3x3
 * column-major matrix; positions: [natoms][3] fractional; demag: 3x3 column-major
 * demagnetisation tensor. mu0_muB2 = 0 disables. Call after sgb_set_sites. Energy,
 * gradient, Langevin, implicit midpoint, SampledCorrelations trajectories and
 * minimize_energy then include the term (the integrators run one launch per stage, since
 * each gradient needs a transform over the whole lattice); LocalSampler, batches and the
 * adjoint return SGB_ERR_ARG. In SU(N) mode (S = expected dipoles) energy, gradient and
 * minimize_energy include it and the integrators return SGB_ERR_ARG. */
int sgb_set_dipole_dipole(sgb_system* sys, double mu0_muB2, const double* demag, const double* latvecs,
                          const double* positions);

/* ---- state ------------------------------------------------------------------ */

/* Copy the spin state in. Dipole modes read `dipoles` (coherents may be NULL);
 * SU(N) mode reads `coherents` and recomputes dipoles = expected_spin(Z)
 * (src/Operators/Spin.jl:72-87). Values are used as given (no renormalisation). */
int sgb_set_state(sgb_system* sys, const double* dipoles, const double* coherents);
/* Copy the spin state out (either pointer may be NULL). */
int sgb_get_state(sgb_system* sys, double* dipoles, double* coherents);

/* ---- the hot path ---------------------------------------------------------- */

/* set_energy_grad_dipoles! (Interactions.jl:516-592) in dipole modes, or
 * set_energy_grad_coherents! (Interactions.jl:596-669) in SU(N) mode, evaluated on the
 * current state. grad: double[ns][3] (dipole) or double[ns][N][2] (SU(N)). */
int sgb_energy_grad(sgb_system* sys, double* grad);

/* sgb_energy_grad without any device allocation (no counterpart in the reference).
 * For callers that may not allocate device memory: a host whose device memory is owned
 * by its own pool allocator or capped by a fixed budget, or a loop that must stay out of
 * the allocator. The gradient goes through one 8 MiB static device array (2^20 doubles) per
 * device, shared by every call: systems needing more (3 doubles per dipole site, 2N per
 * SU(N) site, plus 3 per SU(N) site with dipole-dipole interactions) get SGB_ERR_ARG;
 * calls must not overlap (issue them one after another). Dipole-dipole interactions are
 * included as in sgb_energy_grad. The caller's current device is left unchanged.
 * The state must be set after the last coupling change (else SGB_ERR_STATE). The first
 * call on a device resolves the array's address; make it before any stream capture. */
int sgb_energy_grad_static(sgb_system* sys, double* grad);

/* First fixed-point iterate of each dipole-mode midpoint step within one sgb_midpoint /
 * sgb_corr_add_sample call (no counterpart in the reference, which starts from S' = S,
 * Integrators.jl:389): order 0 does the same; order k in 1..4 starts from the degree-k
 * extrapolation of the last states and accepts a step from its second iteration on (same
 * convergence test, fewer iterations; used when a thread holds 1 or 2 sites). Default 4
 * for FP32 dipole systems, 0 otherwise; SU(N) mode always starts from Z' = Z. */
int sgb_set_midpoint_predictor(sgb_system* sys, int32_t order);

/* energy(sys) (Interactions.jl:401-432) in FP64, and the magnetisation sum(sys.dipoles)
 * (ParallelTempering.jl:31). Either output may be NULL. */
int sgb_energy(sgb_system* sys, double* energy, double* magnetization3);

/* `nsteps` x step!(sys, Langevin(dt; damping, kT)) (Integrators.jl:313-357).
 * noise == NULL: standard normals come from a counter-based generator keyed by
 *   (seed, step0 + k, site, component); `step0` lets a caller continue a stream.
 * noise != NULL: caller-supplied standard normals for every step, laid out
 *   [nsteps][ns][3] (dipole) or [nsteps][ns][N][2] (SU(N): complex normals with
 *   E|z|^2 = 1, i.e. randn(ComplexF64)); they are scaled by sqrt(2 dt damping kT)
 *   exactly as fill_noise! does (Integrators.jl:288-298). */
int sgb_langevin(sgb_system* sys, double dt, double damping, double kT,
                 uint64_t seed, uint64_t step0, int32_t nsteps, const double* noise);

/* Kernel choice of sgb_langevin on dipole lattices (no counterpart in the reference).
 * Small lattices can be held whole by one thread-block cluster in distributed shared
 * memory, where a Heun stage ends at the cluster's hardware barrier instead of a grid
 * barrier. mode -1 (default): time both kernels on the first call and keep the faster;
 * 0: the persistent grid kernel; 1: the cluster kernel (SGB_ERR_ARG if the lattice does
 * not fit one cluster). Both give the same results. */
int sgb_set_langevin_cluster(sgb_system* sys, int32_t mode);

/* The Langevin kernel in use (no counterpart in the reference): *cluster = -1 before the
 * first timed choice, 0 for the persistent grid kernel, c > 0 for the cluster kernel on a
 * cluster of c CTAs. */
int sgb_langevin_kernel(const sgb_system* sys, int32_t* cluster);

/* Writes the standard normals that sgb_langevin(noise=NULL) uses for step `step`
 * into out ([ns][3] or [ns][N][2]), so that an FP64 CPU restatement can replay a
 * device-noise trajectory exactly. */
int sgb_langevin_noise(sgb_system* sys, uint64_t seed, uint64_t step, double* out);

/* `nsteps` x step!(sys, ImplicitMidpoint(dt; damping, tol)) with kT = 0
 * (Integrators.jl:379-452). Convergence test: sum over sites |S'-S''|^2 <= (tol*sqrt(ns))^2,
 * accumulated in FP64 (Integrators.jl:361-371, 383, 426). On non-convergence after
 * `max_iters` iterations the step that failed leaves the state unchanged and
 * SGB_ERR_NOCONVERGE is returned. iters_out (nullable) receives the total number of
 * fixed-point iterations performed. */
int sgb_midpoint(sgb_system* sys, double dt, double damping, double tol, int32_t max_iters,
                 int32_t nsteps, int64_t* iters_out);

/* ---- LocalSampler (MonteCarlo/Samplers.jl) ----------------------------------- */

#define SGB_PROPOSE_UNIFORM 0   /* propose_uniform = randspin (Samplers.jl:14, System.jl:444-447)   */
#define SGB_PROPOSE_FLIP    1   /* propose_flip: S -> -S (Samplers.jl:23, System.jl:440-442)        */
#define SGB_PROPOSE_DELTA   2   /* propose_delta(magnitude) (Samplers.jl:46-48, System.jl:454-460)  */

/* A proposal function, or a @mix_proposals of up to 4 (Samplers.jl:64-98): kind i is
 * chosen with probability weight[i] / sum(weight). magnitude[i] is used by
 * SGB_PROPOSE_DELTA (INFINITY selects propose_uniform, as perturbed_spin does). */
typedef struct {
    int32_t n;
    int32_t kind[4];
    double  weight[4];
    double  magnitude[4];
} sgb_proposal;

/* step!(sys, LocalSampler(; kT, nsweeps, propose)) (Samplers.jl:139-158), dipole and SU(N)
 * modes.
 * Sunny proposes ceil(nsweeps*ns) updates at uniformly drawn sites; here one sweep
 * visits every site once, colour class by colour class of a greedy colouring of the
 * bond graph (sites of one class share no coupling and are updated in parallel), so
 * each sweep is a sequence of exact single-spin Metropolis updates and the chain has
 * the same stationary distribution. A fractional nsweeps adds one sweep in which every
 * site takes part with probability nsweeps - floor(nsweeps). Acceptance: ΔE <= 0 at
 * kT = 0, else u <= exp(-ΔE/kT) with ΔE = local_energy_change.
 * rand == NULL: random numbers from a counter-based generator keyed by
 *   (seed, sweep0 + k, site); rand != NULL: caller-supplied, [nsweeps_total][ns][6]
 *   = (3 standard normals, mixture uniform, acceptance uniform, participation uniform);
 *   in SU(N) mode [nsweeps_total][ns][2N+3] = (N complex normals with E|z|^2 = 1 as
 *   (re, im), then the three uniforms). SU(N) proposals: randspin (System.jl:448-452),
 *   flip_ket (Spin.jl:121-128), perturbed_spin (System.jl:461-468).
 * dE (nullable) receives the summed energy change of the accepted updates and dS3
 * (nullable) the summed dipole change: the sampler's ΔE and ΔS (Samplers.jl:153-156). */
int sgb_local_sweeps(sgb_system* sys, double kT, double nsweeps, const sgb_proposal* propose,
                     uint64_t seed, uint64_t sweep0, const double* rand, double* dE, double* dS3);

/* The colouring used by sgb_local_sweeps: *ncolors classes, color (nullable) [ns]. */
int sgb_local_colors(sgb_system* sys, int32_t* ncolors, int32_t* color);

/* local_energy_change(sys, site, state) (Interactions.jl:311-373): the energy change if
 * the state at `site` (0-based, Sunny's linear order) became S_new: a dipole [3] in dipole
 * modes, a coherent state [N][2] in SU(N) mode. */
int sgb_local_energy_change(sgb_system* sys, int64_t site, const double* S_new, double* dE);

/* minimize_energy!(sys; maxiters, jitter) (Optimization.jl:102-166), dipole and SU(N)
 * modes, FP64 systems: perturb every spin by `jitter` (perturbed_spin with normals keyed by seed),
 * then conjugate-gradient descent on the unit spheres until the largest gradient
 * component is <= 1e-12 * characteristic_energy_scale or the largest step component is
 * <= 1e-12. The state is left at the minimiser; converged/niters/energy_out (nullable)
 * receive the MinimizationResult fields. */
int sgb_minimize_energy(sgb_system* sys, int32_t maxiters, double jitter, uint64_t seed, int32_t* converged,
                        int32_t* niters, double* energy_out);

/* ---- SampledCorrelations --------------------------------------------------- */

typedef struct {
    int32_t nobs;          /* observables per site (3 for ssf_*: MeasureSpec.jl:53-76)       */
    const double* obs;     /* dipole: [nobs][ns][3] row vectors (op . S);
                              SU(N): [nobs][ns][N*N][2] column-major Hermitian matrices     */
    int32_t ncorr;         /* number of correlation pairs (6 for ssf_*: MeasureSpec.jl:117)  */
    const int32_t* pairs;  /* [ncorr][2] 0-based observable pairs (alpha, beta)              */
    int32_t n_all_omega;   /* 2(nω-1)  (SampledCorrelations.jl:157, 207)                    */
    int32_t measperiod;    /* steps between snapshots (SampledCorrelations.jl:163)           */
    double  dt;            /* adjusted integrator time step (SampledCorrelations.jl:164)     */
    double  damping;       /* ImplicitMidpoint damping (0 by default)                        */
    double  tol;           /* ImplicitMidpoint tol                                           */
    int32_t max_iters;     /* 100 in Sunny                                                   */
    int32_t calculate_errors; /* keep the Welford M array (SampledCorrelations.jl:244): each
                                 sample is transformed and folded into the running mean and
                                 M (CorrelationSampling.jl:117-134) instead of summed        */
} sgb_corr_desc;

/* SampledCorrelations(sys; measure, energies, dt, integrator=ImplicitMidpoint)
 * (src/SampledCorrelations/SampledCorrelations.jl:199-269). The accumulator lives in
 * device memory and is tied to `sys`. */
int  sgb_corr_create(sgb_system* sys, const sgb_corr_desc* desc, sgb_corr** out);
void sgb_corr_destroy(sgb_corr* sc);

/* add_sample!(sc, sys; window) (CorrelationSampling.jl:156-176): integrates the
 * trajectory of the system the accumulator was created on (mutating it) and accumulates
 * one sample. window: 0 = :cosine, 1 = :rectangular. */
int sgb_corr_add_sample(sgb_corr* sc, int32_t window);

/* Reads sc.data as complex FP64, laid out exactly as Sunny's
 * Array{ComplexF64,7}(ncorr, npos, npos, L1, L2, L3, n_all_omega) column-major, i.e.
 * double[n_all_omega][L3][L2][L1][npos][npos][ncorr][2]. `M` (nullable; Float64 of the
 * same shape without the complex axis) is filled when calculate_errors was set.
 * nsamples may be NULL. Either array pointer may be NULL. */
int sgb_corr_data(sgb_corr* sc, double* data, double* M, int64_t* nsamples);

/* The phase-averaged, combined part of intensities(sc, qpts; energies, kT)
 * (DataRetrieval.jl:77-171, PhaseAveraging.jl), on the device. For nq wave vectors given
 * by their index in the accumulator's q grid, qidx[k] = m1 + L1 (m2 + L2 m3) with the
 * caller's rounding and wrapping (DataRetrieval.jl pruned_wave_vector_info), their
 * per-atom prefactors pref[k][npos][2] = form factor × exp(-2πi q·r_atom) (complex), and
 * nw energy indices widx into the n_all_omega axis, writes
 *   combiner 0: out[k][t] = tr Re S(q, ω)                        (ssf_trace)
 *   combiner 1: out[k][t] = tr Re S - q·Re S·q / |q|², 2/3 tr at q = 0 (ssf_perp, qcart[k][3])
 *   combiner 2: out[k][t][ncorr][2] = the phase-averaged correlation elements
 * Combiners 0 and 1 need the six ssf_* correlation pairs. The conversion to a density
 * (1/(n_all_omega Δω)) and the classical-to-quantum factor are left to the caller. */
int sgb_corr_intensities(sgb_corr* sc, int32_t nq, const int32_t* qidx, const double* pref, const double* qcart,
                         int32_t nw, const int32_t* widx, int32_t combiner, double* out);

/* merge_correlations([dst, src]) into dst (SampledCorrelations.jl:128-142), with M when
 * both were created with calculate_errors (mixing the two kinds is SGB_ERR_ARG). */
int sgb_corr_merge(sgb_corr* dst, const sgb_corr* src);
/* Statistical comparison of two accumulators of the same shape, both made with
 * calculate_errors and holding >= 2 samples (no counterpart in the reference; it states
 * the error of one sampling path against another). Per bin, Δ = mean_a − mean_b and
 * s = M_a/(n_a(n_a−1)) + M_b/(n_b(n_b−1)), the variance of Δ when both means estimate
 * one S(q,ω). out[9]: Σ|Δ|², Σs, Σs², Σ|mean_b|², Σ|mean_a|², the number of bins with
 * |Δ|² > 9s, the number with s > 0, the number of bins, and the variance of Σ(|Δ|² − s)
 * estimated from the spread of 1024 partial sums over interleaved bin sets. */
int sgb_corr_compare(const sgb_corr* a, const sgb_corr* b, double* out);
/* Systematic difference of two sampling paths from paired samples split into two
 * disjoint halves (no counterpart in the reference): a1/b1 hold the first half's samples
 * on paths a and b (from the same starts), a2/b2 the second half's, all with
 * calculate_errors. out[0] = Σ_bins Re[(a1 − b1)·conj(a2 − b2)], whose expectation is the
 * squared systematic difference summed over bins (the halves' noise is independent);
 * out[1] = Σ_bins |(b1 + b2)/2|²; out[2] = the variance of out[0] estimated from the spread
 * of its partial sums over interleaved bin sets. */
int sgb_corr_cross(const sgb_corr* a1, const sgb_corr* b1, const sgb_corr* a2, const sgb_corr* b2, double* out);
/* The time transform of add_sample! (CorrelationSampling.jl:65-69), no counterpart in the
 * reference: kind 0 (default) runs FP32 accumulators through the hand-written Bluestein
 * kernel whenever 512 < n_all_ω + n_all_ω/2 <= 1024 (its fixed 1024-point convolution),
 * kind 1 always uses cuFFT (FP64 accumulators and other lengths always do). sgb_corr_time_transform returns the kind in effect (0 own kernel, 1 cuFFT). */
int sgb_corr_set_time_transform(sgb_corr* sc, int32_t kind);
int sgb_corr_time_transform(const sgb_corr* sc);

/* Per-phase device time of add_sample!, summed over the samples taken while profiling is
 * on (CUDA events between phases; no Julia analogue): ms4[0] trajectory with snapshots,
 * [1] space FFT, [2] time FFT, [3] accumulation; iterations (nullable) receives the
 * implicit-midpoint fixed-point iterations of those samples. sgb_corr_profile(sc, 1)
 * enables and resets the sums. */
int sgb_corr_profile(sgb_corr* sc, int32_t enable);
int sgb_corr_phase_times(sgb_corr* sc, double* ms4, int64_t* nsamples_timed, int64_t* iterations);

/* ---- batched replicas and parallel tempering -------------------------------- */

/* Many independent dipole-mode replicas, each with its own dims, kT and state, stepped
 * together. Couplings (onsite + bonds) are shared by all replicas; dims differ.
 * dims: int32[nrep][3]; natoms, mode, precision from `proto`. */
int  sgb_batch_create(const sgb_desc* proto, int32_t nrep, const int32_t* dims, sgb_batch** out);
/* A replica group: a batch whose nrep (1..64) replicas are whole systems of one mode,
 * precision, device and dims, SU(N) included (the clones that Sunny's ParallelTempering
 * makes, ParallelTempering.jl:20-37; no counterpart for batched sampling). The systems
 * stay owned by the caller and must outlive the batch; their couplings and states are
 * set through the system entry points. Langevin (member r draws noise with seed + r),
 * energies and batched add_sample! run every member concurrently, each on its own stream
 * with an equal share of the SMs. Replica exchange over systems is done by the caller
 * (sgb_batch_exchange and sgb_batch_step_ensemble return SGB_ERR_ARG for a group). */
int  sgb_batch_create_group(sgb_system* const* systems, int32_t nrep, sgb_batch** out);
void sgb_batch_destroy(sgb_batch* b);
const char* sgb_batch_last_error(const sgb_batch* b);
int64_t sgb_batch_nsites(const sgb_batch* b, int32_t rep);
/* Couplings shared by every replica: kappa/g/field per sublattice ([natoms], [natoms][9],
 * [natoms][3]) plus onsite and bonds as for a single system. */
int sgb_batch_set_couplings(sgb_batch* b, const double* kappa, const double* g, const double* field,
                            const double* onsite /*[natoms][28]*/, const sgb_bond* bonds, int32_t nbonds);
int sgb_batch_set_state(sgb_batch* b, int32_t rep, const double* dipoles);
int sgb_batch_get_state(sgb_batch* b, int32_t rep, double* dipoles);
/* kT of every replica (the tempering ladder position is a property of the replica slot). */
int sgb_batch_set_kT(sgb_batch* b, const double* kT);
int sgb_batch_get_kT(sgb_batch* b, double* kT);
/* nsteps Langevin steps of every replica (each with its own kT), device noise keyed by
 * (seed, replica, step0 + k, site, component). */
int sgb_batch_langevin(sgb_batch* b, double dt, double damping, uint64_t seed, uint64_t step0, int32_t nsteps);
/* FP64 energy of every replica: E[nrep]. */
int sgb_batch_energy(sgb_batch* b, double* E);
/* One replica_exchange!(PT, exch_start) over replicas grouped by equal dims
 * (ParallelTempering.jl:40-73): within each group, ordered by kT, pairs
 * (r, r+1) for r = exch_start, exch_start+2, ... (1-based) attempt a swap of their
 * kT with probability min(1, exp((E1-E2)(1/kT1-1/kT2))). Uniforms come from
 * `uniforms` ([nrep], nullable -> device generator keyed by (seed, round)).
 * n_accept (nullable, int64[nrep]) accumulates accepted swaps per lower slot. */
int sgb_batch_exchange(sgb_batch* b, int32_t exch_start, uint64_t seed, uint64_t round,
                       const double* uniforms, int64_t* n_accept);
/* step_ensemble!(PT, nsteps, exch_interval) (ParallelTempering.jl:80-95): cld(nsteps,
 * exch_interval) rounds of exch_interval Langevin steps, FP64 energies and one exchange
 * (round i uses exch_start = i % 2 + 1), captured once as a CUDA graph and replayed.
 * Langevin noise continues from the step counter of the last sgb_batch_langevin call. */
int sgb_batch_step_ensemble(sgb_batch* b, double dt, double damping, uint64_t seed,
                            int32_t nsteps, int32_t exch_interval, int64_t* n_accept);
/* 1 if the last step_ensemble ran from a captured CUDA graph, 0 if it fell back to
 * direct launches. */
int sgb_batch_graph_active(const sgb_batch* b);
/* The standard normals that replica `rep` uses at Langevin step `step`: [ns][3]. */
int sgb_batch_langevin_noise(sgb_batch* b, int32_t rep, uint64_t seed, uint64_t step, double* out);

/* SampledCorrelations over a batch of equal-size replicas: each sgb_corr_add_sample call
 * integrates every replica's trajectory in one persistent launch and adds nrep samples
 * (the parallel add_sample! pattern of Sunny's docs/src/parallelism.md:82-125, merged
 * on device). The accumulator is then used with sgb_corr_data / merge / destroy. */
int sgb_batch_corr_create(sgb_batch* b, const sgb_corr_desc* desc, sgb_corr** out);
/* Launch shapes of the batched midpoint kernel (no counterpart in the reference). The
 * first batched add_sample after the couplings are set times every shape that fits on a
 * 3-step run and keeps the fastest. Writes up to `cap` rows of (neighbour-index bytes in
 * shared memory or 0 for the global table, bonds gathered together, CTAs per SM, grid,
 * dynamic shared bytes, kernel: 0 sublattice tiles or 1 cell blocks, cells per block and
 * threads per CTA as bx | by << 8 | bz << 16 | (threads / 32) << 24 for kernel 1) into
 * shapes[cap][7] and their tuning times into
 * ms[cap] (either may be NULL); *chosen = the row in use. Returns the number of shapes
 * (0 before the first batched add_sample). */
/* First fixed-point iterate of each batched midpoint step (no counterpart in the
 * reference, which starts from S' = S, Integrators.jl:389): order 0 does the same; order
 * k in 1..4 starts from the degree-k polynomial extrapolation of the last k+1 states,
 * which reaches the same convergence test (sum |S'-S''|^2 <= (tol sqrt(ns))^2) in fewer
 * iterations, so the result differs from order 0 only within the tolerance. Default:
 * 4 for FP32 batches, 0 for FP64 batches. */
int sgb_batch_set_midpoint_predictor(sgb_batch* b, int32_t order);
int sgb_batch_midpoint_shapes(const sgb_batch* b, int32_t cap, int32_t* shapes, float* ms, int32_t* chosen);
/* Uses row `row` of sgb_batch_midpoint_shapes for the following batched trajectories, or
 * -1 to time the shapes again at the next one (no counterpart in the reference). */
int sgb_batch_select_midpoint_shape(sgb_batch* b, int32_t row);
/* Replicas per launch of the batched midpoint trajectories of add_sample! (no counterpart
 * in the reference): the replicas of a batch run in launches of at most this many, so that
 * each launch's working set stays in L2, and one rank-nrep pass then accumulates every
 * replica's sample. 0 (default) sizes the launches for about 72 MB of working set (8
 * replicas of 65,536 FP32 sites), in equal chunks. */
int sgb_batch_set_midpoint_chunk(sgb_batch* b, int32_t replicas);
/* With an extrapolated first iterate (predictor order > 0), also apply the convergence
 * test Σ|S' − S''|² <= (tol √Ns)² to the first iteration, whose S' is the extrapolation,
 * so that a step can end after one iteration when the extrapolation is that good (no
 * counterpart in the reference, whose first iterate S' = S never passes). The next-step
 * data are then prepared at every iteration. Default off. */
int sgb_batch_set_midpoint_first_accept(sgb_batch* b, int32_t on);
/* The batched Langevin kernel's launch shapes (no counterpart in the reference): 4, 3 and
 * 2 CTAs per SM, timed once per couplings on 10 steps at the first Langevin call (FP32;
 * FP64 batches use 2). ms3[k] receives shape k's tuning time (0 not tried, 1e30 does not
 * fit), *chosen_bps the CTAs per SM in use (0 before tuning). Returns 3. */
int sgb_batch_langevin_shapes(const sgb_batch* b, float* ms3, int32_t* chosen_bps);

/* ---- adjoint: S(q,ω) loss gradient through a midpoint trajectory ------------ */
/* No reverse rule exists in the reference; parameters follow the labelled-parameter
 * convention of its fitting code (src/Fitting.jl:123-152, src/ModelParams.jl:140-150):
 * the energy is linear in them, E(θ) = E_rest + Σ_k θ_k E_k, and parameter k is given by
 * its unit coupling set E_k = (bonds of parameter k, onsite coefficients of parameter k).
 * The caller keeps the system's own couplings equal to the current θ (sgb_set_bonds /
 * sgb_set_onsite as usual). Supported: FP64 dipole-mode systems with bilinear pair
 * couplings and onsite anisotropy of rank <= 2, damping 0, one cosine-window sample.
 *
 * typedef of the handle: */
typedef struct sgb_adjoint sgb_adjoint;

/* `desc` as for sgb_corr_create (dt, measperiod, tol; damping must be 0). `bonds` holds
 * the unit bonds of every parameter back to back, nbonds[k] of parameter k; `onsite`
 * is [nparams][natoms][28] Stevens coefficients (or NULL). 1 <= nparams <= 8. */
int sgb_adjoint_create(sgb_system* sys, const sgb_corr_desc* desc, int32_t nparams, const sgb_bond* bonds,
                       const int32_t* nbonds, const double* onsite, sgb_adjoint** out);
void sgb_adjoint_destroy(sgb_adjoint* a);
const char* sgb_adjoint_last_error(const sgb_adjoint* a);
/* Target data in the layout of sgb_corr_data (complex [c,i,j,q1,q2,q3,ω], column-major). */
int sgb_adjoint_set_target(sgb_adjoint* a, const double* target);
/* From S0 (double[ns][3]): integrate measperiod*(nsnaps-1) midpoint steps recording
 * snapshots (add_sample!, CorrelationSampling.jl:1-139), form the sample's S(q,ω) and
 * loss = mean over all complex bins of |data - target|^2; then the discrete adjoint gives
 * grad[k] = dloss/dθ_k and (if not NULL) grad_S0[ns][3] = dloss/dS0. The trajectory is
 * checkpointed every `checkpoint` steps (rounded to whole measurement periods) and
 * recomputed segment by segment. data_out (may be NULL) receives the sample's S(q,ω).
 * Leaves the system in the final state of the trajectory. */
int sgb_adjoint_loss_grad(sgb_adjoint* a, const double* S0, int32_t checkpoint, double* loss, double* grad,
                          double* grad_S0, double* data_out);
/* The forward half only: loss (and data_out) of the sample from S0. */
int sgb_adjoint_loss(sgb_adjoint* a, const double* S0, double* loss, double* data_out);

/* ---- measurement helpers ---------------------------------------------------- */

/* CUDA-event timing on the handle's own stream: slot in [0, 8). */
int sgb_event_record(sgb_system* sys, int32_t slot);
int sgb_event_elapsed(sgb_system* sys, int32_t slot_a, int32_t slot_b, float* ms);
int sgb_batch_event_record(sgb_batch* b, int32_t slot);
int sgb_batch_event_elapsed(sgb_batch* b, int32_t slot_a, int32_t slot_b, float* ms);
/* Wait for all work queued on the handle's stream. */
int sgb_synchronize(sgb_system* sys);
/* Number of this library's own kernels launched on the handle so far (cuFFT excluded). */
int64_t sgb_kernel_launches(const sgb_system* sys);
int64_t sgb_batch_kernel_launches(const sgb_batch* b);
/* Wall-clock limit of the bounded waits (grid barriers) of this handle's persistent
 * kernels (no counterpart in the reference, which has no device waits). A wait that runs
 * past it makes the kernel record SGB_ERR_TIMEOUT and return, so the call fails with
 * SGB_ERR_TIMEOUT and the handle stays usable. seconds = 0 restores the default, 4 s. */
int sgb_set_wait_limit(sgb_system* sys, double seconds);
int sgb_batch_set_wait_limit(sgb_batch* b, double seconds);
/* Runs a grid barrier that expects one more CTA than it launches, so that it can only end
 * at the wait limit (no counterpart in the reference). Returns SGB_ERR_TIMEOUT with the
 * message of a timed-out barrier; lets callers check how their handle reports a wait that
 * gave up. */
int sgb_wait_probe(sgb_system* sys);
/* Writes a 256 MiB device buffer on the handle's stream to evict L2. */
int sgb_flush_l2(sgb_system* sys);
/* Library version string. */
const char* sgb_version(void);

#ifdef __cplusplus
}
#endif
#endif /* SUNNY_GB300_H */
