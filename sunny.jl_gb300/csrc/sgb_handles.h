// sgb_handles.h -- definitions of the opaque C-ABI handles (internal).
#pragma once
#include <cuda_runtime.h>
#include <cufft.h>
#include <string>
#include <vector>
#include "sgb_internal.h"


struct sgb_system {
    sgb_desc d{};
    int ns = 0, ncell = 0, N = 0;
    bool fp32 = false;
    bool sun = false;
    int mid_order = 0;          // first-iterate extrapolation of the dipole midpoint (0: S' = S)
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[8] = {};
    std::string err;
    long long launches = 0;
    int nsm = 0;
    // host copies of the model
    std::vector<double> kappa_h, g_h, field_h, onsite_h;
    std::vector<sgb_bond> bonds_h;
    bool sites_set = false, bonds_set = false, state_set = false;
    bool has_field = false, has_biquad = false;
    bool tables_dirty = true;
    // device data (element type R = float or double)
    void* kappa = nullptr;   // [ns]
    void* h = nullptr;       // [3][ns]
    void* tables = nullptr;
    int tables_bytes = 0;
    int* nbr = nullptr;             // neighbour table of the single system
    Model<float> mf{};
    Model<double> md{};
    // state buffers
    void* S = nullptr;   // dipole: spins [3][ns]; SU(N): dipoles [3][ns]
    void* P = nullptr;   // [3][ns]
    void* H = nullptr;   // [3][3][ns]
    void* Z = nullptr;   // SU(N) [2N][ns]
    void* Q = nullptr;   // SU(N) [5][ns]
    void* QP = nullptr;  // SU(N) [5][ns]
    void* QH = nullptr;  // SU(N) [3][5][ns]
    Ctrl* ctrl = nullptr;
    double* partials = nullptr;
    double* red = nullptr;
    double* dbuf = nullptr;     // device double scratch (noise, grads)
    size_t dbuf_cap = 0;
    void* flush = nullptr;
    char* stage = nullptr;      // pinned host staging
    size_t stage_cap = 0;
    std::vector<sgb_corr*> corrs;   // accumulators created on this system (detached on destroy)
    // LocalSampler: neighbour table on the host, the bond-graph colouring and its device copy
    std::vector<int> nbr_h, boff_h;   // [kb][ns] as nbr; bonds per sublattice offsets [na+1]
    std::vector<int> color_h, perm_h, coff_h;
    bool colors_dirty = true;
    int* mc_perm = nullptr;
    double* mc_part = nullptr;       // [grid][4] per-block ΔE, ΔS partials
    int mc_part_cap = 0;
    // dipole-dipole (Ewald) interactions, when enabled
    bool ewald_on = false;
    EwaldDev ew{};
    double* ew_part = nullptr;       // [EWALD_PART_BLOCKS] energy partials
    double* lr_grad = nullptr;       // [ns][3] gradient of the per-stage integrator path
    int lr_grad_cap = 0;
    void* lr_sun = nullptr;          // SU(N) per-stage scratch: HZ [ns][2N] FP64, kets ZP, D1, XI
    size_t lr_sun_cap = 0;
    // SU(N) general pair couplings (sgb_set_general) and their device rows
    std::vector<int> gen_bond_h;
    std::vector<double> gen_A_h, gen_B_h;
    void* gtab = nullptr;
    // inhomogeneous couplings (sgb_set_bonds_at / sgb_set_onsite_at) and their device rows
    bool inh_bonds = false, inh_onsite = false;
    std::vector<sgb_site_bond> site_bonds_h;
    std::vector<double> onsite_site_h;
    void* inh_dev = nullptr;         // one allocation: ioff, ient, ctab, cbq, oidx, otab, okmax
    std::vector<int> inh_off_h, inh_nbr_h;   // host copies of the per-site lists (LocalSampler colouring)
    // Langevin on small dipole lattices: -1 not yet timed, 0 persistent grid, cs > 0 a
    // cluster of cs CTAs holding the lattice in distributed shared memory
    int heun_cluster = -1;
    int conc = 1;               // systems launched concurrently with this one (replica groups): the
                                // persistent grids are sized for nsm / conc SMs
    bool heun_forced = false;        // set by sgb_set_langevin_cluster
    cudaEvent_t tev[2] = {};         // events of the kernel-choice timing (not the user's slots)
};

struct sgb_corr {
    sgb_system* sys = nullptr;
    std::string err;
    int nobs = 0, ncorr = 0, npos = 0, ncell = 0, nomega = 0, nsnaps = 0, measperiod = 1;
    double dt = 0, damping = 0, tol = 0;
    int max_iters = 100;
    int window = -1;
    int64_t nsamples = 0;
    void* ops = nullptr;      // R
    int* pairs = nullptr;
    void* A = nullptr;        // complex R [n][nobs][npos][ncell]
    void* Ahat = nullptr;
    double* P = nullptr;      // complex double accumulator
    size_t plen = 0;          // complex elements
    double* g = nullptr;      // [n]
    cufftHandle plan_space = 0, plan_time = 0;
    bool have_space = false, have_time = false;
    bool profile = false;
    cudaEvent_t ev[5] = {};
    double phase_ms[4] = {0, 0, 0, 0};
    int64_t nprof = 0;
    int64_t prof_iters = 0;
    sgb_batch* batch = nullptr;   // set when the accumulator samples a replica batch
    int nrep = 1;                 // replicas sampled per add_sample call
    int64_t prof_iters_last = 0;
    cudaStream_t stream = nullptr;  // the owner's stream; null (default stream) once the owner is destroyed
    long long* launches = nullptr;  // the owner's launch counter, else own_launches
    long long own_launches = 0;
    // calculate_errors: P holds the running mean of the transformed samples (not their
    // sum) and M the Welford sums of squared deviations, both in Sunny's layout
    int* err_d = nullptr;           // device flag: a bounded wait of the accumulation gave up
    int accum_variant = 1;          // 0 register streaming, 1 bulk-copy rows
    bool welford = false;
    double* M = nullptr;
    double* ctmp = nullptr;         // [chunk][n] complex work buffer of the per-sample transform
    size_t chunk = 0;
    cufftHandle plan_chunk = 0;
    bool have_chunk = false;
    // FP32 time transform by the hand-written Bluestein kernel (sgb_tdft.cu) when the length
    // allows: chirp, FFT of the chirp / 1024, twiddle table; time_kind 0 uses it, 1 cuFFT
    void* td_chirp = nullptr;
    void* td_fb = nullptr;
    void* td_tw = nullptr;
    int time_kind = 0;
};


// One launch shape of the batched midpoint kernel and its autotuning time.
struct MidShape {
    int idx;        // tile kernel: neighbour indices 2 = uint16 in shared memory, 4 = int32 in shared memory, 0 = global
    int G;          // bonds whose neighbour spins are gathered together
    int bps;        // CTAs per SM
    int grid;
    size_t smem;
    float ms;       // time of the tuning run (0 if not timed)
    int kind = 0;   // 0 tile kernel; 1 cell-block kernel with blocks of 2^lbx x 2^lby x 2^lbz cells
    int lbx = 0, lby = 0, lbz = 0;
    int maps = -1;  // cell-block kernel: its tensor maps in sgb_batch::blk_maps
    int nt = 256;   // threads per CTA (the cell-block kernel has 256, 512 and 1024)
};

struct sgb_batch {
    sgb_desc proto{};
    int nrep = 0, na = 0, nsm = 0;
    bool fp32 = false;
    std::vector<int> dims;          // [nrep][3]
    std::vector<int> off;           // [nrep + 1] first site of each replica
    int NS = 0;                     // total sites
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[8] = {};
    std::string err;
    long long launches = 0;
    // couplings per sublattice
    std::vector<double> kappa_a, g_a, field_a, onsite;
    std::vector<sgb_bond> bonds;
    bool coup_set = false;
    void* tables = nullptr;
    int tables_bytes = 0;
    Model<float> mf{};
    Model<double> md{};
    void* kap = nullptr;            // R[na]
    void* h = nullptr;              // R[3][na]
    bool has_field = false;
    // per replica device data
    int4* rd = nullptr;             // (L1, L2, L3, ncell)
    int* roff = nullptr;
    double* kT = nullptr;
    void* kTR = nullptr;            // kT in the working precision (noise amplitudes)
    std::vector<double> kT_h;
    int* ladder = nullptr;          // replica at each ladder position (group-major)
    int* gstart = nullptr;          // first ladder position of each group
    int* gcount = nullptr;
    int ngroups = 0;
    std::vector<int> ladder_h, gstart_h, gcount_h;
    int4* tiles = nullptr;          // (replica, first site, count, 0)
    int ntiles = 0;
    std::vector<int> tfirst, tcount;  // tiles of each replica (contiguous)
    int* tfirst_d = nullptr;
    int* tcount_d = nullptr;
    int* pc = nullptr;              // [NS] packed site coordinates
    int* nbr = nullptr;             // neighbour tables, one per distinct replica size
    int* nbo = nullptr;             // [nrep] offset of each replica's table in nbr
    int4* td = nullptr;             // [ntiles][2] tile descriptors
    int kb = 0;                     // most bonds of any sublattice (neighbour-table rows)
    int nsr_max = 0;                // sites of the largest replica
    std::vector<MidShape> mid_shapes;   // launch shapes of the batched midpoint kernel that fit
    void* Hpad = nullptr;           // cell-block kernel: 3 padded midpoint-spin buffers (float4)
    size_t hpad_bytes = 0;
    int blk_gw = 0;                 // their ghost width (largest bond offset)
    std::vector<BlkMaps> blk_maps;  // tensor maps of the cell-block shapes
    int mid_choice = -1;            // shape picked by the autotuner (-1: not tuned for these couplings)
    int mid_chunk = 0;              // replicas per midpoint launch requested (0: sized for L2)
    int mid_accept0 = 0;            // convergence test also at the extrapolated first iterate
    int mid_nchunk = 1, mid_per = 0, mid_ntiles = 0;   // launches per trajectory, replicas and tiles per launch
    // batched Langevin launch shapes: CTAs per SM 4, 3, 2 (FP32) or 2 (FP64), timed once per
    // couplings; heun_ms[k] the time of shape k's tuning run (0: not tried, 1e30: does not fit)
    int heun_bps = 0;               // 0: not tuned
    float heun_ms[3] = {0, 0, 0};
    // state
    void* S = nullptr;
    void* P = nullptr;
    void* D1 = nullptr;
    void* Sp = nullptr;             // midpoint iterate
    void* H = nullptr;              // midpoint rotating buffers [3][3][NS]
    void* P1 = nullptr;             // next step's first midpoint iterate (extrapolated)
    void* H1 = nullptr;             // states of the three previous steps (extrapolation history)
    void* H2 = nullptr;
    void* H3 = nullptr;
    int mid_order = 0;              // initial-iterate extrapolation order of the batched midpoint
    // replica group (sgb_batch_create_group): the replicas are whole systems owned by the
    // caller, advanced together on their own streams; empty for an ordinary batch
    std::vector<sgb_system*> grp;
    std::vector<cudaEvent_t> gev;   // [nrep] join events
    cudaEvent_t gfork = nullptr;
    double* racc = nullptr;         // [3][nrep] convergence sums
    Ctrl* ctrl = nullptr;
    double* Epart = nullptr;        // [ntiles]
    double* E = nullptr;            // [nrep]
    unsigned long long* counters = nullptr;   // [0] Langevin step, [1] exchange round
    long long* n_accept = nullptr;  // [nrep]
    char* stage = nullptr;
    size_t stage_cap = 0;
    bool state_set = false;
    cudaGraphExec_t graph = nullptr;
    int graph_interval = -1;
    double graph_dt = 0, graph_damping = 0;
    uint64_t graph_seed = 0;
    std::vector<sgb_corr*> corrs;   // accumulators created on this batch (detached on destroy)
};

// Detach every accumulator of a system or batch that is being destroyed: they keep their
// data (read-out and merge run on the default stream) but can no longer add samples.
inline void sgb_detach_corrs(std::vector<sgb_corr*>& corrs) {
    for (sgb_corr* c : corrs) {
        c->sys = nullptr;
        c->batch = nullptr;
        c->stream = nullptr;
        c->launches = &c->own_launches;
    }
    corrs.clear();
}

// batched add_sample! trajectory (sgb_batch.cu)
int batch_corr_trajectory(sgb_corr* c);
const char* batch_error(sgb_batch* b);

// internal entry points of sgb_api.cu used by the adjoint (sgb_adjoint.cu)
int sgb_int_midpoint_snap(sgb_system* s, double dt, double tol, int max_iters, int nsteps, const SnapArgs<double>& sn,
                          int64_t* iters);
void sgb_int_window_weights(int n, int window, std::vector<double>& g);
int sgb_int_ensure_tables(sgb_system* s);
void sgb_int_set_error(const std::string& msg);

// Replica groups (sgb_api.cu): Langevin, energies and batched S(q,w) trajectories of a
// batch whose replicas are whole systems.
int group_langevin(sgb_batch* b, double dt, double damping, uint64_t seed, uint64_t step0, int nsteps);
int group_energy(sgb_batch* b, double* E);
int group_trajectory(sgb_corr* c);
