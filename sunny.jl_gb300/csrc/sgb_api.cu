// sgb_api.cu -- host implementation of the C ABI declared in include/sunny_gb300.h.
//
// One sgb_system mirrors one Sunny `System` (src/System/Types.jl:106-140) resident on the
// GPU: its spin state, per-site κ/g/field, and coupling tables. The host code validates
// arguments with the reference's own error rules, packs the coupling tables (both
// directions of each bond, as Sunny stores them), sizes the persistent launches from
// the occupancy calculator, and reports kernel status words as SGB_ERR_* codes.
#include <cuda_runtime.h>
#include <cufft.h>
#include <algorithm>
#include <cmath>
#include <complex>
#include <map>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include "sgb_internal.h"
#include "sgb_corr.h"
#include "sgb_tables.h"
#include "sgb_handles.h"

#define SGB_VERSION "sunny-gb300 0.1.0 (sm_103a)"

static thread_local std::string g_last_error;

// ---------------------------------------------------------------------------------
namespace {

int fail(sgb_system* s, int code, const std::string& msg) {
    if (s) s->err = msg;
    g_last_error = msg;
    return code;
}

int cuda_fail(sgb_system* s, cudaError_t e, const char* what) {
    return fail(s, SGB_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                                      \
    do {                                                              \
        cudaError_t _e = (call);                                      \
        if (_e != cudaSuccess) return cuda_fail(s, _e, #call);        \
    } while (0)

size_t rsize(const sgb_system* s) { return s->fp32 ? 4 : 8; }

// Pinned host staging buffer used for every state upload and download.
int ensure_stage(sgb_system* s, size_t bytes) {
    if (s->stage_cap >= bytes) return SGB_OK;
    if (s->stage) cudaFreeHost(s->stage);
    s->stage = nullptr;
    s->stage_cap = 0;
    cudaError_t e = cudaMallocHost((void**)&s->stage, bytes);
    if (e != cudaSuccess) return fail(s, SGB_ERR_NOMEM, std::string("pinned host allocation failed: ") + cudaGetErrorString(e));
    s->stage_cap = bytes;
    return SGB_OK;
}

int dmalloc(sgb_system* s, void** p, size_t bytes) {
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        *p = nullptr;
        return fail(s, SGB_ERR_NOMEM, std::string("device allocation of ") + std::to_string(bytes) + " bytes failed: " + cudaGetErrorString(e));
    }
    return SGB_OK;
}

void dfree(void*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

int ensure_dbuf(sgb_system* s, size_t n) {
    if (s->dbuf_cap >= n) return SGB_OK;
    if (s->dbuf) cudaFree(s->dbuf);
    s->dbuf = nullptr;
    s->dbuf_cap = 0;
    int rc = dmalloc(s, (void**)&s->dbuf, n * sizeof(double));
    if (rc == SGB_OK) s->dbuf_cap = n;
    return rc;
}

template <class R>
int build_inh_tables(sgb_system* s, Model<R>& M);

template <class R>
int build_tables(sgb_system* s, Model<R>& M) {
    std::vector<unsigned char> buf;
    bool any_bq = false;
    sgbhost::GeneralTerms gen;
    gen.bond = s->gen_bond_h;
    gen.A = s->gen_A_h;
    gen.B = s->gen_B_h;
    std::vector<R> grows;
    std::string e = sgbhost::pack_tables<R>(s->d.natoms, s->N, s->sun, s->d.dims, s->bonds_h, s->onsite_h, M, buf, any_bq,
                                            s->sun ? &gen : nullptr, &grows);
    if (!e.empty()) return fail(s, SGB_ERR_ARG, e);
    dfree(s->gtab);
    M.gtab = nullptr;
    if (!grows.empty()) {
        int rg = dmalloc(s, &s->gtab, sizeof(R) * grows.size());
        if (rg) return rg;
        CK(cudaMemcpy(s->gtab, grows.data(), sizeof(R) * grows.size(), cudaMemcpyHostToDevice));
        M.gtab = reinterpret_cast<const R*>(s->gtab);
        // the general terms run in the kernels that publish quadrupoles (and densities)
        M.has_biquad = 1;
        any_bq = true;
    }
    dfree(s->tables);
    int rc = dmalloc(s, &s->tables, buf.size());
    if (rc) return rc;
    CK(cudaMemcpy(s->tables, buf.data(), buf.size(), cudaMemcpyHostToDevice));
    s->tables_bytes = (int)buf.size();
    s->has_biquad = any_bq;
    {
        // neighbour table [k][site] for the k-th bond of each site's sublattice
        const int na = s->d.natoms, L1 = s->d.dims[0], L2 = s->d.dims[1], L3 = s->d.dims[2];
        const int* boff = reinterpret_cast<const int*>(buf.data() + M.off_boff);
        const DBond<R>* bonds = reinterpret_cast<const DBond<R>*>(buf.data() + M.off_bonds);
        int kb = 1;
        for (int a = 0; a < na; a++) kb = std::max(kb, boff[a + 1] - boff[a]);
        std::vector<int> tab((size_t)kb * s->ns, 0);
        for (int a = 0; a < na; a++)
            for (int c3 = 0; c3 < L3; c3++)
                for (int c2 = 0; c2 < L2; c2++)
                    for (int c1 = 0; c1 < L1; c1++) {
                        const int site = c1 + L1 * (c2 + L2 * (c3 + L3 * a));
                        for (int k = 0; k < boff[a + 1] - boff[a]; k++) {
                            const DBond<R>& B = bonds[boff[a] + k];
                            int x1 = (c1 + B.n[0]) % L1, x2 = (c2 + B.n[1]) % L2, x3 = (c3 + B.n[2]) % L3;
                            tab[(size_t)k * s->ns + site] = x1 + L1 * (x2 + L2 * (x3 + L3 * B.j));
                        }
                    }
        s->boff_h.assign(boff, boff + na + 1);
        s->nbr_h = tab;
        s->colors_dirty = true;
        if (!s->heun_forced) s->heun_cluster = -1;
        void* p = s->nbr;
        dfree(p);
        s->nbr = nullptr;
        if ((rc = dmalloc(s, (void**)&s->nbr, sizeof(int) * tab.size()))) return rc;
        CK(cudaMemcpy(s->nbr, tab.data(), sizeof(int) * tab.size(), cudaMemcpyHostToDevice));
        M.nbr = s->nbr;
        M.kb = kb;
    }
    M.L1 = s->d.dims[0]; M.L2 = s->d.dims[1]; M.L3 = s->d.dims[2];
    M.ns = s->ns; M.ncell = s->ncell;
    M.kappa = reinterpret_cast<const R*>(s->kappa);
    M.h = s->has_field ? reinterpret_cast<const R*>(s->h) : nullptr;
    M.tables = reinterpret_cast<const unsigned char*>(s->tables);
    return build_inh_tables<R>(s, M);
}

// Per-site coupling rows of an inhomogeneous system (to_inhomogeneous,
// Interactions.jl:81-100): each non-culled coupling of a site's list becomes the forward
// row at that site and the reversed row (J^T, transposed biquadratic matrix, fwd = 0) at
// bonded_site (System.jl:204-212), as set_pair_coupling_at_aux! stores both
// (PairExchange.jl:447-468). Equal rows are stored once.
template <class R>
int build_inh_tables(sgb_system* s, Model<R>& M) {
    M.ioff = nullptr; M.ient = nullptr; M.ctab = nullptr; M.cbq = nullptr;
    M.oidx = nullptr; M.otab = nullptr; M.okmax = nullptr;
    dfree(s->inh_dev);
    s->inh_off_h.clear();
    s->inh_nbr_h.clear();
    if (!s->inh_bonds && !s->inh_onsite) return SGB_OK;
    const int ns = s->ns;
    const int L1 = s->d.dims[0], L2 = s->d.dims[1], L3 = s->d.dims[2];
    std::vector<int> off(ns + 1, 0);
    std::vector<int2> ent;
    std::vector<DBond<R>> rows;
    std::vector<R> bqrows;
    bool any_bq = false, general = false;
    if (s->inh_bonds) {
        std::map<std::string, int> row_of;
        auto row = [&](const sgb_bond& b, bool fwd) {
            DBond<R> e{};
            bool iso = b.bilin[0] == b.bilin[4] && b.bilin[0] == b.bilin[8];
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) {
                    const double v = fwd ? b.bilin[r + 3 * c] : b.bilin[c + 3 * r];
                    e.J[r + 3 * c] = (R)v;
                    if (r != c && v != 0.0) iso = false;
                }
            e.jkind = iso ? 0 : 1;
            e.scalar = (R)b.scalar;
            e.bqkind = b.biquad_kind;
            std::vector<R> m;
            if (b.biquad_kind == 1) {
                e.bq = (R)b.biquad[0];
                if (b.biquad[0] == 0.0) e.bqkind = 0;
            } else if (b.biquad_kind == 2) {
                for (int c = 0; c < 5; c++)
                    for (int r = 0; r < 5; r++) m.push_back((R)(fwd ? b.biquad[r + 5 * c] : b.biquad[c + 5 * r]));
            }
            e.fwd = fwd ? 1 : 0;
            std::string key(reinterpret_cast<const char*>(&e), sizeof(e));
            key.append(reinterpret_cast<const char*>(m.data()), m.size() * sizeof(R));
            auto it = row_of.find(key);
            if (it != row_of.end()) return it->second;
            if (e.bqkind == 2) {
                e.bqidx = (int)(bqrows.size() / 25);
                bqrows.insert(bqrows.end(), m.begin(), m.end());
            }
            any_bq |= e.bqkind != 0;
            general |= e.jkind != 0 || e.bqkind != 0;
            const int k = (int)rows.size();
            rows.push_back(e);
            row_of.emplace(std::move(key), k);
            return k;
        };
        struct Dir { int from, to, row; };
        std::vector<Dir> dirs;
        dirs.reserve(2 * s->site_bonds_h.size());
        for (const sgb_site_bond& sb : s->site_bonds_h) {
            const sgb_bond& b = sb.bond;
            const int i = sb.cell[0] + L1 * (sb.cell[1] + L2 * (sb.cell[2] + L3 * b.i));
            const int j = sgbhost::imod(sb.cell[0] + b.n[0], L1) +
                          L1 * (sgbhost::imod(sb.cell[1] + b.n[1], L2) + L2 * (sgbhost::imod(sb.cell[2] + b.n[2], L3) + L3 * b.j));
            dirs.push_back({i, j, row(b, true)});
            dirs.push_back({j, i, row(b, false)});
        }
        for (const Dir& d : dirs) off[d.from + 1]++;
        for (int i = 0; i < ns; i++) off[i + 1] += off[i];
        ent.resize(dirs.size());
        std::vector<int> fill(off.begin(), off.end() - 1);
        for (const Dir& d : dirs) ent[fill[d.from]++] = make_int2(d.to, d.row);
        s->inh_off_h = off;
        s->inh_nbr_h.resize(ent.size());
        for (size_t k = 0; k < ent.size(); k++) s->inh_nbr_h[k] = ent[k].x;
    }
    std::vector<int> oidx, okmax;
    std::vector<R> otab;
    if (s->inh_onsite) {
        const int per = s->sun ? 2 * s->N * s->N : 28;
        std::map<std::vector<double>, int> row_of;
        oidx.resize(ns);
        for (int i = 0; i < ns; i++) {
            std::vector<double> c(s->onsite_site_h.begin() + (size_t)per * i, s->onsite_site_h.begin() + (size_t)per * (i + 1));
            int km = 0;
            if (!s->sun) {
                // StevensExpansion drops k-blocks of norm < 1e-12 (Types.jl:12-16)
                const int start[4] = {0, 1, 6, 15}, len[4] = {1, 5, 9, 13};
                for (int g = 0; g < 4; g++) {
                    double nrm = 0;
                    for (int q = 0; q < len[g]; q++) nrm += c[start[g] + q] * c[start[g] + q];
                    const bool zero = std::sqrt(nrm) < 1e-12;
                    if (zero) for (int q = 0; q < len[g]; q++) c[start[g] + q] = 0;
                    if (!zero && g > 0) km = 2 * g;
                }
            }
            auto it = row_of.find(c);
            if (it == row_of.end()) {
                const int k = (int)okmax.size();
                for (double v : c) otab.push_back((R)v);
                okmax.push_back(km);
                it = row_of.emplace(c, k).first;
            }
            oidx[i] = it->second;
        }
    }
    // one device allocation, 16-byte aligned parts
    size_t o_off = 0, o_ent, o_ctab, o_cbq, o_oidx, o_otab, o_okmax, total;
    o_ent = sgbhost::align16(o_off + sizeof(int) * (s->inh_bonds ? ns + 1 : 0));
    o_ctab = sgbhost::align16(o_ent + sizeof(int2) * ent.size());
    o_cbq = sgbhost::align16(o_ctab + sizeof(DBond<R>) * rows.size());
    o_oidx = sgbhost::align16(o_cbq + sizeof(R) * bqrows.size());
    o_otab = sgbhost::align16(o_oidx + sizeof(int) * oidx.size());
    o_okmax = sgbhost::align16(o_otab + sizeof(R) * otab.size());
    total = sgbhost::align16(o_okmax + sizeof(int) * okmax.size());
    std::vector<unsigned char> buf(total, 0);
    auto put = [&](size_t at, const void* src, size_t bytes) { if (bytes) std::memcpy(buf.data() + at, src, bytes); };
    if (s->inh_bonds) put(o_off, off.data(), sizeof(int) * (ns + 1));
    put(o_ent, ent.data(), sizeof(int2) * ent.size());
    put(o_ctab, rows.data(), sizeof(DBond<R>) * rows.size());
    put(o_cbq, bqrows.data(), sizeof(R) * bqrows.size());
    put(o_oidx, oidx.data(), sizeof(int) * oidx.size());
    put(o_otab, otab.data(), sizeof(R) * otab.size());
    put(o_okmax, okmax.data(), sizeof(int) * okmax.size());
    int rc = dmalloc(s, &s->inh_dev, total);
    if (rc) return rc;
    CK(cudaMemcpy(s->inh_dev, buf.data(), total, cudaMemcpyHostToDevice));
    unsigned char* d = reinterpret_cast<unsigned char*>(s->inh_dev);
    if (s->inh_bonds) {
        M.ioff = reinterpret_cast<const int*>(d + o_off);
        M.ient = reinterpret_cast<const int2*>(d + o_ent);
        M.ctab = reinterpret_cast<const DBond<R>*>(d + o_ctab);
        M.cbq = reinterpret_cast<const R*>(d + o_cbq);
        s->has_biquad = any_bq;
        M.has_biquad = any_bq ? 1 : 0;
        M.general = general ? 1 : 0;
    }
    if (s->inh_onsite) {
        M.oidx = reinterpret_cast<const int*>(d + o_oidx);
        M.otab = reinterpret_cast<const R*>(d + o_otab);
        M.okmax = reinterpret_cast<const int*>(d + o_okmax);
    }
    return SGB_OK;
}

int ensure_tables(sgb_system* s) {
    if (!s->sites_set) return fail(s, SGB_ERR_STATE, "sgb_set_sites must be called before stepping");
    if (!s->tables_dirty) return SGB_OK;
    int rc = s->fp32 ? build_tables<float>(s, s->mf) : build_tables<double>(s, s->md);
    if (rc == SGB_OK) s->tables_dirty = false;
    return rc;
}

// Choose sites-per-thread, block and grid for a persistent cooperative launch: the
// smallest SPT whose grid fits on the device, with the block sized so that the sites
// spread evenly, one block per SM (latency, not throughput, bounds these kernels).
template <class R>
int plan_launch(sgb_system* s, LaunchInfo& li) {
    const int sptv_dip[4] = {1, 2, 4, 8}, sptv_sun[2] = {1, 2};
    const int* sptv = s->sun ? sptv_sun : sptv_dip;
    int nspt = s->sun ? 2 : 4;
    size_t smem = (size_t)s->tables_bytes;
    LaunchInfo fallback{0, 0, 0, 0};
    // a system of a replica group shares the GPU with the group's other members
    const int nsm = std::max(1, s->nsm / std::max(1, s->conc));
    for (int i = 0; i < nspt; i++) {
        int spt = sptv[i];
        int maxblock = sgb_maxblock(sizeof(R) == 8, s->sun, spt);
        long long per_sm = ((long long)s->ns + (long long)nsm * spt - 1) / ((long long)nsm * spt);
        int block = (int)std::min<long long>(maxblock, std::max<long long>(128, (per_sm + 31) / 32 * 32));
        int bps = 0;
        int rc = s->sun ? sun_max_blocks<R>(s->N, spt, block, smem, &bps) : dip_max_blocks<R>(spt, block, smem, &bps);
        if (rc != SGB_OK) return fail(s, SGB_ERR_CUDA, "occupancy query failed");
        long long cap = (long long)bps * nsm;
        long long need = ((long long)s->ns + (long long)block * spt - 1) / ((long long)block * spt);
        if (need < 1 || need > cap) continue;
        LaunchInfo cand{(int)need, block, spt, smem};
        if (need <= nsm) { li = cand; return SGB_OK; }   // at most one block per SM
        if (fallback.grid == 0) fallback = cand;
    }
    if (fallback.grid) { li = fallback; return SGB_OK; }
    return fail(s, SGB_ERR_ARG, "system too large for one co-resident persistent launch");
}

int reset_ctrl(sgb_system* s) {
    CK(cudaMemsetAsync(s->ctrl, 0, sgb_ctrl_clear_bytes(), s->stream));
    return SGB_OK;
}

int read_ctrl(sgb_system* s, Ctrl* out) {
    CK(cudaMemcpyAsync(out, s->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return SGB_OK;
}

template <class R>
Model<R>& model(sgb_system* s);
template <>
Model<float>& model<float>(sgb_system* s) { return s->mf; }
template <>
Model<double>& model<double>(sgb_system* s) { return s->md; }

std::string fmt_g(double x) {
    char b[64];
    snprintf(b, sizeof b, "%g", x);
    return b;
}

// Cluster size for a dipole lattice held in distributed shared memory: one site per thread
// where possible, at most 16 CTAs, the slices within 160 KB of shared memory each; 0 when
// the lattice is too large for one cluster.
template <class R>
int do_refresh(sgb_system* s);

template <class R>
size_t cluster_smem(sgb_system* s, int nsl) {
    return s->sun ? sun_cluster_smem<R>(model<R>(s), nsl) : dip_cluster_smem<R>(model<R>(s), nsl);
}

template <class R>
int cluster_size(sgb_system* s) {
    // the cluster kernels read the per-sublattice tables only, without general terms
    if (s->inh_bonds || s->inh_onsite || !s->gen_bond_h.empty()) return 0;
    int cs = 1;
    while (cs < SGB_CLUSTER_MAX && (long long)cs * SGB_CLUSTER_BLOCK < s->ns) cs *= 2;
    const int nsl = (s->ns + cs - 1) / cs;
    if (nsl > 8 * SGB_CLUSTER_BLOCK || cluster_smem<R>(s, nsl) > 160 * 1024) return 0;
    return cs;
}

template <class R>
int launch_heun_cluster(sgb_system* s, int cs, int nsteps, double dt, double damping, double nscale, uint64_t seed,
                        uint64_t step0, const double* noise) {
    Model<R>& M = model<R>(s);
    if (s->sun)
        return sun_launch_heun_cluster<R>(M, (R*)s->Z, (R*)s->S, (R*)s->Q, cs, nsteps, dt, damping, nscale, seed, step0, noise,
                                          s->stream);
    return dip_launch_heun_cluster<R>(M, (R*)s->S, cs, nsteps, dt, damping, nscale, seed, step0, noise, s->stream);
}

// Chooses, once per handle, between the persistent grid kernel and the cluster kernel
// (at the largest cluster size and at 1/2 and 1/4 of it) for Langevin on small lattices,
// by timing 100 steps of each on a copy of the state (restored afterwards). Each timed
// launch follows an untimed one of the same kernel on the stream, so the host-side work
// of the launch (attributes, the cluster occupancy query) overlaps the GPU's run of the
// first and only the kernel itself is timed.
template <class R>
int tune_heun(sgb_system* s, const LaunchInfo& li, double dt, double damping, double nscale, uint64_t seed) {
    if (s->heun_cluster >= 0) return SGB_OK;
    s->heun_cluster = 0;
    const int csmax = cluster_size<R>(s);
    if (csmax == 0) return SGB_OK;
    // the state that a trial run changes: dipoles, or kets (dipoles and quadrupoles are
    // refreshed from them afterwards)
    R* X = (R*)(s->sun ? s->Z : s->S);
    const size_t bytes = sizeof(R) * (s->sun ? 2 * s->N : 3) * (size_t)s->ns;
    for (int e = 0; e < 2; e++)
        if (!s->tev[e] && cudaEventCreate(&s->tev[e]) != cudaSuccess) return cuda_fail(s, cudaGetLastError(), "event creation");
    void* save = nullptr;
    int rc = dmalloc(s, &save, bytes);
    if (rc) return rc;
    Model<R>& M = model<R>(s);
    const int nt = 100;
    const int cand[4] = {0, csmax, csmax / 2, csmax / 4};
    auto launch = [&](int cs) -> int {
        int lrc;
        if (cs > 0) lrc = launch_heun_cluster<R>(s, cs, nt, dt, damping, nscale, seed, 0, nullptr);
        else if (!s->sun) lrc = dip_launch_heun<R>(M, (R*)s->S, (R*)s->P, s->ctrl, nt, dt, damping, nscale, seed, 0, nullptr, li, s->stream);
        else lrc = sun_launch_heun<R>(M, (R*)s->Z, (R*)s->S, (R*)s->Q, (R*)s->P, (R*)s->QP, s->ctrl, nt, dt, damping, nscale, seed, 0,
                                      nullptr, li, s->stream);
        s->launches++;
        if (lrc != SGB_OK) cudaGetLastError();
        return lrc;
    };
    float best = 0;
    for (int v = 0; v < 4; v++) {
        const int cs = cand[v];
        if (v > 0 && (cs < 1 || (long long)cs * 8 * SGB_CLUSTER_BLOCK < s->ns || cluster_smem<R>(s, (s->ns + cs - 1) / cs) > 160 * 1024))
            continue;
        float t = 0;
        const bool saved = cudaMemcpyAsync(save, X, bytes, cudaMemcpyDeviceToDevice, s->stream) == cudaSuccess;
        bool ok = saved && reset_ctrl(s) == SGB_OK && launch(cs) == SGB_OK && reset_ctrl(s) == SGB_OK &&
                  cudaEventRecord(s->tev[0], s->stream) == cudaSuccess && launch(cs) == SGB_OK &&
                  cudaEventRecord(s->tev[1], s->stream) == cudaSuccess;
        // a saved state is restored whether or not the trial ran
        if (saved) {
            ok = cudaMemcpyAsync(X, save, bytes, cudaMemcpyDeviceToDevice, s->stream) == cudaSuccess && ok;
            if (s->sun) ok = do_refresh<R>(s) == SGB_OK && ok;
        }
        ok = cudaStreamSynchronize(s->stream) == cudaSuccess && ok;
        if (ok) ok = cudaEventElapsedTime(&t, s->tev[0], s->tev[1]) == cudaSuccess;
        if (!ok) continue;
        if (v == 0 || t < best) { best = t; s->heun_cluster = cs; }
    }
    dfree(save);
    return SGB_OK;
}

template <class R>
int run_langevin(sgb_system* s, double dt, double damping, double kT, uint64_t seed, uint64_t step0, int nsteps, const double* noise,
                 bool sync = true) {
    LaunchInfo li;
    int rc = plan_launch<R>(s, li);
    if (rc) return rc;
    double nscale = (damping == 0.0 || kT == 0.0) ? 0.0 : std::sqrt(2 * dt * damping * kT);
    if ((rc = tune_heun<R>(s, li, dt, damping, nscale, seed))) return rc;
    const size_t per = s->sun ? (size_t)2 * s->N * s->ns : (size_t)3 * s->ns;
    int chunk = nsteps;
    if (noise) {
        size_t maxel = (size_t)1 << 24;  // 128 MiB of injected noise per launch
        chunk = (int)std::max<size_t>(1, std::min<size_t>((size_t)nsteps, maxel / per));
        if ((rc = ensure_dbuf(s, per * chunk))) return rc;
    }
    Model<R>& M = model<R>(s);
    for (int k0 = 0; k0 < nsteps; k0 += chunk) {
        int nk = std::min(chunk, nsteps - k0);
        const double* dn = nullptr;
        if (noise) {
            CK(cudaMemcpyAsync(s->dbuf, noise + per * k0, per * nk * sizeof(double), cudaMemcpyHostToDevice, s->stream));
            dn = s->dbuf;
        }
        if ((rc = reset_ctrl(s))) return rc;
        if (s->heun_cluster > 0)
            rc = launch_heun_cluster<R>(s, s->heun_cluster, nk, dt, damping, nscale, seed, step0 + k0, dn);
        else if (!s->sun)
            rc = dip_launch_heun<R>(M, (R*)s->S, (R*)s->P, s->ctrl, nk, dt, damping, nscale, seed, step0 + k0, dn, li, s->stream);
        else
            rc = sun_launch_heun<R>(M, (R*)s->Z, (R*)s->S, (R*)s->Q, (R*)s->P, (R*)s->QP, s->ctrl, nk, dt, damping, nscale,
                                    seed, step0 + k0, dn, li, s->stream);
        s->launches++;
        if (rc) return cuda_fail(s, cudaGetLastError(), "Langevin launch");
        if (!sync && !noise) return SGB_OK;   // the caller reads the status
        Ctrl c;
        if ((rc = read_ctrl(s, &c))) return rc;
        if (c.status == SGB_ERR_TIMEOUT) return fail(s, SGB_ERR_TIMEOUT, "a device-side barrier timed out");
        if (c.status != 0) return fail(s, c.status, "Langevin kernel reported an error");
    }
    return SGB_OK;
}

template <class R>
int run_midpoint(sgb_system* s, double dt, double damping, double tol, int max_iters, int nsteps, int64_t* iters,
                 const SnapArgs<R>& snap, bool sync_status = true, int order = 0) {
    LaunchInfo li;
    int rc = plan_launch<R>(s, li);
    if (rc) return rc;
    double atol = tol * std::sqrt((double)s->ns);
    double atol2 = atol * atol;
    Model<R>& M = model<R>(s);
    if ((rc = reset_ctrl(s))) return rc;
    if (!s->sun)
        rc = dip_launch_midpoint<R>(M, (R*)s->S, (R*)s->H, s->ctrl, nsteps, dt, damping, atol2, max_iters, snap, li, s->stream,
                                    order);
    else
        rc = sun_launch_midpoint<R>(M, (R*)s->Z, (R*)s->S, (R*)s->Q, (R*)s->H, (R*)s->QH, s->ctrl, nsteps, dt, damping, atol2,
                                    max_iters, snap, li, s->stream);
    s->launches++;
    if (rc) return cuda_fail(s, cudaGetLastError(), "midpoint launch");
    if (!sync_status) return SGB_OK;
    Ctrl c;
    if ((rc = read_ctrl(s, &c))) return rc;
    if (iters) *iters = c.iters;
    if (c.status == SGB_ERR_NOCONVERGE) {
        if (!s->sun)
            return fail(s, SGB_ERR_NOCONVERGE, "Spherical midpoint method failed to converge to tolerance " + fmt_g(tol) +
                                                   " after " + std::to_string(max_iters) + " iterations.");
        return fail(s, SGB_ERR_NOCONVERGE, "Schrödinger midpoint method failed to converge in " + std::to_string(max_iters) + " iterations.");
    }
    if (c.status == SGB_ERR_TIMEOUT) return fail(s, SGB_ERR_TIMEOUT, "a device-side barrier timed out");
    if (c.status != 0) return fail(s, c.status, "midpoint kernel reported an error");
    return SGB_OK;
}

template <class R>
int do_refresh(sgb_system* s) {
    if (!s->sun) return SGB_OK;
    int rc = sun_launch_refresh<R>(model<R>(s), (const R*)s->Z, (R*)s->S, (R*)s->Q, s->stream);
    s->launches++;
    return rc ? cuda_fail(s, cudaGetLastError(), "refresh launch") : SGB_OK;
}

// <Z|S|Z> of a ket Z [N][2] (Spin.jl:72-87) with the spin-s matrices of N = 2s+1 levels
void host_expected_spin(int N, const double* z, double* out) {
    const double sp = (N - 1) / 2.0;
    double cr = 0, ci = 0, zz = 0;
    for (int j = 1; j <= N - 1; j++) {
        const double off = std::sqrt(2 * (sp + 1) * j - (double)j * (j + 1)) / 2;
        const double ar = z[2 * (j - 1)], ai = z[2 * (j - 1) + 1], br = off * z[2 * j], bi = off * z[2 * j + 1];
        cr += ar * br + ai * bi;
        ci += ar * bi - ai * br;
    }
    for (int k = 0; k < N; k++) zz += (sp - k) * (z[2 * k] * z[2 * k] + z[2 * k + 1] * z[2 * k + 1]);
    out[0] = 2 * cr;
    out[1] = 2 * ci;
    out[2] = zz;
}

void ewald_free(sgb_system* s) {
    EwaldDev& E = s->ew;
    void* p;
    p = E.g; dfree(p); p = E.mu; dfree(p); p = E.phi; dfree(p);
    p = E.FA; dfree(p); p = E.Fmu; dfree(p); p = E.Fphi; dfree(p);
    p = E.Areal; dfree(p);
    p = s->ew_part; dfree(p);
    if (E.have_f) cufftDestroy(E.plan_f);
    if (E.have_b) cufftDestroy(E.plan_b);
    E = EwaldDev{};
    s->ew_part = nullptr;
    s->ewald_on = false;
}

int ensure_lr_grad(sgb_system* s, double** grad);

// Adds the dipole-dipole gradient at state S (device, R) into grad ([ns][3] FP64 on the
// device, may be null); *E (nullable) receives the dipole-dipole energy.
template <class R>
int ewald_add(sgb_system* s, const R* S, double* grad, double* E) {
    if (!s->ewald_on) {
        if (E) *E = 0;
        return SGB_OK;
    }
    if (ewald_apply<R>(s->ew, S, grad, E ? s->ew_part : nullptr, s->stream)) return cuda_fail(s, cudaGetLastError(), "dipole-dipole launch");
    s->launches += 4;
    if (E) {
        double hp[EWALD_PART_BLOCKS];
        CK(cudaMemcpyAsync(hp, s->ew_part, sizeof(hp), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        double t = 0;
        for (int b = 0; b < EWALD_PART_BLOCKS; b++) t += hp[b];
        *E = t;
    }
    return SGB_OK;
}

// SU(N) mode: adds the dipole-dipole term to HZ ([ns][N][2] on the device) through dE/dS
// at the expected dipoles; *E (nullable) receives the dipole-dipole energy.
template <class R>
int ewald_add_sun(sgb_system* s, double* hz, double* E) {
    if (!s->ewald_on) {
        if (E) *E = 0;
        return SGB_OK;
    }
    double* f;
    int rc = ensure_lr_grad(s, &f);
    if (rc) return rc;
    CK(cudaMemsetAsync(f, 0, sizeof(double) * 3 * (size_t)s->ns, s->stream));
    if ((rc = ewald_add<R>(s, (const R*)s->S, f, E))) return rc;
    if (hz && sun_launch_add_dipole_field<R>(model<R>(s), (const R*)s->Z, f, hz, s->stream))
        return cuda_fail(s, cudaGetLastError(), "dipole field launch");
    s->launches++;
    return SGB_OK;
}

int ewald_upload_g(sgb_system* s) {
    if (!s->ewald_on) return SGB_OK;
    CK(cudaMemcpy(s->ew.g, s->g_h.data(), sizeof(double) * 9 * (size_t)s->ns, cudaMemcpyHostToDevice));
    return SGB_OK;
}

// Step loops for systems with dipole-dipole interactions: every gradient needs the
// transform over the whole lattice, so each integrator stage is its own launch (local
// gradient, Ewald gradient, stage update) instead of one persistent launch.
int ensure_lr_grad(sgb_system* s, double** grad) {
    if ((size_t)s->lr_grad_cap < 3 * (size_t)s->ns) {
        void* p = s->lr_grad;
        dfree(p);
        s->lr_grad = nullptr;
        s->lr_grad_cap = 0;
        int rc = dmalloc(s, (void**)&s->lr_grad, sizeof(double) * 3 * (size_t)s->ns);
        if (rc) return rc;
        s->lr_grad_cap = 3 * s->ns;
    }
    *grad = s->lr_grad;
    return SGB_OK;
}

template <class R>
int lr_gradient(sgb_system* s, const R* X, double* grad) {
    if (dip_launch_grad<R>(model<R>(s), X, grad, s->stream)) return cuda_fail(s, cudaGetLastError(), "gradient launch");
    s->launches++;
    return ewald_add<R>(s, X, grad, nullptr);
}

template <class R>
int run_langevin_lr(sgb_system* s, double dt, double damping, double kT, uint64_t seed, uint64_t step0, int nsteps,
                    const double* noise) {
    double* grad;
    int rc = ensure_lr_grad(s, &grad);
    if (rc) return rc;
    const int ns = s->ns;
    const double nscale = (damping == 0.0 || kT == 0.0) ? 0.0 : std::sqrt(2 * dt * damping * kT);
    if (noise && (rc = ensure_dbuf(s, 3 * (size_t)ns))) return rc;
    R* S = (R*)s->S;
    R* P = (R*)s->P;
    R* D1 = (R*)s->H;
    R* XI = D1 + 3 * (size_t)ns;
    const R* kap = (const R*)s->kappa;
    for (int k = 0; k < nsteps; k++) {
        const double* dn = nullptr;
        if (noise) {
            CK(cudaMemcpyAsync(s->dbuf, noise + 3 * (size_t)ns * k, sizeof(double) * 3 * ns, cudaMemcpyHostToDevice, s->stream));
            dn = s->dbuf;
        }
        if ((rc = lr_gradient<R>(s, S, grad))) return rc;
        if (lr_heun_a<R>(S, grad, P, D1, XI, kap, ns, dt, damping, nscale, seed, step0 + k, dn, s->stream))
            return cuda_fail(s, cudaGetLastError(), "Langevin stage launch");
        if ((rc = lr_gradient<R>(s, P, grad))) return rc;
        if (lr_heun_b<R>(S, P, grad, D1, XI, kap, ns, dt, damping, s->stream)) return cuda_fail(s, cudaGetLastError(), "Langevin stage launch");
        s->launches += 2;
    }
    CK(cudaStreamSynchronize(s->stream));
    return SGB_OK;
}

template <class R>
int run_midpoint_lr(sgb_system* s, double dt, double damping, double tol, int max_iters, int nsteps, int64_t* iters,
                    const SnapArgs<R>* snap = nullptr) {
    double* grad;
    int rc = ensure_lr_grad(s, &grad);
    if (rc) return rc;
    const int ns = s->ns;
    const double atol = tol * std::sqrt((double)ns);
    R* S = (R*)s->S;
    R* H = (R*)s->H;
    R* Sp = H + 3 * (size_t)ns;
    const R* kap = (const R*)s->kappa;
    int64_t total = 0;
    double hp[EWALD_PART_BLOCKS];
    // snapshots every measperiod steps (CorrelationSampling.jl:21-46), the first one of the
    // initial state
    if (snap && snap->enabled) {
        if (dip_launch_snapshot<R>(model<R>(s), S, *snap, snap->t0, s->stream)) return cuda_fail(s, cudaGetLastError(), "snapshot launch");
        s->launches++;
    }
    for (int k = 0; k < nsteps; k++) {
        CK(cudaMemcpyAsync(Sp, S, sizeof(R) * 3 * ns, cudaMemcpyDeviceToDevice, s->stream));   // S' = S
        bool conv = false;
        for (int it = 0; it < max_iters; it++) {
            total++;
            if (lr_mid_half<R>(S, Sp, H, kap, ns, s->stream)) return cuda_fail(s, cudaGetLastError(), "midpoint stage launch");
            if ((rc = lr_gradient<R>(s, H, grad))) return rc;
            if (lr_mid_update<R>(S, H, grad, Sp, ns, dt, damping, s->partials, s->stream))
                return cuda_fail(s, cudaGetLastError(), "midpoint stage launch");
            s->launches += 2;
            CK(cudaMemcpyAsync(hp, s->partials, sizeof(hp), cudaMemcpyDeviceToHost, s->stream));
            CK(cudaStreamSynchronize(s->stream));
            double acc = 0;
            for (int b = 0; b < EWALD_PART_BLOCKS; b++) acc += hp[b];
            if (acc <= atol * atol) {   // fast_isapprox (Integrators.jl:361-371)
                if (lr_mid_accept<R>(S, Sp, kap, ns, s->stream)) return cuda_fail(s, cudaGetLastError(), "midpoint stage launch");
                s->launches++;
                conv = true;
                break;
            }
        }
        if (iters) *iters = total;
        if (!conv)
            return fail(s, SGB_ERR_NOCONVERGE, "Spherical midpoint method failed to converge to tolerance " + fmt_g(tol) +
                                                   " after " + std::to_string(max_iters) + " iterations.");
        if (snap && snap->enabled && (k + 1) % snap->measperiod == 0) {
            if (dip_launch_snapshot<R>(model<R>(s), S, *snap, snap->t0 + (k + 1) / snap->measperiod, s->stream))
                return cuda_fail(s, cudaGetLastError(), "snapshot launch");
            s->launches++;
        }
    }
    CK(cudaStreamSynchronize(s->stream));
    return SGB_OK;
}

// SU(N) mode with dipole-dipole interactions: HZ at kets Zs (set_energy_grad_coherents!,
// Interactions.jl:596-669) = local terms at the expected dipoles and quadrupoles of Zs plus
// the dipole-dipole field through dE/dS. The handle's dipoles and quadrupoles are
// overwritten with those of Zs; the drivers refresh them from Z at the end.
template <class R>
int lr_sun_hz(sgb_system* s, const R* Zs, double* hz) {
    const Model<R>& M = model<R>(s);
    R* D = (R*)s->S;
    R* Q = (R*)s->Q;
    if (sun_launch_refresh<R>(M, Zs, D, Q, s->stream) || sun_launch_grad<R>(M, Zs, D, Q, hz, s->stream))
        return cuda_fail(s, cudaGetLastError(), "gradient launch");
    s->launches += 2;
    double* f;
    int rc = ensure_lr_grad(s, &f);
    if (rc) return rc;
    CK(cudaMemsetAsync(f, 0, sizeof(double) * 3 * (size_t)s->ns, s->stream));
    if ((rc = ewald_add<R>(s, D, f, nullptr))) return rc;
    if (sun_launch_add_dipole_field<R>(M, Zs, f, hz, s->stream)) return cuda_fail(s, cudaGetLastError(), "dipole field launch");
    s->launches++;
    return SGB_OK;
}

// scratch of the SU(N) per-stage path: kets ZP, D1, XI ([2N][ns] of R each), HZ ([ns][2N] FP64)
template <class R>
int ensure_lr_sun(sgb_system* s, R** zp, R** d1, R** xi, double** hz) {
    const size_t nk = (size_t)2 * s->N * s->ns;
    const size_t bytes = 3 * nk * sizeof(R) + nk * sizeof(double);
    if (s->lr_sun_cap < bytes) {
        void* p = s->lr_sun;
        dfree(p);
        s->lr_sun = nullptr;
        s->lr_sun_cap = 0;
        int rc = dmalloc(s, &s->lr_sun, bytes);
        if (rc) return rc;
        s->lr_sun_cap = bytes;
    }
    char* b = (char*)s->lr_sun;
    *hz = (double*)b;
    *zp = (R*)(b + nk * sizeof(double));
    *d1 = *zp + nk;
    *xi = *d1 + nk;
    return SGB_OK;
}

// Langevin Heun for coherent states (Integrators.jl:90-108), one launch per stage
template <class R>
int run_langevin_lr_sun(sgb_system* s, double dt, double damping, double kT, uint64_t seed, uint64_t step0, int nsteps,
                        const double* noise) {
    R *ZP, *D1, *XI;
    double* hz;
    int rc = ensure_lr_sun<R>(s, &ZP, &D1, &XI, &hz);
    if (rc) return rc;
    const size_t nk = (size_t)2 * s->N * s->ns;
    const double nscale = (damping == 0.0 || kT == 0.0) ? 0.0 : std::sqrt(2 * dt * damping * kT);
    if (noise && (rc = ensure_dbuf(s, nk))) return rc;
    const Model<R>& M = model<R>(s);
    R* Z = (R*)s->Z;
    for (int k = 0; k < nsteps; k++) {
        const double* dn = nullptr;
        if (noise) {
            CK(cudaMemcpyAsync(s->dbuf, noise + nk * k, sizeof(double) * nk, cudaMemcpyHostToDevice, s->stream));
            dn = s->dbuf;
        }
        if ((rc = lr_sun_hz<R>(s, Z, hz))) return rc;
        if (sun_launch_lr_stage<R>(0, M, Z, ZP, D1, XI, hz, dt, damping, nscale, seed, step0 + k, dn, nullptr, nullptr, 0, s->stream))
            return cuda_fail(s, cudaGetLastError(), "Langevin stage launch");
        if ((rc = lr_sun_hz<R>(s, ZP, hz))) return rc;
        if (sun_launch_lr_stage<R>(1, M, Z, ZP, D1, XI, hz, dt, damping, 0, 0, 0, nullptr, nullptr, nullptr, 0, s->stream))
            return cuda_fail(s, cudaGetLastError(), "Langevin stage launch");
        s->launches += 2;
    }
    if ((rc = do_refresh<R>(s))) return rc;
    CK(cudaStreamSynchronize(s->stream));
    return SGB_OK;
}

// Schrödinger midpoint (Integrators.jl:422-452), one launch per stage and iteration
template <class R>
int run_midpoint_lr_sun(sgb_system* s, double dt, double damping, double tol, int max_iters, int nsteps, int64_t* iters,
                        const SnapArgs<R>* snap = nullptr) {
    R *ZP, *ZB, *XI;
    double* hz;
    int rc = ensure_lr_sun<R>(s, &ZP, &ZB, &XI, &hz);
    if (rc) return rc;
    const size_t nk = (size_t)2 * s->N * s->ns;
    const double atol = tol * std::sqrt((double)s->ns);
    const Model<R>& M = model<R>(s);
    R* Z = (R*)s->Z;
    int64_t total = 0;
    double hp[EWALD_PART_BLOCKS];
    if (snap && snap->enabled) {
        if (sun_launch_lr_stage<R>(5, M, Z, ZP, ZB, XI, hz, 0, 0, 0, 0, 0, nullptr, nullptr, snap, snap->t0, s->stream))
            return cuda_fail(s, cudaGetLastError(), "snapshot launch");
        s->launches++;
    }
    for (int k = 0; k < nsteps; k++) {
        CK(cudaMemcpyAsync(ZP, Z, sizeof(R) * nk, cudaMemcpyDeviceToDevice, s->stream));   // Z' = Z
        bool conv = false;
        for (int it = 0; it < max_iters; it++) {
            total++;
            if (sun_launch_lr_stage<R>(2, M, Z, ZP, ZB, XI, hz, 0, 0, 0, 0, 0, nullptr, nullptr, nullptr, 0, s->stream))
                return cuda_fail(s, cudaGetLastError(), "midpoint stage launch");
            if ((rc = lr_sun_hz<R>(s, ZB, hz))) return rc;
            if (sun_launch_lr_stage<R>(3, M, Z, ZP, ZB, XI, hz, dt, damping, 0, 0, 0, nullptr, s->partials, nullptr, 0, s->stream))
                return cuda_fail(s, cudaGetLastError(), "midpoint stage launch");
            s->launches += 2;
            CK(cudaMemcpyAsync(hp, s->partials, sizeof(hp), cudaMemcpyDeviceToHost, s->stream));
            CK(cudaStreamSynchronize(s->stream));
            double acc = 0;
            for (int b = 0; b < EWALD_PART_BLOCKS; b++) acc += hp[b];
            if (acc <= atol * atol) {   // fast_isapprox (Integrators.jl:361-371)
                if (sun_launch_lr_stage<R>(4, M, Z, ZP, ZB, XI, hz, 0, 0, 0, 0, 0, nullptr, nullptr, nullptr, 0, s->stream))
                    return cuda_fail(s, cudaGetLastError(), "midpoint stage launch");
                s->launches++;
                conv = true;
                break;
            }
        }
        if (iters) *iters = total;
        if (!conv) {
            do_refresh<R>(s);
            return fail(s, SGB_ERR_NOCONVERGE, "Schrödinger midpoint method failed to converge in " + std::to_string(max_iters) + " iterations.");
        }
        if (snap && snap->enabled && (k + 1) % snap->measperiod == 0) {
            if (sun_launch_lr_stage<R>(5, M, Z, ZP, ZB, XI, hz, 0, 0, 0, 0, 0, nullptr, nullptr, snap, snap->t0 + (k + 1) / snap->measperiod,
                                       s->stream))
                return cuda_fail(s, cudaGetLastError(), "snapshot launch");
            s->launches++;
        }
    }
    if ((rc = do_refresh<R>(s))) return rc;
    CK(cudaStreamSynchronize(s->stream));
    return SGB_OK;
}

// Greedy colouring of the bond graph in site order (every bond is listed from both
// ends, so a site's own list holds all its neighbours): class of a site = the smallest
// class none of its already coloured neighbours has. Sites of one class share no
// coupling and can be updated together by the LocalSampler sweep.
int ensure_colors(sgb_system* s) {
    int rc = ensure_tables(s);
    if (rc) return rc;
    if (!s->colors_dirty) return SGB_OK;
    const int ns = s->ns, ncell = s->ncell;
    std::vector<int> col(ns, -1);
    int ncol = 0;
    const bool inh = s->inh_bonds;
    for (int i = 0; i < ns; i++) {
        const int a = i / ncell;
        uint64_t used = 0;
        const int nk = inh ? s->inh_off_h[i + 1] - s->inh_off_h[i] : s->boff_h[a + 1] - s->boff_h[a];
        for (int k = 0; k < nk; k++) {
            const int j = inh ? s->inh_nbr_h[(size_t)s->inh_off_h[i] + k] : s->nbr_h[(size_t)k * ns + i];
            // local_energy_change (Interactions.jl:345)
            if (j == i) return fail(s, SGB_ERR_ARG, "Energy delta for self-interaction not supported");
            if (col[j] >= 0 && col[j] < 64) used |= 1ull << col[j];
        }
        int c = 0;
        while (c < 64 && ((used >> c) & 1ull)) c++;
        if (c >= SGB_MC_MAXCOL) return fail(s, SGB_ERR_ARG, "bond graph needs more than 64 colour classes");
        col[i] = c;
        ncol = std::max(ncol, c + 1);
    }
    s->coff_h.assign(ncol + 1, 0);
    for (int i = 0; i < ns; i++) s->coff_h[col[i] + 1]++;
    for (int c = 0; c < ncol; c++) s->coff_h[c + 1] += s->coff_h[c];
    s->perm_h.assign(ns, 0);
    std::vector<int> pos(s->coff_h.begin(), s->coff_h.end() - 1);
    for (int i = 0; i < ns; i++) s->perm_h[pos[col[i]]++] = i;   // ascending within a class
    s->color_h = col;
    void* p = s->mc_perm;
    dfree(p);
    s->mc_perm = nullptr;
    if ((rc = dmalloc(s, (void**)&s->mc_perm, sizeof(int) * (size_t)ns))) return rc;
    CK(cudaMemcpy(s->mc_perm, s->perm_h.data(), sizeof(int) * (size_t)ns, cudaMemcpyHostToDevice));
    s->colors_dirty = false;
    return SGB_OK;
}

template <class R>
int run_local_sweeps(sgb_system* s, McArgs& A, const double* rnd_host, double* out4) {
    int bps = 0;
    if ((s->sun ? sun_mc_max_blocks<R>(model<R>(s), &bps) : mc_max_blocks<R>((size_t)s->tables_bytes, &bps)) != SGB_OK || bps < 1)
        return fail(s, SGB_ERR_CUDA, "occupancy query failed");
    int maxclass = 1;
    for (int c = 0; c < A.ncol; c++) maxclass = std::max(maxclass, A.coff[c + 1] - A.coff[c]);
    const int grid = std::max(1, std::min(bps * s->nsm, (maxclass + SGB_BLOCK - 1) / SGB_BLOCK));
    int rc;
    if (s->mc_part_cap < grid) {
        void* p = s->mc_part;
        dfree(p);
        s->mc_part = nullptr;
        s->mc_part_cap = 0;
        if ((rc = dmalloc(s, (void**)&s->mc_part, sizeof(double) * 4 * (size_t)grid))) return rc;
        s->mc_part_cap = grid;
    }
    const int total = A.nsweeps;
    const size_t per = (size_t)(s->sun ? 2 * s->N + 3 : 6) * s->ns;
    int chunk = total;
    if (rnd_host) {
        chunk = (int)std::max<size_t>(1, std::min<size_t>((size_t)total, ((size_t)1 << 24) / per));
        if ((rc = ensure_dbuf(s, per * chunk))) return rc;
    }
    double acc[4] = {0, 0, 0, 0};
    const double frac = A.frac;
    double* F = nullptr;
    if (s->ewald_on) {
        // dipole-dipole: one block proposes the sites in sweep order and keeps the field
        // dE/dS of every site current after each accepted move (ewald_energy_delta,
        // Ewald.jl:210-241, whose sum over all sites becomes a rank-one update of F)
        if ((rc = ensure_lr_grad(s, &F))) return rc;
        CK(cudaMemsetAsync(F, 0, sizeof(double) * 3 * (size_t)s->ns, s->stream));
        if ((rc = ewald_add<R>(s, (const R*)s->S, F, nullptr))) return rc;
    }
    for (int k0 = 0; k0 < total; k0 += chunk) {
        const int nk = std::min(chunk, total - k0);
        McArgs a = A;
        a.nsweeps = nk;
        a.sweep0 = A.sweep0 + (uint64_t)k0;
        a.frac = (k0 + nk == total) ? frac : 1.0;
        a.rnd = nullptr;
        if (rnd_host) {
            CK(cudaMemcpyAsync(s->dbuf, rnd_host + per * k0, per * nk * sizeof(double), cudaMemcpyHostToDevice, s->stream));
            a.rnd = s->dbuf;
        }
        if ((rc = reset_ctrl(s))) return rc;
        int gused = grid;
        if (F) {
            rc = s->sun ? sun_launch_local_sweeps_ewald<R>(model<R>(s), (R*)s->Z, (R*)s->S, (R*)s->Q, a, s->ew, F, s->mc_part, s->stream)
                        : mc_launch_sweeps_ewald<R>(model<R>(s), (R*)s->S, a, s->ew, F, s->mc_part, s->stream);
            gused = 1;
        } else {
            rc = s->sun ? sun_launch_local_sweeps<R>(model<R>(s), (R*)s->Z, (R*)s->S, (R*)s->Q, s->ctrl, a, grid, s->mc_part, s->stream)
                        : mc_launch_sweeps<R>(model<R>(s), (R*)s->S, s->ctrl, a, grid, s->mc_part, s->stream);
        }
        s->launches++;
        if (rc) return cuda_fail(s, cudaGetLastError(), "LocalSampler launch");
        if ((rc = util_launch_reduce(s->mc_part, gused, 4, s->red, s->stream))) return cuda_fail(s, cudaGetLastError(), "reduce launch");
        s->launches++;
        double part[4];
        CK(cudaMemcpyAsync(part, s->red, sizeof(part), cudaMemcpyDeviceToHost, s->stream));
        Ctrl c;
        if ((rc = read_ctrl(s, &c))) return rc;
        if (c.status == SGB_ERR_TIMEOUT) return fail(s, SGB_ERR_TIMEOUT, "a device-side barrier timed out");
        if (c.status != 0) return fail(s, c.status, "LocalSampler kernel reported an error");
        for (int q = 0; q < 4; q++) acc[q] += part[q];
    }
    for (int q = 0; q < 4; q++) out4[q] = acc[q];
    return SGB_OK;
}

}  // namespace


// ---------------------------------------------------------------------------------
// Replica groups: a batch whose replicas are whole systems (any mode, SU(N) included,
// with inhomogeneous, general or dipole-dipole couplings), each with its own stream. The
// members' persistent launches are sized for an equal share of the SMs and issued
// back to back, so the replicas advance concurrently; the batch stream waits for them.
// ---------------------------------------------------------------------------------
static int bfail_ext(sgb_batch* b, int code, const std::string& msg) {
    b->err = msg;
    return code;
}

static int group_fork(sgb_batch* b) {
    if (cudaEventRecord(b->gfork, b->stream) != cudaSuccess) return bfail_ext(b, SGB_ERR_CUDA, "event record failed");
    for (sgb_system* s : b->grp)
        if (cudaStreamWaitEvent(s->stream, b->gfork, 0) != cudaSuccess) return bfail_ext(b, SGB_ERR_CUDA, "stream wait failed");
    return SGB_OK;
}

static int group_join(sgb_batch* b) {
    for (size_t r = 0; r < b->grp.size(); r++) {
        if (cudaEventRecord(b->gev[r], b->grp[r]->stream) != cudaSuccess ||
            cudaStreamWaitEvent(b->stream, b->gev[r], 0) != cudaSuccess)
            return bfail_ext(b, SGB_ERR_CUDA, "stream join failed");
    }
    return SGB_OK;
}

// restores every member's SM share when a group operation ends
struct GroupShare {
    sgb_batch* b;
    explicit GroupShare(sgb_batch* bb) : b(bb) {
        for (sgb_system* s : b->grp) s->conc = (int)b->grp.size();
    }
    ~GroupShare() {
        for (sgb_system* s : b->grp) s->conc = 1;
    }
};

static int group_member_ready(sgb_batch* b, sgb_system* s) {
    int rc = ensure_tables(s);
    if (rc) return bfail_ext(b, rc, s->err);
    if (!s->state_set) return bfail_ext(b, SGB_ERR_STATE, "every member system needs a state");
    if (s->d.device != b->proto.device) return bfail_ext(b, SGB_ERR_ARG, "members must share one device");
    return SGB_OK;
}

// Langevin on every member at the batch's kT (member r draws its noise with seed + r)
int group_langevin(sgb_batch* b, double dt, double damping, uint64_t seed, uint64_t step0, int nsteps) {
    GroupShare share(b);
    int rc = group_fork(b);
    if (rc) return rc;
    const int R = (int)b->grp.size();
    std::vector<char> launched(R, 0);
    for (int r = 0; r < R; r++) {
        sgb_system* s = b->grp[r];
        if ((rc = group_member_ready(b, s))) return rc;
        const double kT = b->kT_h[r];
        const uint64_t sd = seed + (uint64_t)r;
        if (s->ewald_on) {
            rc = s->sun ? (s->fp32 ? run_langevin_lr_sun<float>(s, dt, damping, kT, sd, step0, nsteps, nullptr)
                                   : run_langevin_lr_sun<double>(s, dt, damping, kT, sd, step0, nsteps, nullptr))
                        : (s->fp32 ? run_langevin_lr<float>(s, dt, damping, kT, sd, step0, nsteps, nullptr)
                                   : run_langevin_lr<double>(s, dt, damping, kT, sd, step0, nsteps, nullptr));
        } else {
            rc = s->fp32 ? run_langevin<float>(s, dt, damping, kT, sd, step0, nsteps, nullptr, false)
                         : run_langevin<double>(s, dt, damping, kT, sd, step0, nsteps, nullptr, false);
            launched[r] = 1;
        }
        if (rc) return bfail_ext(b, rc, s->err);
    }
    for (int r = 0; r < R; r++) {
        if (!launched[r]) continue;
        sgb_system* s = b->grp[r];
        Ctrl c;
        if ((rc = read_ctrl(s, &c))) return bfail_ext(b, rc, s->err);
        if (c.status == SGB_ERR_TIMEOUT) return bfail_ext(b, SGB_ERR_TIMEOUT, "a device-side barrier timed out");
        if (c.status != 0) return bfail_ext(b, c.status, "Langevin kernel reported an error");
    }
    return group_join(b);
}

int group_energy(sgb_batch* b, double* E) {
    for (size_t r = 0; r < b->grp.size(); r++) {
        sgb_system* s = b->grp[r];
        int rc = group_member_ready(b, s);
        if (rc) return rc;
        if ((rc = sgb_energy(s, &E[r], nullptr))) return bfail_ext(b, rc, s->err);
    }
    return SGB_OK;
}

// Trajectories of a batched add_sample!: member r runs the implicit midpoint with its
// snapshots written to replica r's rows of the accumulator's time series.
int group_trajectory(sgb_corr* c) {
    sgb_batch* b = c->batch;
    GroupShare share(b);
    int rc = group_fork(b);
    if (rc) return rc;
    const int R = (int)b->grp.size();
    const int nsteps = c->measperiod * (c->nsnaps - 1);
    const size_t rep_stride = (size_t)c->nomega * c->nobs * c->npos * c->ncell;
    const double scale = 1.0 / std::sqrt((double)c->ncell);
    std::vector<char> launched(R, 0);
    int64_t total = 0;
    for (int r = 0; r < R; r++) {
        sgb_system* s = b->grp[r];
        if ((rc = group_member_ready(b, s))) return rc;
        int64_t it = 0;
        if (s->fp32) {
            SnapArgs<float> sn{1, c->nobs, c->measperiod, 0, (const float*)c->ops, (float*)c->A + 2 * rep_stride * r, (float)scale};
            if (s->ewald_on) rc = s->sun ? run_midpoint_lr_sun<float>(s, c->dt, c->damping, c->tol, c->max_iters, nsteps, &it, &sn)
                                         : run_midpoint_lr<float>(s, c->dt, c->damping, c->tol, c->max_iters, nsteps, &it, &sn);
            else if (nsteps > 0) rc = run_midpoint<float>(s, c->dt, c->damping, c->tol, c->max_iters, nsteps, nullptr, sn, false, s->mid_order);
            else rc = run_midpoint<float>(s, 1.0, 0.0, 1e300, 1, 0, nullptr, sn, false);
        } else {
            SnapArgs<double> sn{1, c->nobs, c->measperiod, 0, (const double*)c->ops, (double*)c->A + 2 * rep_stride * r, scale};
            if (s->ewald_on) rc = s->sun ? run_midpoint_lr_sun<double>(s, c->dt, c->damping, c->tol, c->max_iters, nsteps, &it, &sn)
                                         : run_midpoint_lr<double>(s, c->dt, c->damping, c->tol, c->max_iters, nsteps, &it, &sn);
            else if (nsteps > 0) rc = run_midpoint<double>(s, c->dt, c->damping, c->tol, c->max_iters, nsteps, nullptr, sn, false, s->mid_order);
            else rc = run_midpoint<double>(s, 1.0, 0.0, 1e300, 1, 0, nullptr, sn, false);
        }
        if (rc) return bfail_ext(b, rc, s->err);
        if (s->ewald_on) total += it;
        else launched[r] = 1;
    }
    for (int r = 0; r < R; r++) {
        if (!launched[r]) continue;
        sgb_system* s = b->grp[r];
        Ctrl st;
        if ((rc = read_ctrl(s, &st))) return bfail_ext(b, rc, s->err);
        total += st.iters;
        if (st.status == SGB_ERR_NOCONVERGE) {
            const std::string m = s->sun ? "Schrödinger midpoint method failed to converge in " + std::to_string(c->max_iters) + " iterations."
                                         : "Spherical midpoint method failed to converge to tolerance " + fmt_g(c->tol) + " after " +
                                               std::to_string(c->max_iters) + " iterations.";
            return bfail_ext(b, SGB_ERR_NOCONVERGE, m);
        }
        if (st.status == SGB_ERR_TIMEOUT) return bfail_ext(b, SGB_ERR_TIMEOUT, "a device-side barrier timed out");
        if (st.status != 0) return bfail_ext(b, st.status, "midpoint kernel reported an error");
    }
    c->prof_iters_last = total;
    return group_join(b);
}

// ---------------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------------
extern "C" {

const char* sgb_version(void) { return SGB_VERSION; }

const char* sgb_last_error(const sgb_system* s) { return s ? s->err.c_str() : g_last_error.c_str(); }

int64_t sgb_nsites(const sgb_system* s) { return s ? s->ns : 0; }

int sgb_create(const sgb_desc* d, sgb_system** out) {
    if (!d || !out) return fail(nullptr, SGB_ERR_ARG, "null argument");
    *out = nullptr;
    for (int k = 0; k < 3; k++)
        if (d->dims[k] < 1) return fail(nullptr, SGB_ERR_ARG, "dims must be positive");
    if (d->natoms < 1 || d->natoms > SGB_MAX_SUBLAT) return fail(nullptr, SGB_ERR_ARG, "natoms must be in [1, 64]");
    if (d->mode != SGB_MODE_DIPOLE && d->mode != SGB_MODE_DIPOLE_UNCORRECTED && d->mode != SGB_MODE_SUN)
        return fail(nullptr, SGB_ERR_ARG, "Mode must be `:SUN`, `:dipole`, or `:dipole_uncorrected`");
    if (d->mode == SGB_MODE_SUN && (d->N < 2 || d->N > SGB_MAX_N))
        return fail(nullptr, SGB_ERR_ARG, "SU(N) mode supports N in [2, 5]");
    if (d->precision != SGB_FP32 && d->precision != SGB_FP64) return fail(nullptr, SGB_ERR_ARG, "precision must be SGB_FP32 or SGB_FP64");
    long long ns = (long long)d->dims[0] * d->dims[1] * d->dims[2] * d->natoms;
    if (ns > (1LL << 30)) return fail(nullptr, SGB_ERR_ARG, "too many sites");
    sgb_system* s = new sgb_system();
    s->d = *d;
    s->ns = (int)ns;
    s->ncell = d->dims[0] * d->dims[1] * d->dims[2];
    s->sun = d->mode == SGB_MODE_SUN;
    s->N = s->sun ? d->N : 0;
    s->fp32 = d->precision == SGB_FP32;
    s->mid_order = (s->fp32 && d->mode != SGB_MODE_SUN) ? 4 : 0;
    auto bad = [&](int code) { sgb_destroy(s); return code; };
    cudaError_t e = cudaSetDevice(d->device);
    if (e != cudaSuccess) { fail(nullptr, SGB_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e)); return bad(SGB_ERR_CUDA); }
    cudaDeviceProp prop;
    e = cudaGetDeviceProperties(&prop, d->device);
    if (e != cudaSuccess) { fail(nullptr, SGB_ERR_CUDA, std::string("cudaGetDeviceProperties: ") + cudaGetErrorString(e)); return bad(SGB_ERR_CUDA); }
    if (!prop.cooperativeLaunch) { fail(nullptr, SGB_ERR_CUDA, "device lacks cooperative launch"); return bad(SGB_ERR_CUDA); }
    s->nsm = prop.multiProcessorCount;
    e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { fail(nullptr, SGB_ERR_CUDA, "cudaStreamCreate failed"); return bad(SGB_ERR_CUDA); }
    for (int i = 0; i < 8; i++) cudaEventCreate(&s->ev[i]);
    size_t R = rsize(s);
    int rc = SGB_OK;
    rc |= dmalloc(s, &s->kappa, R * ns);
    rc |= dmalloc(s, &s->h, R * 3 * ns);
    rc |= dmalloc(s, &s->S, R * 3 * ns);
    rc |= dmalloc(s, &s->P, R * 3 * ns);
    rc |= dmalloc(s, &s->H, R * 9 * ns);
    if (s->sun) {
        rc |= dmalloc(s, &s->Z, R * 2 * s->N * ns);
        // quadrupoles, then the packed density (general couplings) of each site
        const size_t qrows = 5 + (size_t)s->N * s->N;
        rc |= dmalloc(s, &s->Q, R * qrows * ns);
        rc |= dmalloc(s, &s->QP, R * qrows * ns);
        rc |= dmalloc(s, &s->QH, R * 3 * qrows * ns);
    }
    rc |= dmalloc(s, (void**)&s->ctrl, sizeof(Ctrl));
    rc |= dmalloc(s, (void**)&s->partials, sizeof(double) * 4 * SGB_ENERGY_BLOCKS);
    rc |= dmalloc(s, (void**)&s->red, sizeof(double) * 8);
    if (rc) { g_last_error = s->err; return bad(SGB_ERR_NOMEM); }
    cudaMemset(s->S, 0, R * 3 * ns);
    if (s->sun) cudaMemset(s->Z, 0, R * 2 * s->N * ns);
    cudaMemset(s->ctrl, 0, sizeof(Ctrl));
    // defaults: kappa = 1, g = 2I, no field, no couplings
    s->kappa_h.assign(ns, 1.0);
    s->g_h.assign(9 * ns, 0.0);
    for (long long i = 0; i < ns; i++) s->g_h[9 * i] = s->g_h[9 * i + 4] = s->g_h[9 * i + 8] = 2.0;
    s->onsite_h.assign(s->sun ? (size_t)2 * s->N * s->N * d->natoms : (size_t)28 * d->natoms, 0.0);
    *out = s;
    return SGB_OK;
}

void sgb_destroy(sgb_system* s) {
    if (!s) return;
    if (s->stream) cudaStreamSynchronize(s->stream);
    sgb_detach_corrs(s->corrs);
    dfree(s->kappa); dfree(s->h); dfree(s->tables);
    { void* p = s->nbr; dfree(p); } dfree(s->S); dfree(s->P); dfree(s->H);
    dfree(s->Z); dfree(s->Q); dfree(s->QP); dfree(s->QH);
    void* p = s->ctrl; dfree(p);
    p = s->partials; dfree(p);
    p = s->red; dfree(p);
    p = s->dbuf; dfree(p);
    p = s->mc_perm; dfree(p);
    p = s->mc_part; dfree(p);
    dfree(s->inh_dev);
    dfree(s->gtab);
    ewald_free(s);
    p = s->lr_grad; dfree(p);
    p = s->lr_sun; dfree(p);
    dfree(s->flush);
    if (s->stage) cudaFreeHost(s->stage);
    for (int i = 0; i < 8; i++) if (s->ev[i]) cudaEventDestroy(s->ev[i]);
    for (int i = 0; i < 2; i++) if (s->tev[i]) cudaEventDestroy(s->tev[i]);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

int sgb_set_sites(sgb_system* s, const double* kappa, const double* g, const double* field) {
    if (!s || !kappa || !g) return fail(s, SGB_ERR_ARG, "kappa and g are required");
    const int ns = s->ns;
    s->kappa_h.assign(kappa, kappa + ns);
    s->g_h.assign(g, g + 9 * (size_t)ns);
    s->field_h.assign(3 * (size_t)ns, 0.0);
    if (field) s->field_h.assign(field, field + 3 * (size_t)ns);
    // Zeeman gradient h = g' B (Interactions.jl:520-523), stored [3][ns]
    std::vector<double> hh(3 * (size_t)ns, 0.0);
    bool any = false;
    for (int i = 0; i < ns; i++) {
        const double* gi = s->g_h.data() + 9 * (size_t)i;
        const double* B = s->field_h.data() + 3 * (size_t)i;
        for (int r = 0; r < 3; r++) {
            double v = gi[0 + 3 * r] * B[0] + gi[1 + 3 * r] * B[1] + gi[2 + 3 * r] * B[2];
            hh[(size_t)r * ns + i] = v;
            any |= v != 0.0;
        }
    }
    s->has_field = any;
    if (int rc0 = ensure_stage(s, 3 * (size_t)ns * sizeof(double))) return rc0;
    if (s->fp32) {
        float* k = reinterpret_cast<float*>(s->stage);
        for (int i = 0; i < ns; i++) k[i] = (float)kappa[i];
        CK(cudaMemcpy(s->kappa, k, sizeof(float) * ns, cudaMemcpyHostToDevice));
        for (size_t i = 0; i < 3 * (size_t)ns; i++) k[i] = (float)hh[i];
        CK(cudaMemcpy(s->h, k, sizeof(float) * 3 * ns, cudaMemcpyHostToDevice));
    } else {
        CK(cudaMemcpy(s->kappa, kappa, sizeof(double) * ns, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(s->h, hh.data(), sizeof(double) * 3 * ns, cudaMemcpyHostToDevice));
    }
    s->sites_set = true;
    s->tables_dirty = true;
    return ewald_upload_g(s);
}

int sgb_set_onsite(sgb_system* s, int32_t atom, const double* coeffs) {
    if (!s || !coeffs) return fail(s, SGB_ERR_ARG, "null argument");
    if (atom < 0 || atom >= s->d.natoms) return fail(s, SGB_ERR_ARG, "Atom index " + std::to_string(atom + 1) + " is out of range.");
    if (!s->sun) {
        // StevensExpansion(c) requires time-reversal invariance: no odd k (Types.jl:18-21)
        std::copy(coeffs, coeffs + 28, s->onsite_h.begin() + 28 * atom);
    } else {
        const int N = s->N;
        // Hermiticity check, as onsite_coupling (OnsiteCoupling.jl:4)
        for (int r = 0; r < N; r++)
            for (int c = 0; c < N; c++) {
                double ar = coeffs[2 * (r + N * c)], ai = coeffs[2 * (r + N * c) + 1];
                double br = coeffs[2 * (c + N * r)], bi = coeffs[2 * (c + N * r) + 1];
                if (std::fabs(ar - br) > 1e-10 * (1 + std::fabs(ar)) || std::fabs(ai + bi) > 1e-10 * (1 + std::fabs(ai)))
                    return fail(s, SGB_ERR_ARG, "Operator is not Hermitian");
            }
        std::copy(coeffs, coeffs + 2 * N * N, s->onsite_h.begin() + (size_t)2 * N * N * atom);
    }
    s->inh_onsite = false;
    s->tables_dirty = true;
    return SGB_OK;
}

int sgb_set_bonds(sgb_system* s, const sgb_bond* bonds, int32_t nbonds) {
    if (!s || (nbonds > 0 && !bonds) || nbonds < 0) return fail(s, SGB_ERR_ARG, "invalid bond list");
    for (int k = 0; k < nbonds; k++) {
        const sgb_bond& b = bonds[k];
        // validate_bond (PairExchange.jl:1-8)
        if (b.i == b.j && b.n[0] == 0 && b.n[1] == 0 && b.n[2] == 0) return fail(s, SGB_ERR_ARG, "Bond must connect different atoms.");
        if (b.i < 0 || b.i >= s->d.natoms) return fail(s, SGB_ERR_ARG, "Atom index " + std::to_string(b.i + 1) + " is out of range.");
        if (b.j < 0 || b.j >= s->d.natoms) return fail(s, SGB_ERR_ARG, "Atom index " + std::to_string(b.j + 1) + " is out of range.");
        if (b.biquad_kind < 0 || b.biquad_kind > 2) return fail(s, SGB_ERR_ARG, "biquad_kind must be 0, 1 or 2");
    }
    s->bonds_h.assign(bonds, bonds + nbonds);
    // general terms refer to the previous bond list: the caller sets them again
    s->gen_bond_h.clear();
    s->gen_A_h.clear();
    s->gen_B_h.clear();
    s->inh_bonds = false;
    s->site_bonds_h.clear();
    s->bonds_set = true;
    s->tables_dirty = true;
    return SGB_OK;
}

int sgb_set_general(sgb_system* s, const int32_t* bond, int32_t nterms, const double* A, const double* B) {
    if (!s || nterms < 0 || (nterms > 0 && (!bond || !A || !B))) return fail(s, SGB_ERR_ARG, "invalid general terms");
    if (nterms > 0 && !s->sun) return fail(s, SGB_ERR_ARG, "General couplings require mode :SUN");
    if (nterms > 0 && s->inh_bonds) return fail(s, SGB_ERR_ARG, "general couplings are supported on per-sublattice systems only");
    const int N = s->N;
    for (int t = 0; t < nterms; t++) {
        if (bond[t] < 0 || bond[t] >= (int)s->bonds_h.size()) return fail(s, SGB_ERR_ARG, "general term on an unknown bond");
        for (const double* Mx : {A + (size_t)2 * N * N * t, B + (size_t)2 * N * N * t})
            for (int r = 0; r < N; r++)
                for (int c = 0; c < N; c++) {
                    const double ar = Mx[2 * (r + N * c)], ai = Mx[2 * (r + N * c) + 1];
                    const double br = Mx[2 * (c + N * r)], bi = Mx[2 * (c + N * r) + 1];
                    if (std::fabs(ar - br) > 1e-10 * (1 + std::fabs(ar)) || std::fabs(ai + bi) > 1e-10 * (1 + std::fabs(ai)))
                        return fail(s, SGB_ERR_ARG, "Operator is not Hermitian");
                }
    }
    s->gen_bond_h.assign(bond, bond + nterms);
    s->gen_A_h.assign(A, A + (size_t)2 * N * N * nterms);
    s->gen_B_h.assign(B, B + (size_t)2 * N * N * nterms);
    s->tables_dirty = true;
    return SGB_OK;
}

int sgb_set_bonds_at(sgb_system* s, const sgb_site_bond* bonds, int64_t nbonds) {
    if (!s || (nbonds > 0 && !bonds) || nbonds < 0) return fail(s, SGB_ERR_ARG, "invalid bond list");
    if (2 * nbonds > (int64_t)INT32_MAX) return fail(s, SGB_ERR_ARG, "too many couplings");
    const int* L = s->d.dims;
    for (int64_t k = 0; k < nbonds; k++) {
        const sgb_bond& b = bonds[k].bond;
        const int32_t* c = bonds[k].cell;
        if (b.i < 0 || b.i >= s->d.natoms) return fail(s, SGB_ERR_ARG, "Atom index " + std::to_string(b.i + 1) + " is out of range.");
        if (b.j < 0 || b.j >= s->d.natoms) return fail(s, SGB_ERR_ARG, "Atom index " + std::to_string(b.j + 1) + " is out of range.");
        if (b.biquad_kind < 0 || b.biquad_kind > 2) return fail(s, SGB_ERR_ARG, "biquad_kind must be 0, 1 or 2");
        for (int d = 0; d < 3; d++)
            if (c[d] < 0 || c[d] >= L[d]) return fail(s, SGB_ERR_ARG, "cell index out of range");
    }
    if (!s->gen_bond_h.empty()) return fail(s, SGB_ERR_ARG, "general couplings are supported on per-sublattice systems only");
    s->site_bonds_h.assign(bonds, bonds + nbonds);
    s->inh_bonds = true;
    s->bonds_set = true;
    s->tables_dirty = true;
    return SGB_OK;
}

int sgb_set_onsite_at(sgb_system* s, const double* coeffs) {
    if (!s || !coeffs) return fail(s, SGB_ERR_ARG, "null argument");
    const int ns = s->ns;
    if (s->sun) {
        const int N = s->N;
        for (int i = 0; i < ns; i++) {
            const double* m = coeffs + (size_t)2 * N * N * i;
            for (int r = 0; r < N; r++)
                for (int c = 0; c < N; c++) {
                    double ar = m[2 * (r + N * c)], ai = m[2 * (r + N * c) + 1];
                    double br = m[2 * (c + N * r)], bi = m[2 * (c + N * r) + 1];
                    if (std::fabs(ar - br) > 1e-10 * (1 + std::fabs(ar)) || std::fabs(ai + bi) > 1e-10 * (1 + std::fabs(ai)))
                        return fail(s, SGB_ERR_ARG, "Operator is not Hermitian");
                }
        }
        s->onsite_site_h.assign(coeffs, coeffs + (size_t)2 * N * N * ns);
    } else {
        s->onsite_site_h.assign(coeffs, coeffs + (size_t)28 * ns);
    }
    s->inh_onsite = true;
    s->tables_dirty = true;
    return SGB_OK;
}

int sgb_set_dipole_dipole(sgb_system* s, double mu0_muB2, const double* demag, const double* latvecs,
                          const double* positions) {
    if (!s) return fail(s, SGB_ERR_ARG, "null handle");
    ewald_free(s);
    if (mu0_muB2 == 0.0) return SGB_OK;
    if (!demag || !latvecs || !positions) return fail(s, SGB_ERR_ARG, "demag, latvecs and positions are required");
    if (!s->sites_set) return fail(s, SGB_ERR_STATE, "sgb_set_sites must be called before sgb_set_dipole_dipole");
    EwaldGeom G{};
    const int* L = s->d.dims;
    G.L[0] = L[0]; G.L[1] = L[1]; G.L[2] = L[2];
    G.na = s->d.natoms;
    G.mu0 = mu0_muB2;
    for (int q = 0; q < 9; q++) { G.lat[q] = latvecs[q]; G.demag[q] = demag[q]; }
    // supercell vectors and reciprocals (Ewald.jl:65-67), σ = V^(1/3)/3, cut-offs 6√2σ and
    // 6√2/σ, image ranges (Ewald.jl:70-89)
    for (int c = 0; c < 3; c++)
        for (int r = 0; r < 3; r++) G.sup[r + 3 * c] = latvecs[r + 3 * c] * L[c];
    const double* a = G.sup;
    const double det = a[0] * (a[4] * a[8] - a[7] * a[5]) - a[3] * (a[1] * a[8] - a[7] * a[2]) + a[6] * (a[1] * a[5] - a[4] * a[2]);
    if (!(std::fabs(det) > 0)) return fail(s, SGB_ERR_ARG, "lattice vectors are degenerate");
    double inv[9];
    inv[0] = (a[4] * a[8] - a[7] * a[5]) / det; inv[3] = (a[6] * a[5] - a[3] * a[8]) / det; inv[6] = (a[3] * a[7] - a[6] * a[4]) / det;
    inv[1] = (a[7] * a[2] - a[1] * a[8]) / det; inv[4] = (a[0] * a[8] - a[6] * a[2]) / det; inv[7] = (a[6] * a[1] - a[0] * a[7]) / det;
    inv[2] = (a[1] * a[5] - a[4] * a[2]) / det; inv[5] = (a[3] * a[2] - a[0] * a[5]) / det; inv[8] = (a[0] * a[4] - a[3] * a[1]) / det;
    const double twopi = 6.283185307179586476925;
    for (int c = 0; c < 3; c++)
        for (int r = 0; r < 3; r++) G.rec[r + 3 * c] = twopi * inv[c + 3 * r];
    G.V = std::fabs(det);
    G.sig = std::cbrt(G.V) / 3;
    G.rmax = 6 * std::sqrt(2.0) * G.sig;
    G.kmax = 6 * std::sqrt(2.0) / G.sig;
    for (int k = 0; k < 3; k++) {
        const double* ak = G.sup + 3 * k;
        const double* bk = G.rec + 3 * k;
        const double nb = std::sqrt(bk[0] * bk[0] + bk[1] * bk[1] + bk[2] * bk[2]);
        const double nak = std::sqrt(ak[0] * ak[0] + ak[1] * ak[1] + ak[2] * ak[2]);
        const double ab = ak[0] * bk[0] + ak[1] * bk[1] + ak[2] * bk[2];
        G.nmax[k] = (int)std::lround(G.rmax / (ab / nb) + 1e-6) + 1;
        G.mmax[k] = (int)std::lround(G.kmax / (ab / nak) + 1e-6);
    }
    EwaldDev& E = s->ew;
    E.L[0] = L[0]; E.L[1] = L[1]; E.L[2] = L[2];
    E.na = G.na;
    const int ncell = s->ncell, na = G.na;
    E.nm = L[2] * L[1] * (L[0] / 2 + 1);
    const size_t ncomp = (size_t)9 * na * na;
    double* A = nullptr;
    double* pos_d = nullptr;
    int rc;
    if ((rc = dmalloc(s, (void**)&E.g, sizeof(double) * 9 * (size_t)s->ns)) || (rc = dmalloc(s, (void**)&E.mu, sizeof(double) * 3 * (size_t)s->ns)) ||
        (rc = dmalloc(s, (void**)&E.phi, sizeof(double) * 3 * (size_t)s->ns)) ||
        (rc = dmalloc(s, (void**)&E.FA, sizeof(cufftDoubleComplex) * ncomp * E.nm)) ||
        (rc = dmalloc(s, (void**)&E.Fmu, sizeof(cufftDoubleComplex) * 3 * na * (size_t)E.nm)) ||
        (rc = dmalloc(s, (void**)&E.Fphi, sizeof(cufftDoubleComplex) * 3 * na * (size_t)E.nm)) ||
        (rc = dmalloc(s, (void**)&s->ew_part, sizeof(double) * EWALD_PART_BLOCKS)) ||
        (rc = dmalloc(s, (void**)&A, sizeof(double) * ncomp * ncell)) || (rc = dmalloc(s, (void**)&pos_d, sizeof(double) * 3 * na))) {
        void* p = A; dfree(p); p = pos_d; dfree(p);
        ewald_free(s);
        return rc;
    }
    s->ewald_on = true;
    E.Areal = A;   // kept for the LocalSampler's pairwise energy updates; freed by ewald_free
    auto bail = [&](const char* what) {
        void* p = pos_d; dfree(p);
        ewald_free(s);
        return fail(s, SGB_ERR_CUDA, what);
    };
    if (cudaMemcpy(pos_d, positions, sizeof(double) * 3 * na, cudaMemcpyHostToDevice) != cudaSuccess) return bail("position upload failed");
    if (ewald_upload_g(s)) return bail("g upload failed");
    if (ewald_precompute(G, pos_d, A, s->stream)) return bail("Ewald matrix launch failed");
    s->launches++;
    int n[3] = {L[2], L[1], L[0]};
    cufftHandle pa;
    if (cufftPlanMany(&pa, 3, n, nullptr, 1, ncell, nullptr, 1, E.nm, CUFFT_D2Z, (int)ncomp) != CUFFT_SUCCESS) return bail("cuFFT plan failed");
    cufftSetStream(pa, s->stream);
    const bool ok = cufftExecD2Z(pa, A, E.FA) == CUFFT_SUCCESS;
    cudaStreamSynchronize(s->stream);
    cufftDestroy(pa);
    if (!ok) return bail("cuFFT transform failed");
    if (cufftPlanMany(&E.plan_f, 3, n, nullptr, 1, ncell, nullptr, 1, E.nm, CUFFT_D2Z, 3 * na) != CUFFT_SUCCESS) return bail("cuFFT plan failed");
    E.have_f = true;
    if (cufftPlanMany(&E.plan_b, 3, n, nullptr, 1, E.nm, nullptr, 1, ncell, CUFFT_Z2D, 3 * na) != CUFFT_SUCCESS) return bail("cuFFT plan failed");
    E.have_b = true;
    void* p = pos_d; dfree(p);
    return SGB_OK;
}

int sgb_set_state(sgb_system* s, const double* dipoles, const double* coherents) {
    if (!s) return fail(s, SGB_ERR_ARG, "null handle");
    int rc = ensure_tables(s);
    if (rc) return rc;
    const int ns = s->ns;
    const size_t R = rsize(s);
    if (!s->sun) {
        if (!dipoles) return fail(s, SGB_ERR_ARG, "dipoles required in dipole mode");
        if ((rc = ensure_stage(s, R * 3 * (size_t)ns))) return rc;
        for (int i = 0; i < ns; i++)
            for (int c = 0; c < 3; c++) {
                if (s->fp32) reinterpret_cast<float*>(s->stage)[(size_t)c * ns + i] = (float)dipoles[3 * (size_t)i + c];
                else reinterpret_cast<double*>(s->stage)[(size_t)c * ns + i] = dipoles[3 * (size_t)i + c];
            }
        CK(cudaMemcpyAsync(s->S, s->stage, R * 3 * ns, cudaMemcpyHostToDevice, s->stream));
    } else {
        if (!coherents) return fail(s, SGB_ERR_ARG, "coherents required in SU(N) mode");
        const int N = s->N;
        if ((rc = ensure_stage(s, R * 2 * N * (size_t)ns))) return rc;
        for (int i = 0; i < ns; i++)
            for (int c = 0; c < 2 * N; c++) {
                double v = coherents[(size_t)2 * N * i + c];
                if (s->fp32) reinterpret_cast<float*>(s->stage)[(size_t)c * ns + i] = (float)v;
                else reinterpret_cast<double*>(s->stage)[(size_t)c * ns + i] = v;
            }
        CK(cudaMemcpyAsync(s->Z, s->stage, R * 2 * N * ns, cudaMemcpyHostToDevice, s->stream));
        rc = s->fp32 ? do_refresh<float>(s) : do_refresh<double>(s);
        if (rc) return rc;
    }
    CK(cudaStreamSynchronize(s->stream));
    s->state_set = true;
    return SGB_OK;
}

int sgb_get_state(sgb_system* s, double* dipoles, double* coherents) {
    if (!s) return fail(s, SGB_ERR_ARG, "null handle");
    const int ns = s->ns;
    const size_t R = rsize(s);
    int rc = SGB_OK;
    if (dipoles) {
        if ((rc = ensure_stage(s, R * 3 * (size_t)ns))) return rc;
        CK(cudaMemcpyAsync(s->stage, s->S, R * 3 * ns, cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        for (int i = 0; i < ns; i++)
            for (int c = 0; c < 3; c++)
                dipoles[3 * (size_t)i + c] = s->fp32 ? (double)reinterpret_cast<float*>(s->stage)[(size_t)c * ns + i]
                                                     : reinterpret_cast<double*>(s->stage)[(size_t)c * ns + i];
    }
    if (coherents && s->sun) {
        const int N = s->N;
        if ((rc = ensure_stage(s, R * 2 * N * (size_t)ns))) return rc;
        CK(cudaMemcpyAsync(s->stage, s->Z, R * 2 * N * ns, cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        for (int i = 0; i < ns; i++)
            for (int c = 0; c < 2 * N; c++)
                coherents[(size_t)2 * N * i + c] = s->fp32 ? (double)reinterpret_cast<float*>(s->stage)[(size_t)c * ns + i]
                                                           : reinterpret_cast<double*>(s->stage)[(size_t)c * ns + i];
    }
    return SGB_OK;
}

int sgb_langevin_kernel(const sgb_system* s, int32_t* cluster) {
    if (!s || !cluster) return SGB_ERR_ARG;
    *cluster = s->heun_cluster;
    return SGB_OK;
}

int sgb_set_langevin_cluster(sgb_system* s, int32_t mode) {
    if (!s) return fail(nullptr, SGB_ERR_ARG, "null handle");
    if (mode < -1 || mode > 1) return fail(s, SGB_ERR_ARG, "mode must be -1 (timed choice), 0 (grid) or 1 (cluster)");
    if (mode == 1) {
        int rc = ensure_tables(s);
        if (rc) return rc;
        const int cs = s->fp32 ? cluster_size<float>(s) : cluster_size<double>(s);
        if (cs == 0) return fail(s, SGB_ERR_ARG, "the lattice is too large for one thread-block cluster");
        s->heun_cluster = cs;
    } else {
        s->heun_cluster = mode;
    }
    s->heun_forced = mode >= 0;
    return SGB_OK;
}

int sgb_set_midpoint_predictor(sgb_system* s, int32_t order) {
    if (!s) return fail(nullptr, SGB_ERR_ARG, "null handle");
    if (order < 0 || order > 4) return fail(s, SGB_ERR_ARG, "predictor order must be in 0..4");
    s->mid_order = order;
    return SGB_OK;
}

int sgb_energy_grad(sgb_system* s, double* grad) {
    if (!s || !grad) return fail(s, SGB_ERR_ARG, "null argument");
    int rc = ensure_tables(s);
    if (rc) return rc;
    size_t n = s->sun ? (size_t)2 * s->N * s->ns : (size_t)3 * s->ns;
    if ((rc = ensure_dbuf(s, n))) return rc;
    if (!s->sun) {
        rc = s->fp32 ? dip_launch_grad<float>(s->mf, (const float*)s->S, s->dbuf, s->stream)
                     : dip_launch_grad<double>(s->md, (const double*)s->S, s->dbuf, s->stream);
        if (rc == SGB_OK && s->ewald_on) {
            s->launches++;
            rc = s->fp32 ? ewald_add<float>(s, (const float*)s->S, s->dbuf, nullptr)
                         : ewald_add<double>(s, (const double*)s->S, s->dbuf, nullptr);
            if (rc) return rc;
        }
    } else {
        rc = s->fp32 ? sun_launch_grad<float>(s->mf, (const float*)s->Z, (const float*)s->S, (const float*)s->Q, s->dbuf, s->stream)
                     : sun_launch_grad<double>(s->md, (const double*)s->Z, (const double*)s->S, (const double*)s->Q, s->dbuf, s->stream);
        if (rc == SGB_OK && s->ewald_on) {
            s->launches++;
            if ((rc = s->fp32 ? ewald_add_sun<float>(s, s->dbuf, nullptr) : ewald_add_sun<double>(s, s->dbuf, nullptr))) return rc;
        }
    }
    s->launches++;
    if (rc) return cuda_fail(s, cudaGetLastError(), "gradient launch");
    CK(cudaMemcpyAsync(grad, s->dbuf, n * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return SGB_OK;
}

int sgb_energy(sgb_system* s, double* E, double* M3) {
    if (!s) return fail(s, SGB_ERR_ARG, "null handle");
    int rc = ensure_tables(s);
    if (rc) return rc;
    int nb = std::min(SGB_ENERGY_BLOCKS, (s->ns + SGB_BLOCK - 1) / SGB_BLOCK);
    if (!s->sun) {
        rc = s->fp32 ? dip_launch_energy<float>(s->mf, (const float*)s->S, s->partials, nb, s->stream)
                     : dip_launch_energy<double>(s->md, (const double*)s->S, s->partials, nb, s->stream);
    } else {
        rc = s->fp32 ? sun_launch_energy<float>(s->mf, (const float*)s->Z, (const float*)s->S, (const float*)s->Q, s->partials, nb, s->stream)
                     : sun_launch_energy<double>(s->md, (const double*)s->Z, (const double*)s->S, (const double*)s->Q, s->partials, nb, s->stream);
    }
    s->launches++;
    if (rc) return cuda_fail(s, cudaGetLastError(), "energy launch");
    if ((rc = util_launch_reduce(s->partials, nb, 4, s->red, s->stream))) return cuda_fail(s, cudaGetLastError(), "reduce launch");
    s->launches++;
    double out[4];
    CK(cudaMemcpyAsync(out, s->red, sizeof(out), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    if (s->ewald_on) {
        double Ed = 0;
        rc = s->fp32 ? ewald_add<float>(s, (const float*)s->S, nullptr, &Ed) : ewald_add<double>(s, (const double*)s->S, nullptr, &Ed);
        if (rc) return rc;
        out[0] += Ed;
    }
    if (E) *E = out[0];
    if (M3) { M3[0] = out[1]; M3[1] = out[2]; M3[2] = out[3]; }
    return SGB_OK;
}

int sgb_langevin(sgb_system* s, double dt, double damping, double kT, uint64_t seed, uint64_t step0, int32_t nsteps,
                 const double* noise) {
    if (!s) return fail(s, SGB_ERR_ARG, "null handle");
    // Langevin constructor checks (src/Integrators.jl:61-73)
    if (damping == 0.0) return fail(s, SGB_ERR_ARG, "Use ImplicitMidpoint instead for energy-conserving dynamics");
    if (!(dt > 0)) return fail(s, SGB_ERR_ARG, "Select positive dt");
    if (kT < 0) return fail(s, SGB_ERR_ARG, "Select nonnegative kT");
    if (damping < 0) return fail(s, SGB_ERR_ARG, "Select positive damping");
    if (nsteps < 0) return fail(s, SGB_ERR_ARG, "nsteps must be nonnegative");
    if (nsteps == 0) return SGB_OK;
    int rc = ensure_tables(s);
    if (rc) return rc;
    if (!s->state_set) return fail(s, SGB_ERR_STATE, "sgb_set_state must be called before stepping");
    if (s->ewald_on && s->sun)
        return s->fp32 ? run_langevin_lr_sun<float>(s, dt, damping, kT, seed, step0, nsteps, noise)
                       : run_langevin_lr_sun<double>(s, dt, damping, kT, seed, step0, nsteps, noise);
    if (s->ewald_on)
        return s->fp32 ? run_langevin_lr<float>(s, dt, damping, kT, seed, step0, nsteps, noise)
                       : run_langevin_lr<double>(s, dt, damping, kT, seed, step0, nsteps, noise);
    return s->fp32 ? run_langevin<float>(s, dt, damping, kT, seed, step0, nsteps, noise)
                   : run_langevin<double>(s, dt, damping, kT, seed, step0, nsteps, noise);
}

int sgb_langevin_noise(sgb_system* s, uint64_t seed, uint64_t step, double* out) {
    if (!s || !out) return fail(s, SGB_ERR_ARG, "null argument");
    size_t n = s->sun ? (size_t)2 * s->N * s->ns : (size_t)3 * s->ns;
    int rc = ensure_dbuf(s, n);
    if (rc) return rc;
    rc = s->fp32 ? util_launch_noise_export<float>(s->sun, s->N, s->ns, seed, step, s->dbuf, s->stream)
                 : util_launch_noise_export<double>(s->sun, s->N, s->ns, seed, step, s->dbuf, s->stream);
    s->launches++;
    if (rc) return cuda_fail(s, cudaGetLastError(), "noise launch");
    CK(cudaMemcpyAsync(out, s->dbuf, n * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return SGB_OK;
}

int sgb_midpoint(sgb_system* s, double dt, double damping, double tol, int32_t max_iters, int32_t nsteps, int64_t* iters_out) {
    if (!s) return fail(s, SGB_ERR_ARG, "null handle");
    // ImplicitMidpoint constructor checks (src/Integrators.jl:113-130)
    if (!(dt > 0)) return fail(s, SGB_ERR_ARG, "Select positive dt");
    if (damping < 0) return fail(s, SGB_ERR_ARG, "Select nonnegative damping");
    if (tol < 0 || max_iters < 1 || nsteps < 0) return fail(s, SGB_ERR_ARG, "invalid tol, max_iters or nsteps");
    if (iters_out) *iters_out = 0;
    if (nsteps == 0) return SGB_OK;
    int rc = ensure_tables(s);
    if (rc) return rc;
    if (!s->state_set) return fail(s, SGB_ERR_STATE, "sgb_set_state must be called before stepping");
    if (s->ewald_on && s->sun)
        return s->fp32 ? run_midpoint_lr_sun<float>(s, dt, damping, tol, max_iters, nsteps, iters_out)
                       : run_midpoint_lr_sun<double>(s, dt, damping, tol, max_iters, nsteps, iters_out);
    if (s->ewald_on)
        return s->fp32 ? run_midpoint_lr<float>(s, dt, damping, tol, max_iters, nsteps, iters_out)
                       : run_midpoint_lr<double>(s, dt, damping, tol, max_iters, nsteps, iters_out);
    if (s->fp32) {
        SnapArgs<float> sn{};
        return run_midpoint<float>(s, dt, damping, tol, max_iters, nsteps, iters_out, sn, true, s->mid_order);
    }
    SnapArgs<double> sn{};
    return run_midpoint<double>(s, dt, damping, tol, max_iters, nsteps, iters_out, sn, true, s->mid_order);
}

int sgb_local_sweeps(sgb_system* s, double kT, double nsweeps, const sgb_proposal* prop, uint64_t seed, uint64_t sweep0,
                     const double* rand, double* dE, double* dS3) {
    if (!s) return fail(s, SGB_ERR_ARG, "null handle");
    if (!(kT >= 0)) return fail(s, SGB_ERR_ARG, "Select nonnegative kT");
    if (!(nsweeps >= 0) || nsweeps > 1e9) return fail(s, SGB_ERR_ARG, "nsweeps must be nonnegative");
    if (!prop || prop->n < 1 || prop->n > 4) return fail(s, SGB_ERR_ARG, "a proposal mixture has 1 to 4 functions");
    McArgs A{};
    double wsum = 0;
    for (int i = 0; i < prop->n; i++) {
        const int k = prop->kind[i];
        if (k != SGB_PROPOSE_UNIFORM && k != SGB_PROPOSE_FLIP && k != SGB_PROPOSE_DELTA)
            return fail(s, SGB_ERR_ARG, "unknown proposal kind");
        if (!(prop->weight[i] >= 0)) return fail(s, SGB_ERR_ARG, "proposal weights must be nonnegative");
        if (k == SGB_PROPOSE_DELTA && !(prop->magnitude[i] >= 0)) return fail(s, SGB_ERR_ARG, "propose_delta magnitude must be nonnegative");
        wsum += prop->weight[i];
    }
    if (!(wsum > 0)) return fail(s, SGB_ERR_ARG, "proposal weights must not all be zero");
    // cumulative probabilities (Samplers.jl:77-81)
    double run = 0;
    for (int i = 0; i < prop->n; i++) {
        run += prop->weight[i] / wsum;
        A.kind[i] = prop->kind[i];
        A.cum[i] = run;
        A.mag[i] = prop->magnitude[i];
    }
    A.nkind = prop->n;
    if (dE) *dE = 0;
    if (dS3) dS3[0] = dS3[1] = dS3[2] = 0;
    const double nfull = std::floor(nsweeps);
    const double frac = nsweeps - nfull;
    const int total = (int)nfull + (frac > 0 ? 1 : 0);
    if (total == 0) return SGB_OK;
    int rc = ensure_colors(s);
    if (rc) return rc;
    if (!s->state_set) return fail(s, SGB_ERR_STATE, "sgb_set_state must be called before stepping");
    A.perm = s->mc_perm;
    A.ncol = (int)s->coff_h.size() - 1;
    for (int c = 0; c <= A.ncol; c++) A.coff[c] = s->coff_h[c];
    A.nsweeps = total;
    A.frac = frac > 0 ? frac : 1.0;
    A.kT = kT;
    A.seed = seed;
    A.sweep0 = sweep0;
    double out[4];
    rc = s->fp32 ? run_local_sweeps<float>(s, A, rand, out) : run_local_sweeps<double>(s, A, rand, out);
    if (rc) return rc;
    if (dE) *dE = out[0];
    if (dS3) { dS3[0] = out[1]; dS3[1] = out[2]; dS3[2] = out[3]; }
    return SGB_OK;
}

// minimize_energy! (Optimization.jl:102-166), FP64 systems: dipoles, or coherent states
// (gradient HZ, complex tangent projection; the dipoles and quadrupoles are refreshed
// from the kets before every evaluation). Riemannian
// nonlinear conjugate gradient on the unit spheres: Hager-Zhang β with the η = 0.4 lower
// bound (Optim.jl ConjugateGradient defaults), a bracketing line search (secant on φ',
// else bisection) on φ(α) = E(κ·normalize(x + α d)) that accepts the strong Wolfe
// conditions, first step ψ0/|g|∞ (Hager & Zhang's I0 with |x|∞ = 1), then
// α_prev·φ'_prev(0)/φ'(0), capped at αmax = 10 (the bracketing phase may expand past
// it, which lets a jittered start leave a saddle). Converged when the largest projected-gradient component is at most
// 1e-12·characteristic_energy_scale or the largest step component at most 1e-12
// (Optimization.jl:149-156); on a failed line search the direction restarts from -g
// once, as optimize_with_restarts does (Optimization.jl:59-70).
int sgb_minimize_energy(sgb_system* s, int32_t maxiters, double jitter, uint64_t seed, int32_t* converged,
                        int32_t* niters, double* energy_out) {
    if (!s) return fail(s, SGB_ERR_ARG, "null handle");
    if (s->fp32) return fail(s, SGB_ERR_ARG, "minimize_energy needs an FP64 system (its tolerances are 1e-12)");
    if (maxiters < 0 || !(jitter >= 0)) return fail(s, SGB_ERR_ARG, "invalid maxiters or jitter");
    int rc = ensure_tables(s);
    if (rc) return rc;
    if (!s->state_set) return fail(s, SGB_ERR_STATE, "sgb_set_state must be called first");
    const int ns = s->ns;
    const int grid = opt_grid(ns);
    const int K = s->sun ? 2 * s->N : 3;            // reals per site
    const double gdiv = s->sun ? 2.0 : 1.0;          // the kernels' ket gradient is 2·√κ·HZ
    double *x = nullptr, *g = nullptr, *d = nullptr, *grad = nullptr, *part = nullptr;
    struct Guard {
        double** p[5];
        ~Guard() { for (auto q : p) if (*q) { cudaFree(*q); *q = nullptr; } }
    } guard{{&x, &g, &d, &grad, &part}};
    const size_t vb = sizeof(double) * K * (size_t)ns;
    if ((rc = dmalloc(s, (void**)&x, vb)) || (rc = dmalloc(s, (void**)&g, vb)) || (rc = dmalloc(s, (void**)&d, vb)) ||
        (rc = dmalloc(s, (void**)&grad, vb)) || (rc = dmalloc(s, (void**)&part, sizeof(double) * 10 * grid)))
        return rc;
    double* S = (double*)(s->sun ? s->Z : s->S);   // the optimised state: dipoles or kets
    const double* kap = (const double*)s->kappa;
    cudaStream_t st = s->stream;
    CK(cudaMemsetAsync(g, 0, vb, st));
    CK(cudaMemsetAsync(d, 0, vb, st));
    if (opt_launch_init(K, S, kap, ns, jitter, seed, x, st)) return cuda_fail(s, cudaGetLastError(), "optimizer launch");
    const int nbE = std::min(SGB_ENERGY_BLOCKS, (ns + SGB_BLOCK - 1) / SGB_BLOCK);
    std::vector<double> hp(10 * (size_t)grid);
    auto pull = [&](int K, double* out, const bool* is_max) -> int {
        CK(cudaMemcpyAsync(hp.data(), part, sizeof(double) * K * grid, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        for (int k = 0; k < K; k++) {
            double a = 0;
            for (int b = 0; b < grid; b++) a = is_max[k] ? std::max(a, hp[(size_t)b * K + k]) : a + hp[(size_t)b * K + k];
            out[k] = a;
        }
        return SGB_OK;
    };
    int nevals = 0;
    // E and φ'(α) at κ·normalize(x + α d); the gradient stays in `grad`
    auto eval = [&](double alpha, double* f, double* dphi) -> int {
        nevals++;
        int lrc;
        if (!s->sun) {
            lrc = opt_launch_point(K, x, d, alpha, kap, ns, S, st) || dip_launch_grad<double>(s->md, S, grad, st) ||
                  dip_launch_energy<double>(s->md, S, s->partials, nbE, st);
        } else {
            double* D = (double*)s->S;
            double* Q = (double*)s->Q;
            lrc = opt_launch_point(K, x, d, alpha, kap, ns, S, st) || sun_launch_refresh<double>(s->md, S, D, Q, st) ||
                  sun_launch_grad<double>(s->md, S, D, Q, grad, st) || sun_launch_energy<double>(s->md, S, D, Q, s->partials, nbE, st);
        }
        if (lrc || util_launch_reduce(s->partials, nbE, 4, s->red, st)) return cuda_fail(s, cudaGetLastError(), "optimizer evaluation");
        s->launches += 4;
        double Ed = 0;
        int erc = s->sun ? ewald_add_sun<double>(s, grad, s->ewald_on ? &Ed : nullptr)
                         : ewald_add<double>(s, S, grad, s->ewald_on ? &Ed : nullptr);
        if (erc) return erc;
        if (dphi) {
            if (opt_launch_dphi(K, x, d, alpha, grad, kap, ns, part, st)) return cuda_fail(s, cudaGetLastError(), "optimizer launch");
            s->launches++;
        }
        CK(cudaMemcpyAsync(f, s->red, sizeof(double), cudaMemcpyDeviceToHost, st));
        if (dphi) {
            const bool mx[1] = {false};
            int prc = pull(1, dphi, mx);
            *f += Ed;
            return prc;
        }
        CK(cudaStreamSynchronize(st));
        *f += Ed;
        return SGB_OK;
    };
    const bool acc_max[10] = {false, false, false, false, false, false, false, true, true, false};
    auto accept = [&](double alpha, double* v) -> int {
        if (opt_launch_accept(K, x, d, alpha, grad, kap, ns, g, part, st)) return cuda_fail(s, cudaGetLastError(), "optimizer launch");
        s->launches++;
        return pull(10, v, acc_max);
    };
    const bool dir_max[2] = {false, true};
    auto direction = [&](double beta, double* v) -> int {
        if (opt_launch_dir(K, g, d, beta, ns, part, st)) return cuda_fail(s, cudaGetLastError(), "optimizer launch");
        s->launches++;
        return pull(2, v, dir_max);
    };
    double f = 0, v[10], w[2];
    if ((rc = eval(0.0, &f, nullptr)) || (rc = accept(0.0, v))) return rc;
    const double v9_0 = v[9] / (gdiv * gdiv);
    const double g_abstol = gdiv * 1e-12 * std::sqrt(v9_0) / std::sqrt((double)ns);   // characteristic_energy_scale, in the kernels' units
    const double x_abstol = 1e-12;
    bool conv = v[7] <= g_abstol;
    int iters = 0;
    if (!conv && (rc = direction(0.0, w))) return rc;
    double alpha_prev = 0, dphi_prev = 0, gmax = v[7];
    bool restarted = false;
    while (!conv && iters < maxiters) {
        const double phi0 = f, dphi0 = w[0];
        // strong Wolfe with σ = 0.1 (near-exact steps, which CG needs); sufficient decrease
        // is relaxed to the FP64 noise level of E once E no longer changes measurably
        const double eps = 1e-12 * std::fabs(phi0), sig = 0.1, del = 1e-4, amax = 10.0;
        auto wolfe = [&](double a, double fa, double da) {
            return std::fabs(da) <= -sig * dphi0 && (fa <= phi0 + del * a * dphi0 || fa <= phi0 + eps);
        };
        double a = alpha_prev == 0 ? 0.01 / gmax : alpha_prev * dphi_prev / dphi0;   // N&W (3.60)
        a = std::min(a, amax);
        double lo = 0, flo = phi0, dlo = dphi0, hi = -1, dhi = 0;
        double acc_a = -1, acc_f = 0;
        for (int k = 0; k < 60 && acc_a < 0; k++) {
            double fa, da;
            if ((rc = eval(a, &fa, &da))) return rc;
            if (!std::isfinite(fa) || !std::isfinite(da)) {
                hi = a; dhi = INFINITY;
            } else if (wolfe(a, fa, da)) {
                acc_a = a; acc_f = fa;
                break;
            } else if (da >= 0 || (fa > phi0 + eps && fa > phi0 + del * a * dphi0) || (hi < 0 && fa > flo + eps)) {
                hi = a; dhi = da;
            } else {
                lo = a; flo = fa; dlo = da;
            }
            if (hi < 0) {                       // still descending: expand (past the cap of the
                if (a * w[1] >= 10.0) break;     // initial guess, as Hager-Zhang does) until a
                a = 5.0 * a;                     // component would turn by 10 radians
                continue;
            }
            // next trial inside (lo, hi): secant on φ', else bisection
            const double wdt = hi - lo;
            if (std::fabs(wdt) <= 1e-15 * std::max(1.0, std::fabs(lo))) break;
            double t = 0.5 * (lo + hi);
            if (std::isfinite(dhi) && dhi > dlo) {
                const double sec = lo - dlo * (hi - lo) / (dhi - dlo);
                if (sec > lo + 0.05 * wdt && sec < hi - 0.05 * wdt) t = sec;
            }
            a = t;
        }
        if (acc_a < 0) {
            if (restarted) {
                // second failure in a row: no step decreases E at FP64 resolution, so x no
                // longer moves (Optim then reports x_abschange = 0 <= x_abstol). Accept that
                // as convergence only near a stationary point.
                conv = gmax <= gdiv * 1e-6 * std::sqrt(v9_0) / std::sqrt((double)ns);
                break;
            }
            restarted = true;
            if ((rc = eval(0.0, &f, nullptr)) || (rc = accept(0.0, v)) || (rc = direction(0.0, w))) return rc;
            gmax = v[7];
            alpha_prev = 0;
            continue;
        }
        restarted = false;
        if (acc_a != a) { double fa, da; if ((rc = eval(acc_a, &fa, &da))) return rc; }
        if ((rc = accept(acc_a, v))) return rc;
        iters++;
        f = acc_f;
        gmax = v[7];
        if (v[7] <= g_abstol || v[8] <= x_abstol) { conv = true; break; }
        // Hager-Zhang β with the η lower bound (vectors already transported)
        double beta = 0;
        if (v[0] != 0) {
            beta = (v[2] - 2.0 * v[1] * v[3] / v[0]) / v[0];
            const double eta = -1.0 / (std::sqrt(v[4]) * std::min(0.4, std::sqrt(v[5])));
            beta = std::max(beta, eta);
        }
        if ((rc = direction(beta, w))) return rc;
        if (!(w[0] < 0) && (rc = direction(0.0, w))) return rc;   // not a descent direction: restart
        alpha_prev = acc_a;
        dphi_prev = dphi0;
    }
    if (opt_launch_point(K, x, d, 0.0, kap, ns, S, st)) return cuda_fail(s, cudaGetLastError(), "optimizer launch");
    s->launches++;
    double E = f;
    if ((rc = eval(0.0, &E, nullptr))) return rc;
    CK(cudaStreamSynchronize(st));
    if (converged) *converged = conv ? 1 : 0;
    if (niters) *niters = iters;
    if (energy_out) *energy_out = E;
    return SGB_OK;
}

int sgb_local_colors(sgb_system* s, int32_t* ncolors, int32_t* color) {
    if (!s || !ncolors) return fail(s, SGB_ERR_ARG, "null argument");
    int rc = ensure_colors(s);
    if (rc) return rc;
    *ncolors = (int32_t)s->coff_h.size() - 1;
    if (color)
        for (int i = 0; i < s->ns; i++) color[i] = s->color_h[i];
    return SGB_OK;
}

int sgb_local_energy_change(sgb_system* s, int64_t site, const double* S_new, double* dE) {
    if (!s || !S_new || !dE) return fail(s, SGB_ERR_ARG, "null argument");
    if (site < 0 || site >= s->ns) return fail(s, SGB_ERR_ARG, "site out of range");
    int rc = ensure_colors(s);   // also rejects self-interaction
    if (rc) return rc;
    if (!s->state_set) return fail(s, SGB_ERR_STATE, "sgb_set_state must be called first");
    if ((rc = ensure_dbuf(s, 4))) return rc;
    if (s->sun) {
        SunKet zk{};
        for (int q = 0; q < 2 * s->N; q++) zk.v[q] = S_new[q];
        rc = s->fp32 ? sun_launch_local_dE<float>(s->mf, (const float*)s->Z, (const float*)s->S, (const float*)s->Q, (int)site, zk, s->dbuf, s->stream)
                     : sun_launch_local_dE<double>(s->md, (const double*)s->Z, (const double*)s->S, (const double*)s->Q, (int)site, zk, s->dbuf, s->stream);
    } else {
        rc = s->fp32 ? mc_launch_local_dE<float>(s->mf, (const float*)s->S, (int)site, S_new[0], S_new[1], S_new[2], s->dbuf, s->stream)
                     : mc_launch_local_dE<double>(s->md, (const double*)s->S, (int)site, S_new[0], S_new[1], S_new[2], s->dbuf, s->stream);
    }
    s->launches++;
    if (rc) return cuda_fail(s, cudaGetLastError(), "local energy launch");
    double out[2] = {0, 0};
    if (s->ewald_on) {
        // ewald_energy_delta (Ewald.jl:210-241) at the old dipoles, with ΔS the change of
        // the (expected) dipole
        double snew[3], sold[3];
        if (s->sun) host_expected_spin(s->N, S_new, snew);
        else for (int c = 0; c < 3; c++) snew[c] = S_new[c];
        for (int c = 0; c < 3; c++) {
            if (s->fp32) {
                float v;
                CK(cudaMemcpyAsync(&v, (const float*)s->S + (size_t)c * s->ns + site, sizeof(v), cudaMemcpyDeviceToHost, s->stream));
                CK(cudaStreamSynchronize(s->stream));
                sold[c] = v;
            } else {
                CK(cudaMemcpyAsync(&sold[c], (const double*)s->S + (size_t)c * s->ns + site, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
                CK(cudaStreamSynchronize(s->stream));
            }
        }
        const double dS[3] = {snew[0] - sold[0], snew[1] - sold[1], snew[2] - sold[2]};
        rc = s->fp32 ? ewald_launch_delta<float>(s->ew, (const float*)s->S, (int)site, dS, s->dbuf + 1, s->stream)
                     : ewald_launch_delta<double>(s->ew, (const double*)s->S, (int)site, dS, s->dbuf + 1, s->stream);
        s->launches++;
        if (rc) return cuda_fail(s, cudaGetLastError(), "dipole-dipole energy launch");
        CK(cudaMemcpyAsync(out, s->dbuf, 2 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    } else {
        CK(cudaMemcpyAsync(out, s->dbuf, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    }
    CK(cudaStreamSynchronize(s->stream));
    *dE = out[0] + out[1];
    return SGB_OK;
}

int sgb_event_record(sgb_system* s, int32_t slot) {
    if (!s || slot < 0 || slot >= 8) return fail(s, SGB_ERR_ARG, "bad event slot");
    CK(cudaEventRecord(s->ev[slot], s->stream));
    return SGB_OK;
}

int sgb_event_elapsed(sgb_system* s, int32_t a, int32_t b, float* ms) {
    if (!s || !ms || a < 0 || a >= 8 || b < 0 || b >= 8) return fail(s, SGB_ERR_ARG, "bad event slot");
    CK(cudaEventSynchronize(s->ev[b]));
    CK(cudaEventElapsedTime(ms, s->ev[a], s->ev[b]));
    return SGB_OK;
}

int sgb_set_wait_limit(sgb_system* s, double seconds) {
    if (!s) return fail(s, SGB_ERR_ARG, "null handle");
    if (!(seconds >= 0) || seconds > 3600) return fail(s, SGB_ERR_ARG, "wait limit must be in [0, 3600] s (0: the 4 s default)");
    const unsigned long long ns = (unsigned long long)(seconds * 1e9);
    CK(cudaMemcpyAsync(&s->ctrl->wait_ns, &ns, sizeof(ns), cudaMemcpyHostToDevice, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return SGB_OK;
}

int sgb_wait_probe(sgb_system* s) {
    if (!s) return fail(s, SGB_ERR_ARG, "null handle");
    int rc = reset_ctrl(s);
    if (rc) return rc;
    if (util_launch_wait_probe(s->ctrl, 2, s->stream)) return cuda_fail(s, cudaGetLastError(), "wait probe launch");
    s->launches++;
    Ctrl c;
    if ((rc = read_ctrl(s, &c))) return rc;
    if (c.status == SGB_ERR_TIMEOUT) return fail(s, SGB_ERR_TIMEOUT, "a device-side barrier timed out");
    if (c.status) return fail(s, c.status, "the wait probe ended with an unexpected status");
    return fail(s, SGB_ERR_STATE, "the wait probe's barrier completed, which it cannot");
}

int sgb_synchronize(sgb_system* s) {
    if (!s) return fail(s, SGB_ERR_ARG, "null handle");
    CK(cudaStreamSynchronize(s->stream));
    return SGB_OK;
}

int64_t sgb_kernel_launches(const sgb_system* s) { return s ? s->launches : 0; }

int sgb_flush_l2(sgb_system* s) {
    if (!s) return fail(s, SGB_ERR_ARG, "null handle");
    const size_t bytes = (size_t)256 << 20;
    if (!s->flush) {
        int rc = dmalloc(s, &s->flush, bytes);
        if (rc) return rc;
    }
    CK(cudaMemsetAsync(s->flush, s->launches & 0xff, bytes, s->stream));
    return SGB_OK;
}

// ---------------------------------------------------------------------------------
// SampledCorrelations
// ---------------------------------------------------------------------------------
static int cfail(sgb_corr* c, int code, const std::string& msg) {
    if (c) { c->err = msg; if (c->sys) c->sys->err = msg; if (c->batch) c->batch->err = msg; }
    g_last_error = msg;
    return code;
}

void sgb_corr_destroy(sgb_corr* c) {
    if (!c) return;
    if (c->stream) cudaStreamSynchronize(c->stream);
    auto unlink = [c](std::vector<sgb_corr*>& v) { v.erase(std::remove(v.begin(), v.end(), c), v.end()); };
    if (c->sys) unlink(c->sys->corrs);
    if (c->batch) unlink(c->batch->corrs);
    dfree(c->ops);
    void* p = c->pairs; dfree(p);
    dfree(c->A); dfree(c->Ahat);
    dfree(c->td_chirp); dfree(c->td_fb); dfree(c->td_tw);
    p = c->P; dfree(p);
    p = c->g; dfree(p);
    if (c->have_space) cufftDestroy(c->plan_space);
    if (c->have_time) cufftDestroy(c->plan_time);
    if (c->have_chunk) cufftDestroy(c->plan_chunk);
    p = c->M; dfree(p);
    p = c->ctmp; dfree(p);
    p = c->err_d; dfree(p);
    for (int i = 0; i < 5; i++) if (c->ev[i]) cudaEventDestroy(c->ev[i]);
    delete c;
}

// Shared set-up of an accumulator for `nrep` identical systems of `ns` sites.
static int corr_setup(sgb_corr* c, const sgb_corr_desc* d, bool fp32, bool sun, int N, int ns, int natoms,
                      const int* dims, int nrep) {
    const size_t R = fp32 ? 4 : 8;
    c->nobs = d->nobs; c->ncorr = d->ncorr; c->npos = natoms; c->ncell = dims[0] * dims[1] * dims[2];
    c->nomega = d->n_all_omega;
    c->nsnaps = d->n_all_omega / 2 + 1;   // CorrelationSampling.jl:37-38
    c->measperiod = d->measperiod;
    c->dt = d->dt; c->damping = d->damping; c->tol = d->tol; c->max_iters = d->max_iters;
    c->nrep = nrep;
    // observables, device layout dipole [nobs][3][ns], SU(N) [nobs][N*N][2][ns]
    size_t per = sun ? (size_t)2 * N * N : 3;
    std::vector<char> host(R * per * d->nobs * ns);
    for (int o = 0; o < d->nobs; o++)
        for (int i = 0; i < ns; i++)
            for (size_t k = 0; k < per; k++) {
                double v = d->obs[((size_t)o * ns + i) * per + k];
                size_t idx = ((size_t)o * per + k) * ns + i;
                if (fp32) reinterpret_cast<float*>(host.data())[idx] = (float)v;
                else reinterpret_cast<double*>(host.data())[idx] = v;
            }
    auto alloc = [&](void** p, size_t bytes) -> int {
        if (cudaMalloc(p, bytes ? bytes : 16) != cudaSuccess) { *p = nullptr; return cfail(c, SGB_ERR_NOMEM, "device allocation failed"); }
        return SGB_OK;
    };
    int rc;
    if ((rc = alloc(&c->ops, host.size()))) return rc;
    if (cudaMemcpy(c->ops, host.data(), host.size(), cudaMemcpyHostToDevice) != cudaSuccess) return cfail(c, SGB_ERR_CUDA, "copy observables");
    if ((rc = alloc((void**)&c->pairs, sizeof(int) * 2 * d->ncorr))) return rc;
    cudaMemcpy(c->pairs, d->pairs, sizeof(int) * 2 * d->ncorr, cudaMemcpyHostToDevice);
    size_t nA = (size_t)nrep * c->nomega * c->nobs * c->npos * c->ncell;  // complex elements
    if ((rc = alloc(&c->A, 2 * R * nA))) return rc;
    if ((rc = alloc(&c->Ahat, 2 * R * nA))) return rc;
    cudaMemset(c->A, 0, 2 * R * nA);
    c->plen = (size_t)c->nomega * c->ncell * c->npos * c->npos * c->ncorr;
    if ((rc = alloc((void**)&c->P, 16 * c->plen))) return rc;
    cudaMemset(c->P, 0, 16 * c->plen);
    if ((rc = alloc((void**)&c->g, sizeof(double) * c->nomega))) return rc;
    if ((rc = alloc((void**)&c->err_d, sizeof(int)))) return rc;
    cudaMemset(c->err_d, 0, sizeof(int));
    if (d->calculate_errors) {
        c->welford = true;
        if ((rc = alloc((void**)&c->M, 8 * c->plen))) return rc;
        cudaMemset(c->M, 0, 8 * c->plen);
    }
    // cuFFT plans: space FFT over (L3, L2, L1) for every snapshot row; time FFT along ω
    const cufftType ty = fp32 ? CUFFT_C2C : CUFFT_Z2Z;
    int n3[3] = {dims[2], dims[1], dims[0]};
    int batch_space = c->nsnaps * c->nobs * c->npos;
    if (cufftPlanMany(&c->plan_space, 3, n3, nullptr, 1, c->ncell, nullptr, 1, c->ncell, ty, batch_space) != CUFFT_SUCCESS)
        return cfail(c, SGB_ERR_CUDA, "cufftPlanMany (space) failed");
    c->have_space = true;
    cufftSetStream(c->plan_space, c->stream);
    if (c->nomega > 1) {
        int n1[1] = {c->nomega};
        int stride = c->nobs * c->npos * c->ncell;
        if (cufftPlanMany(&c->plan_time, 1, n1, n1, stride, 1, n1, stride, 1, ty, stride) != CUFFT_SUCCESS)
            return cfail(c, SGB_ERR_CUDA, "cufftPlanMany (time) failed");
        c->have_time = true;
        cufftSetStream(c->plan_time, c->stream);
        if (fp32 && tdft_supported(c->nomega, c->nsnaps)) {
            int trc = tdft_tables(c->nomega, c->nsnaps, &c->td_chirp, &c->td_fb, &c->td_tw);
            if (trc) return cfail(c, trc, "time transform tables");
        }
    }
    return SGB_OK;
}

static int corr_check_desc(const sgb_corr_desc* d) {
    if (d->nobs < 1 || d->ncorr < 1 || !d->obs || !d->pairs) return fail(nullptr, SGB_ERR_ARG, "observables and correlation pairs are required");
    if (d->n_all_omega < 1 || d->measperiod < 1) return fail(nullptr, SGB_ERR_ARG, "n_all_omega and measperiod must be positive");
    if (d->n_all_omega > 1 && !(d->dt > 0)) return fail(nullptr, SGB_ERR_ARG, "Select positive dt");
    for (int k = 0; k < 2 * d->ncorr; k++)
        if (d->pairs[k] < 0 || d->pairs[k] >= d->nobs) return fail(nullptr, SGB_ERR_ARG, "correlation pair index out of range");
    return SGB_OK;
}

int sgb_corr_create(sgb_system* s, const sgb_corr_desc* d, sgb_corr** out) {
    if (!s || !d || !out) return fail(s, SGB_ERR_ARG, "null argument");
    *out = nullptr;
    int rc = corr_check_desc(d);
    if (rc) { s->err = g_last_error; return rc; }
    if ((rc = ensure_tables(s))) return rc;
    sgb_corr* c = new sgb_corr();
    c->sys = s;
    c->stream = s->stream;
    c->launches = &s->launches;
    rc = corr_setup(c, d, s->fp32, s->sun, s->N, s->ns, s->d.natoms, s->d.dims, 1);
    if (rc) { sgb_corr_destroy(c); return rc; }
    s->corrs.push_back(c);
    *out = c;
    return SGB_OK;
}

int sgb_batch_corr_create(sgb_batch* b, const sgb_corr_desc* d, sgb_corr** out) {
    if (!b || !d || !out) return fail(nullptr, SGB_ERR_ARG, "null argument");
    *out = nullptr;
    int rc = corr_check_desc(d);
    if (rc) { b->err = g_last_error; return rc; }
    for (int r = 1; r < b->nrep; r++)
        for (int k = 0; k < 3; k++)
            if (b->dims[3 * r + k] != b->dims[k]) { b->err = "batched sampling needs replicas of equal size"; return SGB_ERR_ARG; }
    if (!b->coup_set) { b->err = "couplings must be set first"; return SGB_ERR_STATE; }
    if (!b->grp.empty()) {
        sgb_system* s0 = b->grp[0];
        if ((rc = ensure_tables(s0))) { b->err = s0->err; return rc; }
        sgb_corr* c = new sgb_corr();
        c->batch = b;
        c->stream = b->stream;
        c->launches = &b->launches;
        rc = corr_setup(c, d, b->fp32, s0->sun, s0->N, s0->ns, b->na, b->dims.data(), b->nrep);
        if (rc) { b->err = c->err; sgb_corr_destroy(c); return rc; }
        b->corrs.push_back(c);
        *out = c;
        return SGB_OK;
    }
    const size_t R = b->fp32 ? 4 : 8;
    auto lazy = [&](void** p, size_t bytes) -> int {
        if (*p) return SGB_OK;
        if (cudaMalloc(p, bytes) != cudaSuccess) { *p = nullptr; b->err = "device allocation failed"; return SGB_ERR_NOMEM; }
        return SGB_OK;
    };
    // midpoint buffers: three rotating neighbour-gathered buffers of one 4-element vector
    // per site (FP32 float4 layout), and the private 3-vector buffers [3][NS]
    if ((rc = lazy(&b->Sp, R * 3 * b->NS)) || (rc = lazy(&b->H, R * 12 * b->NS)) ||
        (rc = lazy(&b->P1, R * 3 * b->NS)) || (rc = lazy(&b->H1, R * 3 * b->NS)) ||
        (rc = lazy(&b->H2, R * 3 * b->NS)) || (rc = lazy(&b->H3, R * 3 * b->NS)) ||
        (rc = lazy((void**)&b->racc, sizeof(double) * 3 * b->nrep)))
        return rc;
    sgb_corr* c = new sgb_corr();
    c->batch = b;
    c->stream = b->stream;
    c->launches = &b->launches;
    const int ns = b->off[1] - b->off[0];
    rc = corr_setup(c, d, b->fp32, false, 0, ns, b->na, b->dims.data(), b->nrep);
    if (rc) { b->err = c->err; sgb_corr_destroy(c); return rc; }
    b->corrs.push_back(c);
    *out = c;
    return SGB_OK;
}

// window(t)/n_contrib(t)/n for the read-out transform (CorrelationSampling.jl:52-107)
static void window_weights(int n, int window, std::vector<double>& g) {
    g.assign(n, 0.0);
    int T = n / 2 + 1;
    for (int k = 0; k < n; k++) {
        // FFTW.fftfreq(n, n): 0..ceil(n/2)-1 then negative
        int dtk = (k < (n + 1) / 2) ? k : k - n;
        int contrib = T - std::abs(dtk);
        double w = 1.0;
        if (window == 0) {
            double c = std::cos(M_PI * k / n);
            w = c * c;
        }
        g[k] = contrib <= 0 ? 0.0 : w / contrib / n;
    }
}

// calculate_errors path of add_sample!: for every replica's sample, in order, form the
// products column chunk by column chunk, apply IFFT -> window/n_contrib/n -> FFT
// (CorrelationSampling.jl:71-109) and update the running mean and M (:117-134).
static int welford_samples(sgb_corr* c, const void* spec, bool fp32, size_t rep_stride) {
    const int n = c->nomega;
    const size_t ld = c->plen / n;
    if (!c->ctmp) {
        size_t chunk = std::max<size_t>(1, ((size_t)64 << 20) / ((size_t)16 * n));
        c->chunk = std::min(chunk, ld);
        if (cudaMalloc((void**)&c->ctmp, 16 * c->chunk * n) != cudaSuccess) {
            c->ctmp = nullptr;
            return cfail(c, SGB_ERR_NOMEM, "device allocation failed");
        }
        if (n > 1) {
            int n1[1] = {n};
            if (cufftPlanMany(&c->plan_chunk, 1, n1, nullptr, 1, n, nullptr, 1, n, CUFFT_Z2Z, (int)c->chunk) != CUFFT_SUCCESS)
                return cfail(c, SGB_ERR_CUDA, "cufftPlanMany (per-sample transform) failed");
            c->have_chunk = true;
        }
    }
    if (c->have_chunk) cufftSetStream(c->plan_chunk, c->stream);
    const size_t esz = fp32 ? 8 : 16;
    for (int r = 0; r < c->nrep; r++) {
        const void* Ar = (const char*)spec + esz * rep_stride * r;
        const double count = (double)(c->nsamples + r + 1);
        for (size_t col0 = 0; col0 < ld; col0 += c->chunk) {
            const int ncol = (int)std::min(c->chunk, ld - col0);
            int rc = fp32 ? corr_launch_product<float>((const float*)Ar, c->pairs, c->ncorr, c->nobs, c->npos, c->ncell, n,
                                                       col0, ncol, c->ctmp, c->stream)
                          : corr_launch_product<double>((const double*)Ar, c->pairs, c->ncorr, c->nobs, c->npos, c->ncell, n,
                                                        col0, ncol, c->ctmp, c->stream);
            if (rc) return cfail(c, SGB_ERR_CUDA, "product launch");
            if (c->have_chunk &&
                cufftExecZ2Z(c->plan_chunk, (cufftDoubleComplex*)c->ctmp, (cufftDoubleComplex*)c->ctmp, CUFFT_INVERSE) != CUFFT_SUCCESS)
                return cfail(c, SGB_ERR_CUDA, "per-sample transform failed");
            if (corr_launch_window(c->ctmp, ncol, n, c->g, c->stream)) return cfail(c, SGB_ERR_CUDA, "window launch");
            if (c->have_chunk &&
                cufftExecZ2Z(c->plan_chunk, (cufftDoubleComplex*)c->ctmp, (cufftDoubleComplex*)c->ctmp, CUFFT_FORWARD) != CUFFT_SUCCESS)
                return cfail(c, SGB_ERR_CUDA, "per-sample transform failed");
            if (corr_launch_welford(c->ctmp, ncol, n, col0, ld, count, c->P, c->M, c->stream))
                return cfail(c, SGB_ERR_CUDA, "Welford launch");
            (*c->launches) += 3;
        }
    }
    return SGB_OK;
}

int sgb_corr_add_sample(sgb_corr* c, int32_t window) {
    if (!c) return fail(nullptr, SGB_ERR_ARG, "null handle");
    sgb_system* s = c->sys;
    sgb_batch* b = c->batch;
    if (!s && !b) return cfail(c, SGB_ERR_STATE, "the System (or replica batch) of this accumulator was destroyed");
    if (window != 0 && window != 1) return cfail(c, SGB_ERR_ARG, "window must be 0 (:cosine) or 1 (:rectangular)");
    if (c->window >= 0 && c->window != window)
        return cfail(c, SGB_ERR_ARG, "all samples of one accumulator must use the same window");
    int rc = SGB_OK;
    if (s) {
        if (!s->state_set) return cfail(c, SGB_ERR_STATE, "sgb_set_state must be called before add_sample");
        if ((rc = ensure_tables(s))) return rc;
    } else if (!b->state_set) {
        return cfail(c, SGB_ERR_STATE, "replica states must be set before add_sample");
    }
    const bool fp32 = s ? s->fp32 : b->fp32;
    if (c->window < 0) {
        std::vector<double> g;
        window_weights(c->nomega, window, g);
        if (cudaMemcpy(c->g, g.data(), sizeof(double) * c->nomega, cudaMemcpyHostToDevice) != cudaSuccess)
            return cfail(c, SGB_ERR_CUDA, "copy window");
        c->window = window;
    }
    const int nsteps = c->measperiod * (c->nsnaps - 1);
    const double scale = 1.0 / std::sqrt((double)c->ncell);
    if (c->profile) cudaEventRecord(c->ev[0], c->stream);
    int64_t iters = 0;
    // 1. trajectory with fused observable snapshots (CorrelationSampling.jl:21-46)
    if (b) {
        rc = batch_corr_trajectory(c);
        iters = c->prof_iters_last;
        if (rc) return cfail(c, rc, batch_error(b));
    } else if (fp32) {
        SnapArgs<float> sn{1, c->nobs, c->measperiod, 0, (const float*)c->ops, (float*)c->A, (float)scale};
        if (s->ewald_on && s->sun) rc = run_midpoint_lr_sun<float>(s, c->dt, c->damping, c->tol, c->max_iters, nsteps, &iters, &sn);
        else if (s->ewald_on) rc = run_midpoint_lr<float>(s, c->dt, c->damping, c->tol, c->max_iters, nsteps, &iters, &sn);
        else if (nsteps > 0) rc = run_midpoint<float>(s, c->dt, c->damping, c->tol, c->max_iters, nsteps, &iters, sn, true, s->mid_order);
        else rc = run_midpoint<float>(s, 1.0, 0.0, 1e300, 1, 0, nullptr, sn, true);
    } else {
        SnapArgs<double> sn{1, c->nobs, c->measperiod, 0, (const double*)c->ops, (double*)c->A, scale};
        if (s->ewald_on && s->sun) rc = run_midpoint_lr_sun<double>(s, c->dt, c->damping, c->tol, c->max_iters, nsteps, &iters, &sn);
        else if (s->ewald_on) rc = run_midpoint_lr<double>(s, c->dt, c->damping, c->tol, c->max_iters, nsteps, &iters, &sn);
        else if (nsteps > 0) rc = run_midpoint<double>(s, c->dt, c->damping, c->tol, c->max_iters, nsteps, &iters, sn, true, s->mid_order);
        else rc = run_midpoint<double>(s, 1.0, 0.0, 1e300, 1, 0, nullptr, sn, true);
    }
    if (rc) return rc;
    if (c->profile) cudaEventRecord(c->ev[1], c->stream);
    const size_t rep_stride = (size_t)c->nomega * c->nobs * c->npos * c->ncell;  // complex elements
    const size_t esz = fp32 ? 8 : 16;                                              // bytes per complex
    // 2. space FFT, A(q) = sum_r exp(+iqr) A(r) / sqrt(Ncell) (CorrelationSampling.jl:58-63)
    for (int r = 0; r < c->nrep; r++) {
        void* Ar = (char*)c->A + esz * rep_stride * r;
        cufftResult fr = fp32 ? cufftExecC2C(c->plan_space, (cufftComplex*)Ar, (cufftComplex*)Ar, CUFFT_INVERSE)
                              : cufftExecZ2Z(c->plan_space, (cufftDoubleComplex*)Ar, (cufftDoubleComplex*)Ar, CUFFT_INVERSE);
        if (fr != CUFFT_SUCCESS) return cfail(c, SGB_ERR_CUDA, "space FFT failed");
    }
    if (c->profile) cudaEventRecord(c->ev[2], c->stream);
    // 3. time FFT, A(ω) = sum_t exp(-iωt) A(t), zero padded (CorrelationSampling.jl:65-69)
    const void* spec = c->A;
    if (c->have_time) {
        const long long stride = (long long)c->nobs * c->npos * c->ncell;
        if (fp32 && c->td_fb && c->time_kind == 0) {
            // every replica's series in one launch of the hand-written transform
            if (tdft_launch((const float*)c->A, (float*)c->Ahat, stride * c->nrep, stride, (long long)rep_stride, c->nomega, c->nsnaps,
                            c->td_chirp, c->td_fb, c->td_tw, c->stream))
                return cfail(c, SGB_ERR_CUDA, std::string("time transform launch: ") + cudaGetErrorString(cudaGetLastError()));
            (*c->launches)++;
        } else {
            for (int r = 0; r < c->nrep; r++) {
                void* Ar = (char*)c->A + esz * rep_stride * r;
                void* Hr = (char*)c->Ahat + esz * rep_stride * r;
                cufftResult fr = fp32 ? cufftExecC2C(c->plan_time, (cufftComplex*)Ar, (cufftComplex*)Hr, CUFFT_FORWARD)
                                      : cufftExecZ2Z(c->plan_time, (cufftDoubleComplex*)Ar, (cufftDoubleComplex*)Hr, CUFFT_FORWARD);
                if (fr != CUFFT_SUCCESS) return cfail(c, SGB_ERR_CUDA, "time FFT failed");
            }
        }
        spec = c->Ahat;
    }
    if (c->profile) cudaEventRecord(c->ev[3], c->stream);
    // 4. accumulate sum_r conj(A_alpha,i) A_beta,j into the FP64 sum, or (calculate_errors)
    //    transform every sample and fold it into the running mean and M
    if (c->welford) {
        if ((rc = welford_samples(c, spec, fp32, rep_stride))) return rc;
    } else {
        rc = fp32 ? corr_launch_accum<float>((const float*)spec, c->P, c->pairs, c->ncorr, c->nobs, c->npos, c->ncell,
                                             c->nomega, c->nrep, rep_stride, c->stream, c->accum_variant, c->err_d)
                  : corr_launch_accum<double>((const double*)spec, c->P, c->pairs, c->ncorr, c->nobs, c->npos, c->ncell,
                                              c->nomega, c->nrep, rep_stride, c->stream, c->accum_variant, c->err_d);
        (*c->launches)++;
        if (rc) return cfail(c, SGB_ERR_CUDA, std::string("accumulate launch: ") + cudaGetErrorString(cudaGetLastError()));
    }
    c->nsamples += c->nrep;
    if (c->profile) {
        cudaEventRecord(c->ev[4], c->stream);
        if (cudaEventSynchronize(c->ev[4]) != cudaSuccess) return cfail(c, SGB_ERR_CUDA, "profiling event failed");
        for (int k = 0; k < 4; k++) {
            float ms = 0;
            cudaEventElapsedTime(&ms, c->ev[k], c->ev[k + 1]);
            c->phase_ms[k] += ms;
        }
        c->nprof += 1;
        c->prof_iters += iters;
    }
    return SGB_OK;
}

int sgb_corr_profile(sgb_corr* c, int32_t enable) {
    if (!c) return fail(nullptr, SGB_ERR_ARG, "null handle");
    if (enable && !c->ev[0])
        for (int i = 0; i < 5; i++)
            if (cudaEventCreate(&c->ev[i]) != cudaSuccess) return cfail(c, SGB_ERR_CUDA, "cudaEventCreate failed");
    c->profile = enable != 0;
    for (int k = 0; k < 4; k++) c->phase_ms[k] = 0;
    c->nprof = 0;
    c->prof_iters = 0;
    return SGB_OK;
}

int sgb_corr_phase_times(sgb_corr* c, double* ms4, int64_t* n, int64_t* iters) {
    if (!c || !ms4) return fail(nullptr, SGB_ERR_ARG, "null argument");
    for (int k = 0; k < 4; k++) ms4[k] = c->phase_ms[k];
    if (n) *n = c->nprof;
    if (iters) *iters = c->prof_iters;
    return SGB_OK;
}

int sgb_corr_data(sgb_corr* c, double* data, double* M, int64_t* nsamples) {
    if (!c) return fail(nullptr, SGB_ERR_ARG, "null handle");
    cudaStream_t stream = c->stream;
    if (nsamples) *nsamples = c->nsamples;
    if (M && !c->welford) return cfail(c, SGB_ERR_ARG, "M is kept only with calculate_errors");
    {
        int flag = 0;
        if (cudaMemcpyAsync(&flag, c->err_d, sizeof(int), cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
            cudaStreamSynchronize(stream) != cudaSuccess)
            return cfail(c, SGB_ERR_CUDA, "reading the accumulation status failed");
        if (flag) return cfail(c, SGB_ERR_TIMEOUT, "a bounded wait of the accumulation kernel gave up; the data are incomplete");
    }
    if (c->welford) {
        // running mean and M are kept transformed, in Sunny's layout
        cudaError_t e = cudaSuccess;
        if (data) e = cudaMemcpyAsync(data, c->P, 16 * c->plen, cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess && M) e = cudaMemcpyAsync(M, c->M, 8 * c->plen, cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess) return cfail(c, SGB_ERR_CUDA, std::string("copy data: ") + cudaGetErrorString(e));
        return SGB_OK;
    }
    if (!data) return SGB_OK;
    const int n = c->nomega;
    const size_t ld = c->plen / n;  // columns
    if (c->nsamples == 0) {
        std::memset(data, 0, 16 * c->plen);
        return SGB_OK;
    }
    const double inv = 1.0 / (double)c->nsamples;
    if (n == 1) {
        // static: data = P / nsamples (window weight 1 at Δt = 0)
        std::vector<double> tmp(2 * c->plen);
        if (cudaMemcpy(tmp.data(), c->P, 16 * c->plen, cudaMemcpyDeviceToHost) != cudaSuccess) return cfail(c, SGB_ERR_CUDA, "copy data");
        for (size_t k = 0; k < 2 * c->plen; k++) data[k] = tmp[k] * inv;
        return SGB_OK;
    }
    // chunked read-out transform: IFFT_ω -> × window/n_contrib/n -> FFT_ω
    size_t chunk = std::max<size_t>(1, ((size_t)64 << 20) / ((size_t)16 * n));
    chunk = std::min(chunk, ld);
    double *tmp = nullptr, *outb = nullptr;
    if (cudaMalloc((void**)&tmp, 16 * chunk * n) != cudaSuccess) return cfail(c, SGB_ERR_NOMEM, "device allocation failed");
    if (cudaMalloc((void**)&outb, 16 * chunk * n) != cudaSuccess) { cudaFree(tmp); return cfail(c, SGB_ERR_NOMEM, "device allocation failed"); }
    cufftHandle plan;
    int n1[1] = {n};
    if (cufftPlanMany(&plan, 1, n1, nullptr, 1, n, nullptr, 1, n, CUFFT_Z2Z, (int)chunk) != CUFFT_SUCCESS) {
        cudaFree(tmp); cudaFree(outb);
        return cfail(c, SGB_ERR_CUDA, "cufftPlanMany (read-out) failed");
    }
    cufftSetStream(plan, stream);
    int status = SGB_OK;
    for (size_t col0 = 0; col0 < ld && status == SGB_OK; col0 += chunk) {
        int ncol = (int)std::min(chunk, ld - col0);
        if (corr_launch_gather(c->P, ld, col0, ncol, n, inv, tmp, stream)) { status = SGB_ERR_CUDA; break; }
        if (cufftExecZ2Z(plan, (cufftDoubleComplex*)tmp, (cufftDoubleComplex*)tmp, CUFFT_INVERSE) != CUFFT_SUCCESS) { status = SGB_ERR_CUDA; break; }
        if (corr_launch_window(tmp, ncol, n, c->g, stream)) { status = SGB_ERR_CUDA; break; }
        if (cufftExecZ2Z(plan, (cufftDoubleComplex*)tmp, (cufftDoubleComplex*)tmp, CUFFT_FORWARD) != CUFFT_SUCCESS) { status = SGB_ERR_CUDA; break; }
        if (corr_launch_scatter(tmp, ncol, n, outb, stream)) { status = SGB_ERR_CUDA; break; }
        (*c->launches) += 3;
        if (cudaMemcpy2DAsync(data + 2 * col0, 16 * ld, outb, 16 * (size_t)ncol, 16 * (size_t)ncol, n, cudaMemcpyDeviceToHost,
                              stream) != cudaSuccess) { status = SGB_ERR_CUDA; break; }
    }
    cudaStreamSynchronize(stream);
    cufftDestroy(plan);
    cudaFree(tmp);
    cudaFree(outb);
    if (status != SGB_OK) return cfail(c, status, "read-out transform failed");
    return SGB_OK;
}

int sgb_corr_intensities(sgb_corr* c, int32_t nq, const int32_t* qidx, const double* pref, const double* qcart,
                         int32_t nw, const int32_t* widx, int32_t combiner, double* out) {
    if (!c || nq < 0 || nw < 1 || (nq > 0 && (!qidx || !pref || !out)) || !widx) return cfail(c, SGB_ERR_ARG, "invalid arguments");
    if (combiner < 0 || combiner > 2) return cfail(c, SGB_ERR_ARG, "combiner must be 0 (trace), 1 (perp) or 2 (raw)");
    if (combiner == 1 && !qcart) return cfail(c, SGB_ERR_ARG, "the perpendicular combiner needs the absolute wave vectors");
    if (combiner < 2 && c->ncorr != 6) return cfail(c, SGB_ERR_ARG, "trace and perp combiners need the six ssf correlation pairs");
    if (c->ncorr > 8) return cfail(c, SGB_ERR_ARG, "at most 8 correlation pairs");
    const int n = c->nomega;
    for (int t = 0; t < nw; t++)
        if (widx[t] < 0 || widx[t] >= n) return cfail(c, SGB_ERR_ARG, "energy index out of range");
    for (int k = 0; k < nq; k++)
        if (qidx[k] < 0 || qidx[k] >= c->ncell) return cfail(c, SGB_ERR_ARG, "wave vector index out of range");
    const size_t per_out = combiner == 2 ? (size_t)2 * c->ncorr : 1;
    if (nq == 0) return SGB_OK;
    if (c->nsamples == 0) {
        std::memset(out, 0, sizeof(double) * per_out * nw * nq);
        return SGB_OK;
    }
    cudaStream_t st = c->stream;
    const int B = c->ncorr * c->npos * c->npos;
    const size_t ld = c->plen / n;
    const size_t per_q = (size_t)B * n * 16;
    const int qc = (int)std::max<size_t>(1, std::min<size_t>((size_t)nq, ((size_t)256 << 20) / per_q));
    double *tmp = nullptr, *pref_d = nullptr, *qcart_d = nullptr, *out_d = nullptr;
    int *qidx_d = nullptr, *widx_d = nullptr;
    int status = SGB_OK;
    std::string what;
    auto al = [&](void** p, size_t bytes) { if (status == SGB_OK && cudaMalloc(p, bytes) != cudaSuccess) { *p = nullptr; status = SGB_ERR_NOMEM; what = "device allocation failed"; } };
    al((void**)&tmp, per_q * qc);
    al((void**)&pref_d, 16 * (size_t)c->npos * qc);
    al((void**)&qcart_d, 24 * (size_t)qc);
    al((void**)&out_d, sizeof(double) * per_out * nw * qc);
    al((void**)&qidx_d, sizeof(int) * qc);
    al((void**)&widx_d, sizeof(int) * nw);
    cufftHandle plan = 0;
    int plan_batch = 0;
    const bool transform = !c->welford && n > 1;
    if (status == SGB_OK && cudaMemcpyAsync(widx_d, widx, sizeof(int) * nw, cudaMemcpyHostToDevice, st) != cudaSuccess) {
        status = SGB_ERR_CUDA; what = "copy energy indices";
    }
    for (int q0 = 0; q0 < nq && status == SGB_OK; q0 += qc) {
        const int m = std::min(qc, nq - q0);
        if (transform && plan_batch != m * B) {
            if (plan) cufftDestroy(plan);
            plan = 0;
            int n1[1] = {n};
            if (cufftPlanMany(&plan, 1, n1, nullptr, 1, n, nullptr, 1, n, CUFFT_Z2Z, m * B) != CUFFT_SUCCESS) {
                status = SGB_ERR_CUDA; what = "cufftPlanMany (intensities) failed"; break;
            }
            cufftSetStream(plan, st);
            plan_batch = m * B;
        }
        if (cudaMemcpyAsync(qidx_d, qidx + q0, sizeof(int) * m, cudaMemcpyHostToDevice, st) != cudaSuccess ||
            cudaMemcpyAsync(pref_d, pref + (size_t)2 * c->npos * q0, 16 * (size_t)c->npos * m, cudaMemcpyHostToDevice, st) != cudaSuccess ||
            (qcart && cudaMemcpyAsync(qcart_d, qcart + 3 * (size_t)q0, 24 * (size_t)m, cudaMemcpyHostToDevice, st) != cudaSuccess)) {
            status = SGB_ERR_CUDA; what = "copy wave vectors"; break;
        }
        const double scale = c->welford ? 1.0 : 1.0 / (double)c->nsamples;
        if (corr_launch_gather_q(c->P, ld, qidx_d, m, B, n, scale, tmp, st)) { status = SGB_ERR_CUDA; what = "gather launch"; break; }
        if (transform) {
            if (cufftExecZ2Z(plan, (cufftDoubleComplex*)tmp, (cufftDoubleComplex*)tmp, CUFFT_INVERSE) != CUFFT_SUCCESS ||
                corr_launch_window(tmp, m * B, n, c->g, st) ||
                cufftExecZ2Z(plan, (cufftDoubleComplex*)tmp, (cufftDoubleComplex*)tmp, CUFFT_FORWARD) != CUFFT_SUCCESS) {
                status = SGB_ERR_CUDA; what = "read-out transform failed"; break;
            }
        }
        if (corr_launch_intensity(tmp, c->ncorr, c->npos, n, pref_d, qcart ? qcart_d : nullptr, widx_d, nw, combiner, m,
                                  out_d, st)) {
            status = SGB_ERR_CUDA; what = "intensity launch"; break;
        }
        (*c->launches) += transform ? 3 : 2;
        if (cudaMemcpyAsync(out + per_out * nw * (size_t)q0, out_d, sizeof(double) * per_out * nw * m, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess) {
            status = SGB_ERR_CUDA; what = "copy intensities"; break;
        }
    }
    cudaStreamSynchronize(st);
    if (plan) cufftDestroy(plan);
    void* bufs[] = {tmp, pref_d, qcart_d, out_d, qidx_d, widx_d};
    for (void* p : bufs) if (p) cudaFree(p);
    if (status != SGB_OK) return cfail(c, status, std::string("intensities: ") + what);
    return SGB_OK;
}

int sgb_corr_merge(sgb_corr* dst, const sgb_corr* src) {
    if (!dst || !src) return fail(nullptr, SGB_ERR_ARG, "null handle");
    if (dst->plen != src->plen || dst->nomega != src->nomega || dst->ncorr != src->ncorr)
        return cfail(dst, SGB_ERR_ARG, "accumulators have different shapes");
    if (src->nsamples > 0 && dst->window >= 0 && src->window >= 0 && dst->window != src->window)
        return cfail(dst, SGB_ERR_ARG, "accumulators used different windows");
    if (dst->welford != src->welford)
        return cfail(dst, SGB_ERR_ARG, "accumulators with and without calculate_errors cannot be merged");
    if (src->stream != dst->stream) cudaStreamSynchronize(src->stream);
    if (dst->welford) {
        if (src->nsamples > 0 &&
            corr_launch_merge_welford(dst->P, dst->M, src->P, src->M, (double)dst->nsamples, (double)src->nsamples,
                                      dst->plen, dst->stream) != SGB_OK)
            return cfail(dst, SGB_ERR_CUDA, "merge launch");
    } else if (corr_launch_add(dst->P, src->P, 2 * dst->plen, dst->stream) != SGB_OK) {
        return cfail(dst, SGB_ERR_CUDA, "merge launch");
    }
    (*dst->launches)++;
    if (dst->window < 0 && src->window >= 0) {
        dst->window = src->window;
        cudaMemcpyAsync(dst->g, src->g, sizeof(double) * dst->nomega, cudaMemcpyDeviceToDevice, dst->stream);
    }
    dst->nsamples += src->nsamples;
    cudaStreamSynchronize(dst->stream);
    return SGB_OK;
}

int sgb_corr_compare(const sgb_corr* a, const sgb_corr* b, double* out) {
    if (!a || !b || !out) return fail(nullptr, SGB_ERR_ARG, "null argument");
    sgb_corr* ca = const_cast<sgb_corr*>(a);
    if (!a->welford || !b->welford) return cfail(ca, SGB_ERR_ARG, "both accumulators need calculate_errors");
    if (a->plen != b->plen || a->nomega != b->nomega || a->ncorr != b->ncorr || a->npos != b->npos)
        return cfail(ca, SGB_ERR_ARG, "accumulators have different shapes");
    if (a->nsamples < 2 || b->nsamples < 2) return cfail(ca, SGB_ERR_ARG, "each accumulator needs at least 2 samples");
    if (b->stream != a->stream) cudaStreamSynchronize(b->stream);
    double* part = nullptr;
    if (cudaMalloc((void**)&part, sizeof(double) * 7 * SGB_CMP_BLOCKS) != cudaSuccess)
        return cfail(ca, SGB_ERR_NOMEM, "device allocation failed");
    const double na = (double)a->nsamples, nb = (double)b->nsamples;
    int rc = corr_launch_compare_welford(a->P, a->M, b->P, b->M, 1.0 / (na * (na - 1)), 1.0 / (nb * (nb - 1)), a->plen,
                                         part, a->stream);
    (*ca->launches)++;
    std::vector<double> h(7 * SGB_CMP_BLOCKS);
    cudaError_t e = rc == SGB_OK ? cudaMemcpyAsync(h.data(), part, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, a->stream)
                                 : cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(a->stream);
    cudaFree(part);
    if (rc != SGB_OK || e != cudaSuccess) return cfail(ca, SGB_ERR_CUDA, std::string("compare: ") + cudaGetErrorString(e));
    for (int k = 0; k < 7; k++) {
        double t = 0;
        for (int q = 0; q < SGB_CMP_BLOCKS; q++) t += h[(size_t)q * 7 + k];
        out[k] = t;
    }
    out[7] = (double)a->plen;
    // variance of Σ(|Δ|² − s) estimated from the spread of the per-block partial sums
    // (blocks own interleaved bin sets, so correlated neighbouring bins stay in one block)
    const double G = SGB_CMP_BLOCKS, mean = (out[0] - out[1]) / G;
    double v = 0;
    for (int q = 0; q < SGB_CMP_BLOCKS; q++) {
        const double d = (h[(size_t)q * 7] - h[(size_t)q * 7 + 1]) - mean;
        v += d * d;
    }
    out[8] = G * v / (G - 1);
    return SGB_OK;
}

int sgb_corr_set_time_transform(sgb_corr* c, int32_t kind) {
    if (!c) return fail(nullptr, SGB_ERR_ARG, "null handle");
    if (kind != 0 && kind != 1) return cfail(c, SGB_ERR_ARG, "time transform kind must be 0 (own kernel where it applies) or 1 (cuFFT)");
    c->time_kind = kind;
    return SGB_OK;
}

int sgb_corr_time_transform(const sgb_corr* c) {
    if (!c) return -1;
    return (c->td_fb && c->time_kind == 0) ? 0 : 1;
}

int sgb_corr_cross(const sgb_corr* a1, const sgb_corr* b1, const sgb_corr* a2, const sgb_corr* b2, double* out) {
    if (!a1 || !b1 || !a2 || !b2 || !out) return fail(nullptr, SGB_ERR_ARG, "null argument");
    sgb_corr* ca = const_cast<sgb_corr*>(a1);
    for (const sgb_corr* c : {b1, a2, b2})
        if (c->plen != a1->plen || c->nomega != a1->nomega || c->ncorr != a1->ncorr || c->npos != a1->npos)
            return cfail(ca, SGB_ERR_ARG, "accumulators have different shapes");
    for (const sgb_corr* c : {a1, b1, a2, b2})
        if (!c->welford) return cfail(ca, SGB_ERR_ARG, "the accumulators need calculate_errors (per-sample means)");
    for (const sgb_corr* c : {b1, a2, b2})
        if (c->stream != a1->stream) cudaStreamSynchronize(c->stream);
    double* part = nullptr;
    if (cudaMalloc((void**)&part, sizeof(double) * 2 * SGB_CMP_BLOCKS) != cudaSuccess)
        return cfail(ca, SGB_ERR_NOMEM, "device allocation failed");
    int rc = corr_launch_cross_diff(a1->P, b1->P, a2->P, b2->P, a1->plen, part, a1->stream);
    (*ca->launches)++;
    std::vector<double> h(2 * SGB_CMP_BLOCKS);
    cudaError_t e = rc == SGB_OK ? cudaMemcpyAsync(h.data(), part, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, a1->stream)
                                 : cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(a1->stream);
    cudaFree(part);
    if (rc != SGB_OK || e != cudaSuccess) return cfail(ca, SGB_ERR_CUDA, std::string("cross: ") + cudaGetErrorString(e));
    double t0 = 0, t1 = 0;
    for (int q = 0; q < SGB_CMP_BLOCKS; q++) { t0 += h[2 * q]; t1 += h[2 * q + 1]; }
    // variance of the cross sum from the spread of the per-block partial sums
    const double G = SGB_CMP_BLOCKS, mean = t0 / G;
    double v = 0;
    for (int q = 0; q < SGB_CMP_BLOCKS; q++) v += (h[2 * q] - mean) * (h[2 * q] - mean);
    out[0] = t0;
    out[1] = t1;
    out[2] = G * v / (G - 1);
    return SGB_OK;
}

}  // extern "C"

// ---- internal entry points used by the adjoint (sgb_adjoint.cu) -------------------------------
int sgb_int_midpoint_snap(sgb_system* s, double dt, double tol, int max_iters, int nsteps, const SnapArgs<double>& sn,
                          int64_t* iters) {
    return run_midpoint<double>(s, dt, 0.0, tol, max_iters, nsteps, iters, sn);
}
void sgb_int_window_weights(int n, int window, std::vector<double>& g) { window_weights(n, window, g); }
int sgb_int_ensure_tables(sgb_system* s) { return ensure_tables(s); }
void sgb_int_set_error(const std::string& msg) { g_last_error = msg; }
