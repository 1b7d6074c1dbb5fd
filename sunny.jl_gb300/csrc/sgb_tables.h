// sgb_tables.h -- host-side packing of coupling tables for the kernels (internal).
//
// Sunny stores each pair coupling from both ends: the non-culled copy with J and the
// culled reverse copy with J^T (src/System/PairExchange.jl:228-236, 466-467). The packer
// emits both directed copies per sublattice so that the kernels gather. Onsite Stevens
// coefficients follow StevensExpansion's rule of dropping k-blocks with norm < 1e-12
// (src/System/Types.jl:12-16).
#pragma once
#include <cmath>
#include <complex>
#include <string>
#include <vector>
#include "sgb_internal.h"

namespace sgbhost {

inline int imod(int x, int L) {
    int r = x % L;
    return r < 0 ? r + L : r;
}

inline size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

// Stevens quadrupoles O[2,q], q = 2..-2, of dimension N (src/Operators/Stevens.jl:12-86),
// column-major complex.
inline void stevens_quadrupoles(int N, std::vector<std::complex<double>>& out) {
    typedef std::complex<double> cd;
    out.assign(5 * N * N, cd(0, 0));
    if (N <= 2) return;
    double s = (N - 1) / 2.0;
    std::vector<cd> Sx(N * N), Sy(N * N), Sz(N * N);
    for (int j = 1; j <= N - 1; j++) {
        double off = std::sqrt(2 * (s + 1) * j - (double)j * (j + 1)) / 2;
        int r = j - 1, c = j;
        Sx[r + N * c] = off; Sx[c + N * r] = off;
        Sy[r + N * c] = cd(0, -off); Sy[c + N * r] = cd(0, off);
    }
    for (int k = 0; k < N; k++) Sz[k + N * k] = s - k;
    auto mul = [N](const std::vector<cd>& A, const std::vector<cd>& B) {
        std::vector<cd> C(N * N);
        for (int c = 0; c < N; c++)
            for (int r = 0; r < N; r++) {
                cd acc = 0;
                for (int k = 0; k < N; k++) acc += A[r + N * k] * B[k + N * c];
                C[r + N * c] = acc;
            }
        return C;
    };
    std::vector<cd> Jp(N * N), Jm(N * N);
    for (int i = 0; i < N * N; i++) { Jp[i] = Sx[i] + cd(0, 1) * Sy[i]; Jm[i] = Sx[i] - cd(0, 1) * Sy[i]; }
    auto Jp2 = mul(Jp, Jp), Jm2 = mul(Jm, Jm), Jz2 = mul(Sz, Sz);
    auto X = mul(Sx, Sx);
    { auto t = mul(Sy, Sy); for (int i = 0; i < N * N; i++) X[i] += t[i] + Jz2[i]; }
    std::vector<cd> A(N * N);
    for (int i = 0; i < N * N; i++) out[0 * N * N + i] = 0.5 * (Jp2[i] + Jm2[i]);
    for (int i = 0; i < N * N; i++) A[i] = 0.5 * (Jp[i] + Jm[i]);
    { auto a = mul(A, Sz), b = mul(Sz, A); for (int i = 0; i < N * N; i++) out[1 * N * N + i] = 0.5 * (a[i] + b[i]); }
    for (int i = 0; i < N * N; i++) out[2 * N * N + i] = 3.0 * Jz2[i] - X[i];
    for (int i = 0; i < N * N; i++) A[i] = (Jp[i] - Jm[i]) / cd(0, 2);
    { auto a = mul(A, Sz), b = mul(Sz, A); for (int i = 0; i < N * N; i++) out[3 * N * N + i] = 0.5 * (a[i] + b[i]); }
    for (int i = 0; i < N * N; i++) out[4 * N * N + i] = (Jp2[i] - Jm2[i]) / cd(0, 2);
}

// Packs the tables. `dims` reduces bond offsets mod L (single systems); nullptr keeps the
// raw offsets (replica batches of different sizes). Returns "" or an error message.
// Coefficients a(M) with <Z|M|Z> = a(M)·ρ for the packed density ρ of a ket (Re M_rr; then
// 2 Re M_rc, -2 Im M_rc for r < c). M: N x N complex, column-major (re, im).
template <class R>
inline void density_coeffs(int N, const double* Mx, R* out) {
    for (int r = 0; r < N; r++) out[r] = (R)Mx[2 * (r + N * r)];
    int k = N;
    for (int r = 0; r < N; r++)
        for (int c = r + 1; c < N; c++) {
            out[k++] = (R)(2 * Mx[2 * (r + N * c)]);
            out[k++] = (R)(-2 * Mx[2 * (r + N * c) + 1]);
        }
}

// SU(N) general pair couplings: term t (A[t] ⊗ B[t]) on input bond gbond[t].
struct GeneralTerms {
    std::vector<int> bond;
    std::vector<double> A, B;   // [nterms][N][N] complex column-major (re, im)
};

template <class R>
std::string pack_tables(int na, int N, bool sun, const int* dims, const std::vector<sgb_bond>& bonds_in,
                        const std::vector<double>& onsite, Model<R>& M, std::vector<unsigned char>& buf,
                        bool& any_bq, const GeneralTerms* gen = nullptr, std::vector<R>* grows = nullptr) {
    std::vector<std::vector<DBond<R>>> per(na);
    std::vector<R> bqtab;
    any_bq = false;
    if (grows) grows->clear();
    const int NN = N * N;
    for (size_t bi = 0; bi < bonds_in.size(); bi++) {
        const sgb_bond& b = bonds_in[bi];
        for (int dir = 0; dir < 2; dir++) {
            DBond<R> e{};
            if (gen && grows) {
                // rows (a(first), first, a(second)): the site's own operator first; the
                // reversed copy swaps A and B (reverse(tensordec))
                const size_t gidx = grows->size() / (4 * NN);
                int gcnt = 0;
                for (size_t t = 0; t < gen->bond.size(); t++) {
                    if (gen->bond[t] != (int)bi) continue;
                    const double* A = gen->A.data() + 2 * NN * t;
                    const double* Bm = gen->B.data() + 2 * NN * t;
                    const double* first = dir == 0 ? A : Bm;
                    const double* second = dir == 0 ? Bm : A;
                    std::vector<R> row(4 * NN);
                    density_coeffs<R>(N, first, row.data());
                    for (int k = 0; k < 2 * NN; k++) row[NN + k] = (R)first[k];
                    density_coeffs<R>(N, second, row.data() + 3 * NN);
                    grows->insert(grows->end(), row.begin(), row.end());
                    gcnt++;
                }
                if (gidx >= (1u << 20) || gcnt >= (1 << 12)) return "too many general coupling terms";
                e.gref = gcnt ? (int)gidx | (gcnt << 20) : 0;
            }
            int from = dir == 0 ? b.i : b.j;
            int to = dir == 0 ? b.j : b.i;
            e.j = to;
            for (int k = 0; k < 3; k++) {
                int n = dir == 0 ? b.n[k] : -b.n[k];
                e.n[k] = dims ? imod(n, dims[k]) : n;
            }
            bool iso = true;
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) {
                    double v = dir == 0 ? b.bilin[r + 3 * c] : b.bilin[c + 3 * r];
                    e.J[r + 3 * c] = (R)v;
                    if (r != c && v != 0.0) iso = false;
                }
            if (!(b.bilin[0] == b.bilin[4] && b.bilin[0] == b.bilin[8])) iso = false;
            e.jkind = iso ? 0 : 1;
            e.scalar = (R)b.scalar;
            e.bqkind = b.biquad_kind;
            e.bq = 0;
            e.bqidx = 0;
            if (b.biquad_kind == 1) {
                e.bq = (R)b.biquad[0];
                if (b.biquad[0] == 0.0) e.bqkind = 0;
            } else if (b.biquad_kind == 2) {
                e.bqidx = (int)(bqtab.size() / 25);
                for (int c = 0; c < 5; c++)
                    for (int r = 0; r < 5; r++)
                        bqtab.push_back((R)(dir == 0 ? b.biquad[r + 5 * c] : b.biquad[c + 5 * r]));
            }
            if (e.bqkind != 0) any_bq = true;
            e.fwd = dir == 0 ? 1 : 0;
            {
                int n0 = dir == 0 ? b.n[0] : -b.n[0], n1 = dir == 0 ? b.n[1] : -b.n[1], n2 = dir == 0 ? b.n[2] : -b.n[2];
                if (n0 < -128 || n0 > 127 || n1 < -128 || n1 > 127 || n2 < -128 || n2 > 127) return "bond offset exceeds 127 cells";
                e.pk = (n0 + 128) | ((n1 + 128) << 8) | ((n2 + 128) << 16) | (to << 24);
            }
            per[from].push_back(e);
        }
    }
    int nb = 0;
    for (auto& v : per) nb += (int)v.size();
    int nbq = (int)(bqtab.size() / 25);
    size_t off = 0;
    M.off_stev = (int)off; off = align16(off + sizeof(R) * 28 * na);
    M.off_kmax = (int)off; off = align16(off + sizeof(int) * na);
    M.off_boff = (int)off; off = align16(off + sizeof(int) * (na + 1));
    M.off_bonds = (int)off; off = align16(off + sizeof(DBond<R>) * nb);
    M.off_bq = (int)off; off = align16(off + sizeof(R) * 25 * nbq);
    M.off_lam = (int)off; off = align16(off + sizeof(R) * 2 * N * N * (sun ? na : 0));
    M.off_qmat = (int)off; off = align16(off + sizeof(R) * 2 * N * N * 5 * (sun ? 1 : 0));
    size_t bytes = align16(off);
    if (bytes > 200 * 1024) return "coupling tables exceed 200 KiB of shared memory";
    buf.assign(bytes, 0);
    R* stev = reinterpret_cast<R*>(buf.data() + M.off_stev);
    int* kmax = reinterpret_cast<int*>(buf.data() + M.off_kmax);
    int* boff = reinterpret_cast<int*>(buf.data() + M.off_boff);
    DBond<R>* bonds = reinterpret_cast<DBond<R>*>(buf.data() + M.off_bonds);
    R* bq = reinterpret_cast<R*>(buf.data() + M.off_bq);
    if (!sun) {
        for (int a = 0; a < na; a++) {
            const double* c = onsite.data() + 28 * a;
            const int start[4] = {0, 1, 6, 15}, len[4] = {1, 5, 9, 13};
            int km = 0;
            for (int g = 0; g < 4; g++) {
                double nrm = 0;
                for (int q = 0; q < len[g]; q++) nrm += c[start[g] + q] * c[start[g] + q];
                bool zero = std::sqrt(nrm) < 1e-12;
                for (int q = 0; q < len[g]; q++) stev[28 * a + start[g] + q] = zero ? (R)0 : (R)c[start[g] + q];
                if (!zero && g > 0) km = 2 * g;
            }
            kmax[a] = km;
        }
    } else {
        R* lam = reinterpret_cast<R*>(buf.data() + M.off_lam);
        for (int i = 0; i < 2 * N * N * na; i++) lam[i] = (R)onsite[i];
        std::vector<std::complex<double>> qm;
        stevens_quadrupoles(N, qm);
        R* q = reinterpret_cast<R*>(buf.data() + M.off_qmat);
        for (int i = 0; i < 5 * N * N; i++) { q[2 * i] = (R)qm[i].real(); q[2 * i + 1] = (R)qm[i].imag(); }
    }
    int k = 0;
    for (int a = 0; a < na; a++) {
        boff[a] = k;
        for (auto& e : per[a]) bonds[k++] = e;
    }
    boff[na] = k;
    for (size_t i = 0; i < bqtab.size(); i++) bq[i] = bqtab[i];
    M.na = na;
    M.N = N;
    M.dipole_mode = sun ? 0 : 1;
    M.has_biquad = any_bq ? 1 : 0;
    M.general = 0;
    for (auto& v : per)
        for (auto& e : v)
            if (e.jkind != 0 || e.bqkind != 0) M.general = 1;
    M.has_general = (grows && !grows->empty()) ? 1 : 0;
    M.qrows = sun ? 5 + N * N : 5;
    M.tables_bytes = (int)bytes;
    M.nb = nb;
    M.nbq = nbq;
    return "";
}

}  // namespace sgbhost
