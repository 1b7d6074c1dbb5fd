// sgb_batch.cuh -- structures shared by the replica-batch kernels (sgb_batch.cu and
// the cell-block midpoint kernel, sgb_batch_blk.cu). Internal.
#pragma once
#include "sgb_device.cuh"

namespace sgbbatch {
using namespace sgbdev;

// Sites per tile = threads per CTA of the batch kernels (9 warps): 65,536-site replicas split
// into 228 tiles each, so 8 of them give 1,824 tiles, 4 per CTA of a 3-CTA-per-SM grid.
#define SGB_TILE 288
#define SGB_MAXT 8    // tiles one CTA of the midpoint kernel may own

template <class R>
struct BatchArgs {
    Model<R> M;
    const int4* tiles;
    int ntiles;
    const int4* rd;     // (L1, L2, L3, ncell)
    const int* roff;
    const int* pc;      // [NS] packed (c1 | c2<<8 | c3<<16 | atom<<24) of every site
    const int* nbr;     // neighbour tables
    const int* nbo;     // [nrep] table offset of each replica
    const int4* td;     // [ntiles][2] descriptors: (replica, first site, count, uniform atom or -1),
                        //                          (replica offset, replica sites, table offset, 0)
    int NS;
    const R* kap;       // [na]
    const R* h;         // [3][na] or nullptr
    R* S;
    R* P;
    R* D1;
    Ctrl* ctrl;
};

template <class R>
struct MidArgs {
    R* Sp;          // current iterate S' (PV layout)
    R* H;           // 3 rotating buffers of midpoint spins, MV<R>::W * NS elements each
    double* racc;   // [3][nrep] FP64 convergence sums
    R* P1;          // first iterate of the next step (PV layout), ord > 0
    R* H1;          // extrapolation history (PV layout), stepping from S_n. Cell-block kernel:
    R* H2;          // S_{n-1}, S_{n-2}, S_{n-3}. Tile kernel: H1 = S_{n-1}, H2 = S_{n-2} and H3 the
    R* H3;          // history term K of the next first iterate
    int ord;        // initial iterate of each step: 0 S' = S (as the reference), k > 0 polynomial extrapolation of order k
    int nrep;       // replicas of this launch: r0 .. r0 + nrep - 1 (convergence sums and masks relative to r0)
    int r0;
    int accept0;    // with ord > 0: the convergence test also applies at the first iteration (whose
                    // iterate is the extrapolated one), so the next-step data are prepared at every iteration
    double atol2;
    int max_iters;
};

template <class R>
struct BSnap {
    int enabled, nobs, measperiod, t0, ncell, na;
    const R* ops;        // [nobs][3][ns_rep] of one replica (identical replicas)
    R* buf;              // replica r at buf + r*rep_stride (complex)
    size_t rep_stride;   // complex elements between replicas
    R scale;
};

template <class R>
__device__ __forceinline__ void snap_write(const BSnap<R>& sn, int r, int t, int s, int nsr, R x, R y, R z) {
    const int cell = s % sn.ncell, a = s / sn.ncell;
    R* buf = sn.buf + 2 * (size_t)r * sn.rep_stride;
    for (int o = 0; o < sn.nobs; o++) {
        const R* op = sn.ops + (size_t)o * 3 * nsr;
        R v = op[s] * x + op[nsr + s] * y + op[2 * nsr + s] * z;
        size_t idx = (((size_t)t * sn.nobs + o) * sn.na + a) * sn.ncell + cell;
        buf[2 * idx] = v * sn.scale;
        buf[2 * idx + 1] = 0;
    }
}

#define SGB_MAXREP_CORR 64

// Midpoint-private 3-vector buffers (iterate, candidate, rotating midpoint spins). FP32
// keeps one float4 per site so that a neighbour costs one 16-byte load; FP64 keeps SoA
// [3][NS]. K: elements from one site to the next; W * NS: elements of one buffer.
// Midpoint-private 3-vector buffers, read and written only by the thread that owns the
// site (the iterate, the extrapolation history, the next step's first iterate): SoA
// [3][NS] in both precisions, 12 bytes per site in FP32, so that they take less of L2 than
// the float4 layout that neighbour-gathered buffers use.
template <class R>
struct PV {
    __device__ static __forceinline__ void ld(const R* b, int n, int i, R& x, R& y, R& z) {
        x = b[i]; y = b[n + i]; z = b[2 * n + i];
    }
    __device__ static __forceinline__ void st(R* b, int n, int i, R x, R y, R z) {
        b[i] = x; b[n + i] = y; b[2 * n + i] = z;
    }
};

template <class R>
struct MV;
template <>
struct MV<float> {
    static constexpr int K = 4, W = 4;
    __device__ static __forceinline__ void ld(const float* b, int, int i, float& x, float& y, float& z) {
        const float4 v = reinterpret_cast<const float4*>(b)[i];
        x = v.x; y = v.y; z = v.z;
    }
    __device__ static __forceinline__ void st(float* b, int, int i, float x, float y, float z) {
        reinterpret_cast<float4*>(b)[i] = make_float4(x, y, z, 0.f);
    }
};
template <>
struct MV<double> {
    static constexpr int K = 1, W = 3;
    __device__ static __forceinline__ void ld(const double* b, int n, int i, double& x, double& y, double& z) {
        x = b[i]; y = b[n + i]; z = b[2 * n + i];
    }
    __device__ static __forceinline__ void st(double* b, int n, int i, double x, double y, double z) {
        b[i] = x; b[n + i] = y; b[2 * n + i] = z;
    }
};


}  // namespace sgbbatch
