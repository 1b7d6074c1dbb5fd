// sgb_batch_blk.h -- host interface of the cell-block batched midpoint kernel
// (sgb_batch_blk.cu). Internal.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include "sgb_batch.cuh"

#define SGB_BLK_MAXB 4          // blocks of cells one CTA may own
// threads per CTA of the cell-block kernel: 256, 512 or 1024 (one CTA per SM holds the
// whole block's halo, so the thread count sets the warps that hide the global latency)
#define SGB_BLK_THREADS_MAX 1024

// Geometry of one launch: replicas of L1 x L2 x L3 cells and na atoms, cut into blocks of
// 2^lbx x 2^lby x 2^lbz cells; the midpoint spins live in buffers padded by gw ghost
// cells per side (PX = L1 + 2gw, ...), and a block's halo box is HX = 2^lbx + 2gw, ...
struct BlkGeom {
    int L1, L2, L3, na, gw;
    int lbx, lby, lbz;
    int HX, HY, HZ;
    int PX, PY, PZ;
    int nbx, nby, nbz, nblk;
    int nsr;
    unsigned int tx_bytes;       // bytes of one halo box
    unsigned int halo_bytes;     // shared memory reserved for it (aligned)
};


int blk_occupancy(bool gen, int G, int nt, size_t smem, int* bps);
int blk_launch(bool gen, int G, int nt, int grid, size_t smem, const sgbbatch::BatchArgs<float>& A,
               const sgbbatch::MidArgs<float>& X, const BlkGeom& B, const BlkMaps& maps, float* Hpad, int nsteps,
               float dt, float lam, const sgbbatch::BSnap<float>& sn, cudaStream_t st);
int blk_encode_map(CUtensorMap* out, float* base, const BlkGeom& B, int nrep);
