// sgb_corr.h -- launchers of the correlation kernels (sgb_corr.cu). Internal.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include "../../include/sunny_gb300.h"

// variant 0: loads/stores through registers; 1: rows moved by warp-specialised bulk
// copies (falls back to 0 when the staging does not fit); err (device int, needed for
// variant 1) is set to 1 if a bounded wait of the bulk variant gave up.
template <class R>
int corr_launch_accum(const R* A, double* P, const int* pairs, int ncorr, int nobs, int npos, int ncell, int nomega,
                      int nrep, size_t rep_stride, cudaStream_t st, int variant = 0, int* err = nullptr);
int corr_launch_gather(const double* P, size_t ld, size_t col0, int ncol, int n, double scale, double* tmp, cudaStream_t st);
int corr_launch_window(double* tmp, int ncol, int n, const double* g, cudaStream_t st);
int corr_launch_scatter(const double* tmp, int ncol, int n, double* out, cudaStream_t st);
int corr_launch_add(double* dst, const double* src, size_t n, cudaStream_t st);
// calculate_errors: per-sample products of a column range, Welford update, merge with M
template <class R>
int corr_launch_product(const R* A, const int* pairs, int ncorr, int nobs, int npos, int ncell, int n, size_t col0,
                        int ncol, double* tmp, cudaStream_t st);
int corr_launch_welford(const double* tmp, int ncol, int n, size_t col0, size_t ld, double count, double* mean, double* M,
                        cudaStream_t st);
int corr_launch_merge_welford(double* d1, double* M1, const double* d2, const double* M2, double n, double m, size_t len,
                              cudaStream_t st);
// 7 partial sums per block of SGB_CMP_BLOCKS blocks (sgb_corr_compare)
#define SGB_CMP_BLOCKS 1024
int corr_launch_compare_welford(const double* ma, const double* Ma, const double* mb, const double* Mb, double fa, double fb,
                                size_t len, double* part, cudaStream_t st);
int corr_launch_cross_diff(const double* a1, const double* b1, const double* a2, const double* b2, size_t len, double* part,
                           cudaStream_t st);
// intensities: gather the columns of a list of wave vectors; phase averaging + combiner
int corr_launch_gather_q(const double* P, size_t ld, const int* qidx, int nq, int B, int n, double scale, double* tmp,
                         cudaStream_t st);
int corr_launch_intensity(const double* tmp, int ncorr, int npos, int n, const double* pref, const double* qcart,
                          const int* widx, int nw, int combiner, int nq, double* out, cudaStream_t st);

// Hand-written time transform of FP32 accumulators (sgb_tdft.cu): Bluestein over a
// 1024-point four-step FFT, for n + m - 1 <= 1024 (n points, the first m of them samples).
bool tdft_supported(int n, int m);
int tdft_tables(int n, int m, void** chirp, void** fb, void** tw);
int tdft_launch(const float* A, float* Ahat, long long ncols, long long stride, long long rep_stride, int n, int m,
                const void* chirp, const void* fb, const void* tw, cudaStream_t st);
