/*
 * NDFT2_2D.cuh -- drop-in replacement for the reference header
 * NFFT/NDFT2_2D.cuh:1-8 (extern "C" NDFT2_2D_GPU), implemented in
 * libnfft2d_gb300.so by the matrix-free FP64 kernel behind
 * nfft2d_ndft2d_f64 (nfft2d_gb300.h).
 *
 *   out[q] = sum_p in[p] exp(-2 pi i (u[q] X[p] / Nu + v[q] Y[p] / Nv)),
 *   M points, N frequencies, device pointers, legacy default stream,
 *   returns after the result is complete (NFFT/NDFT2_2D.cu:37-72).
 * Differences: the cuBLAS handle is accepted and ignored (no GEMV is used),
 * no M x N matrix is allocated and nothing is written to a file.
 *
 * double2_ is the reference's complex type (from its BBComplex.h, which is
 * not part of this library).  A caller that already has that type defines
 * NFFT2D_DOUBLE2_T before including this header; otherwise double2_ is
 * declared here as CUDA's layout-identical double2.
 */
#ifndef NDFT2_2D_CUH
#define NDFT2_2D_CUH

#include <cuda_runtime.h>

typedef struct cublasContext *cublasHandle_t;

#ifndef NFFT2D_DOUBLE2_T
typedef double2 double2_;
#define NFFT2D_DOUBLE2_T double2_
#endif

extern "C" void NDFT2_2D_GPU(cublasHandle_t, const double *__restrict__, const double *__restrict__,
                             const double *__restrict__, const double *__restrict__,
                             const NFFT2D_DOUBLE2_T *__restrict__, NFFT2D_DOUBLE2_T *__restrict__, const int,
                             const int, const int, const int);

#endif
