/*
 * NFFT2_2D.cuh -- drop-in replacement for the reference header
 * NFFT/NFFT2_2D.cuh:1-13 (same declarations, same C++ overloads and name
 * mangling), implemented in libnfft2d_gb300.so on top of the C ABI in
 * nfft2d_gb300.h.  Reference callers (e.g. Synthesis/PSO/Synthesis.cu:395,508
 * and PSO.cu:216) relink against libnfft2d_gb300.so unchanged.
 *
 * Semantics kept from the reference (NFFT/NFFT2_2D.cu:329-495):
 *   NFFT2_2D_GPU(result, data, x, y, N1, N2, M) computes
 *       result[i*N2 + j] = sum_p data[p] exp(-2 pi i ((i - N1/2) x[p] / N1 + (j - N2/2) y[p] / N2))
 *   with the reference's window (c = 2, K = 6), points in grid units, all
 *   pointers device pointers, on the legacy default stream, returning after
 *   the result is complete.
 * Differences, all deliberate:
 *   - no cudaMalloc/cudaFree or constant-memory uploads per call: work
 *     buffers live in a plan cached per (N1, N2, precision);
 *   - Calculate_cuFFT_plan_*_NFFT2_2D create (or re-create) that cached plan;
 *     NFFT2_2D_GPU also creates it on first use if the caller did not;
 *   - NFFT2_2D_GPUplan holds the cuFFT handle of the most recently created
 *     plan; it is owned by the library (its layout is the library's padded
 *     grid), so callers must not execute or destroy it themselves;
 *   - errors print one line to stderr and return instead of exit()ing.
 */
#ifndef NFFT2_2D_CUH
#define NFFT2_2D_CUH

#include <cuda_runtime.h>
#include <cufft.h>

extern cufftHandle NFFT2_2D_GPUplan;
void Calculate_cuFFT_plan_Z2Z_NFFT2_2D(const int, const int);
void Calculate_cuFFT_plan_C2C_NFFT2_2D(const int, const int);
void Destroy_cuFFT_plan_NFFT2_2D();
void NFFT2_2D_GPU(float2 *__restrict__, const float2 *__restrict__, const float *__restrict__, const float *__restrict__,
                  const int, const int, const int);
void NFFT2_2D_GPU(double2 *__restrict__, const double2 *__restrict__, const double *__restrict__,
                  const double *__restrict__, const int, const int, const int);

#endif
