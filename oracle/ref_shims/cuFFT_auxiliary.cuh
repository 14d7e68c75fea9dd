/*
 * Stand-in for the reference's cuFFT_auxiliary.cuh (not shipped;
 * NFFT/NFFT2_2D.cu:7).  TEST INFRASTRUCTURE ONLY.
 *
 *   cufftSafeCall(call)       report a failing cuFFT call (no exit)
 *   fftshift_2D(d, n1, n2)    the reference applies it before and after the
 *                             forward cuFFT so that the pair computes
 *                             fftshift(fft2(ifftshift(u))) as in
 *                             NFFT/NFFT2/Matlab/NFFT2_2D.m:63.  For even
 *                             n1, n2 (n = c N, N even) that is a multiply
 *                             of cell (i, j) by (-1)^(i+j) before and after
 *                             the FFT: the shift theorem, the same device
 *                             as NFFT/NFFT3/C/NFFT3_2D_C.cpp:147-148.
 *                             One thread per cell; threads outside the
 *                             n1 x n2 grid do nothing.
 */
#ifndef ORACLE_REF_SHIM_CUFFT_AUXILIARY_CUH
#define ORACLE_REF_SHIM_CUFFT_AUXILIARY_CUH

#include <cstdio>
#include <cufft.h>

#define cufftSafeCall(call)                                                                    \
    do {                                                                                       \
        cufftResult r_ = (call);                                                               \
        if (r_ != CUFFT_SUCCESS) printf("cuFFT error %d at %s:%d\n", (int)r_, __FILE__, __LINE__); \
    } while (0)

template <class T>
__global__ void fftshift_2D(T *__restrict__ data, const int n1, const int n2)
{
    const int i = threadIdx.x + blockDim.x * blockIdx.x;
    const int j = threadIdx.y + blockDim.y * blockIdx.y;
    if (i < n1 && j < n2 && ((i + j) & 1)) {
        T v = data[(long long)i * n2 + j];
        v.x = -v.x;
        v.y = -v.y;
        data[(long long)i * n2 + j] = v;
    }
}

#endif
