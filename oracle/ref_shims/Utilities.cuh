/*
 * Stand-in for the reference's Utilities.cuh, which the reference does not
 * ship (NFFT/NFFT2_2D.cu:5 includes it).  Written here from the way
 * NFFT/NFFT2_2D.cu uses each name; TEST INFRASTRUCTURE ONLY (the reference
 * GPU spreading is built from it as a parity oracle).
 *
 *   iDivUp(a, b)     ceil(a / b) for positive ints (grid sizing, :352,370)
 *   gpuErrchk(call)  report a failing CUDA runtime call (no exit: the
 *                    oracle build never runs host code, but keeps it valid)
 *   modulo(a, n)     non-negative remainder of an integer-valued real a by
 *                    a positive int n, as an int (:124-125,151-152): the
 *                    wrapped oversampled-grid index of a tap
 */
#ifndef ORACLE_REF_SHIM_UTILITIES_CUH
#define ORACLE_REF_SHIM_UTILITIES_CUH

#include <cstdio>
#include <cuda_runtime.h>

__host__ __device__ inline int iDivUp(int a, int b) { return (a % b != 0) ? (a / b + 1) : (a / b); }

#define gpuErrchk(call)                                                                        \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess) printf("CUDA error %s at %s:%d\n", cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

template <class T>
__host__ __device__ inline int modulo(T a, int n)
{
    /* a is integral by construction (rint(c x) + tap offset + c N / 2). */
    long long ai = (long long)a;
    long long r = ai % n;
    if (r < 0) r += n;
    return (int)r;
}

#endif
