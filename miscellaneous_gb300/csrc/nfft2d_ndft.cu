// nfft2d_ndft.cu -- exact 2D direct sum in FP64 at arbitrary frequencies,
// matrix-free.  Replaces NDFT2_2D_GPU (NFFT/NDFT2_2D.cu:15-72), which fills an
// explicit M x N FP64 kernel matrix (M*N*16 bytes), writes it to a text file
// and calls cublasZgemv(OP_T).  Here each thread owns one frequency q and
// streams the points through shared memory in tiles; nothing is materialised.
#include <cuda_runtime.h>

#include "nfft2d_internal.h"

namespace {

constexpr int kNdftThreads = 128;
constexpr int kNdftTile = 128;

__global__ void __launch_bounds__(kNdftThreads) k_ndft2d_f64(const double *__restrict__ X,
                                                             const double *__restrict__ Y,
                                                             const double *__restrict__ u,
                                                             const double *__restrict__ v,
                                                             const double2 *__restrict__ in,
                                                             double2 *__restrict__ out, double inv_nu,
                                                             double inv_nv, long long M, long long N, double sgn) {
    __shared__ double sx[kNdftTile], sy[kNdftTile];
    __shared__ double2 sin_[kNdftTile];
    const long long q = static_cast<long long>(blockIdx.x) * kNdftThreads + threadIdx.x;
    const double uq = q < N ? u[q] : 0.0, vq = q < N ? v[q] : 0.0;
    double ar = 0.0, ai = 0.0;
    for (long long p0 = 0; p0 < M; p0 += kNdftTile) {
        const long long p = p0 + threadIdx.x;
        __syncthreads();
        if (threadIdx.x < kNdftTile) {
            sx[threadIdx.x] = p < M ? X[p] : 0.0;
            sy[threadIdx.x] = p < M ? Y[p] : 0.0;
            sin_[threadIdx.x] = p < M ? in[p] : make_double2(0.0, 0.0);
        }
        __syncthreads();
        const long long rem = M - p0;
        const int cnt = rem < kNdftTile ? static_cast<int>(rem) : kNdftTile;
        for (int j = 0; j < cnt; ++j) {
            // phase in turns, reduced to [-1/2, 1/2] before sincospi:
            // (u X) / Nu + (v Y) / Nv  (NDFT2_2D.cu:41-42)
            double a = (uq * sx[j]) * inv_nu;
            a -= rint(a);
            double b = (vq * sy[j]) * inv_nv;
            b -= rint(b);
            double f = a + b;
            f -= rint(f);
            double s, c;
            sincospi(2.0 * f, &s, &c);
            s *= sgn;
            const double2 d = sin_[j];
            ar += d.x * c - d.y * s;
            ai += d.x * s + d.y * c;
        }
    }
    if (q < N) out[q] = make_double2(ar, ai);
}

}  // namespace

extern "C" int nfft2d_ndft2d_f64(const double *X, const double *Y, const double *u, const double *v, const void *in,
                                 void *out, int Nu, int Nv, long long M, long long N, int sign, void *stream) {
    if (M < 0 || N < 0 || Nu == 0 || Nv == 0) return NFFT2D_ERR_INVALID_ARG;
    if (sign != 1 && sign != -1) return NFFT2D_ERR_INVALID_ARG;
    if (N == 0) return NFFT2D_OK;
    if (!u || !v || !out) return NFFT2D_ERR_INVALID_ARG;
    if (M > 0 && (!X || !Y || !in)) return NFFT2D_ERR_INVALID_ARG;
    const long long blocks = (N + kNdftThreads - 1) / kNdftThreads;
    if (blocks > 0x7fffffffLL) return NFFT2D_ERR_INVALID_ARG;
    k_ndft2d_f64<<<static_cast<unsigned>(blocks), kNdftThreads, 0, static_cast<cudaStream_t>(stream)>>>(
        X, Y, u, v, static_cast<const double2 *>(in), static_cast<double2 *>(out), 1.0 / Nu, 1.0 / Nv, M, N,
        static_cast<double>(sign));
    const cudaError_t e = cudaGetLastError();
    if (e == cudaErrorMemoryAllocation) return NFFT2D_ERR_OOM;
    return e == cudaSuccess ? NFFT2D_OK : NFFT2D_ERR_CUDA;
}
