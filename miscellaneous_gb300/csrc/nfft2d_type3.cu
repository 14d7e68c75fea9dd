// nfft2d_type3.cu -- type-3 2D NUFFT (nonuniform points to nonuniform
// frequencies) by Gaussian gridding, the reference's other native NUFFT:
//     F_k = sum_j f_j exp(-i (s_k x_j + t_k y_j))
// following NUFFT_2D_CPU (NFFT/NFFT3/C/NFFT3_2D_C.cpp:199-312): extents and
// centres of both point sets, R = 2.2 and the Gaussian half-width msp for
// the requested accuracy (:234-238), a rescaling that maps the points onto
// [-pi/2, pi/2] around their centre (:243-264), then
//   1) Gaussian spreading of the phase-shifted values onto an Mry x Mrx grid
//      with the pre-compensation exp(b (Dy^2 n_j^2 + Dx^2 n_i^2)) (:38-85);
//   2) a forward 2D FFT (cuFFT here, MKL there, :283-292);
//   3) Gaussian gathering at the scaled frequencies with the
//      post-compensation and the phase of the centres (:156-194).
// The reference's circular shift by half the grid with the (-1)^(i+j)
// checkerboard (:135-151) is folded into the gather's indexing: no pass.
//
// Kernels: one warp per input point for the spread (lanes walk the columns
// of the (2 msp + 1)^2 footprint, so each row's atomic adds are contiguous)
// and one warp per output frequency for the gather (the same footprint,
// coalesced row reads, a warp-shuffle reduction).  Weights and coordinates
// are FP64; the grid and the sums use the data precision.
#include <cuda_runtime.h>
#include <cufft.h>

#include <cfloat>
#include <cmath>
#include <cstring>

#include "nfft2d_internal.h"

namespace {

constexpr double kPi = 3.141592653589793238463;  // the reference's PI (NFFT3_2D_C.cpp:24)
constexpr int kWarpsPerBlock = 8;

__device__ __forceinline__ unsigned long long ord_key(double v) {
    const unsigned long long u = static_cast<unsigned long long>(__double_as_longlong(v));
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
double ord_value(unsigned long long k) {
    const unsigned long long u = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    double v;
    std::memcpy(&v, &u, sizeof v);
    return v;
}

// min / max of two arrays of n values: mm[0..3] = keys of min a, max a, min b, max b
__global__ void k_minmax2(const double *__restrict__ a, const double *__restrict__ b, long long n,
                          unsigned long long *mm) {
    double amin = DBL_MAX, amax = -DBL_MAX, bmin = DBL_MAX, bmax = -DBL_MAX;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        amin = fmin(amin, a[i]);
        amax = fmax(amax, a[i]);
        bmin = fmin(bmin, b[i]);
        bmax = fmax(bmax, b[i]);
    }
    for (int o = 16; o > 0; o >>= 1) {
        amin = fmin(amin, __shfl_xor_sync(0xffffffffu, amin, o));
        amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, o));
        bmin = fmin(bmin, __shfl_xor_sync(0xffffffffu, bmin, o));
        bmax = fmax(bmax, __shfl_xor_sync(0xffffffffu, bmax, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(mm + 0, ord_key(amin));
        atomicMax(mm + 1, ord_key(amax));
        atomicMin(mm + 2, ord_key(bmin));
        atomicMax(mm + 3, ord_key(bmax));
    }
}

struct Params {
    double xb, yb, sb, tb;   // centres after the rescaling
    double kx, ky;           // rescaling X1 / (pi/2), Y1 / (pi/2)
    double Dx, Dy;           // grid steps 2 pi / Mr
    double b, t1, fact;      // Gaussian constants, fact = (1 / (4 pi b))^2
    int Mrx, Mry, ms;        // grid and footprint half-width
};

__device__ __forceinline__ int wrap(long long i, int n) {
    long long r = i % n;
    return static_cast<int>(r < 0 ? r + n : r);
}

template <typename C2, typename Real>
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
    k_t3_spread(const double *__restrict__ x, const double *__restrict__ y, const C2 *__restrict__ f, long long n,
                Params P, C2 *__restrict__ grid) {
    const long long p = blockIdx.x * static_cast<long long>(kWarpsPerBlock) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (p >= n) return;
    const double xs = x[p] / P.kx, ys = y[p] / P.ky;  // :245-246
    // value with the centre phase removed (:48-51) and the constant factor
    const double arg = P.sb * xs + P.tb * ys;
    double sa, ca;
    sincos(arg, &sa, &ca);
    const double fr = static_cast<double>(f[p].x), fi = static_cast<double>(f[p].y);
    const double re = (fr * ca + fi * sa) * P.fact, im = (fi * ca - fr * sa) * P.fact;
    const double x_temp = (xs - P.xb) / P.Dx, y_temp = (ys - P.yb) / P.Dy;  // :53-54
    const long long nn_off = static_cast<long long>(floor(P.Mrx / 2 + x_temp));
    const long long mm_off = static_cast<long long>(floor(P.Mry / 2 + y_temp));
    const int W = 2 * P.ms + 1;
    for (int c = lane; c < W; c += 32) {
        const long long i = c - P.ms + nn_off;
        const double dsi = static_cast<double>(i - P.Mrx / 2);
        const double ex = P.b * P.Dx * P.Dx * dsi * dsi - P.t1 * (x_temp - dsi) * (x_temp - dsi);
        const int ii = wrap(i, P.Mrx);
        for (int r = 0; r < W; ++r) {
            const long long j = r - P.ms + mm_off;
            const double dsj = static_cast<double>(j - P.Mry / 2);
            const double e = exp(ex + P.b * P.Dy * P.Dy * dsj * dsj - P.t1 * (y_temp - dsj) * (y_temp - dsj));  // :74
            Real *cell = reinterpret_cast<Real *>(grid + static_cast<size_t>(wrap(j, P.Mry)) * P.Mrx + ii);
            atomicAdd(cell, static_cast<Real>(re * e));
            atomicAdd(cell + 1, static_cast<Real>(im * e));
        }
    }
}

template <typename C2>
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
    k_t3_gather(const double *__restrict__ s, const double *__restrict__ t, long long n, Params P,
                const C2 *__restrict__ grid, C2 *__restrict__ F) {
    const long long k = blockIdx.x * static_cast<long long>(kWarpsPerBlock) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (k >= n) return;
    const double ss = s[k] * P.kx, ts = t[k] * P.ky;  // :247-248
    const double us = P.Mrx / 2 + (ss - P.sb), ut = P.Mry / 2 + (ts - P.tb);  // Ds = Dt = 1 (:163-166)
    const long long nsn = static_cast<long long>(floor(us)), ntn = static_cast<long long>(floor(ut));
    const double difs = us - nsn, dift = ut - ntn;
    const int W = 2 * P.ms + 1;
    double a0 = 0.0, a1 = 0.0;
    for (int c = lane; c < W; c += 32) {
        const long long nn = nsn - P.ms + c;  // shifted column; source column (nn + Mrx/2) mod Mrx
        const double npj = static_cast<double>(c - P.ms);
        const double es = -P.t1 * (difs - npj) * (difs - npj);
        const int i = wrap(nn + P.Mrx / 2, P.Mrx);
        for (int r = 0; r < W; ++r) {
            const long long mm = ntn - P.ms + r;
            const double npi = static_cast<double>(r - P.ms);
            const double e = exp(es - P.t1 * (dift - npi) * (dift - npi));  // :182
            const int j = wrap(mm + P.Mry / 2, P.Mry);
            const C2 v = grid[static_cast<size_t>(j) * P.Mrx + i];
            const double sg = ((i + j) & 1) ? -e : e;  // the (-1)^(i+j) of :147-148
            a0 += static_cast<double>(v.x) * sg;
            a1 += static_cast<double>(v.y) * sg;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        a0 += __shfl_xor_sync(0xffffffffu, a0, o);
        a1 += __shfl_xor_sync(0xffffffffu, a1, o);
    }
    if (lane == 0) {
        double tmp1 = P.Dy * (ts - P.tb);
        tmp1 = tmp1 * tmp1;
        double tmp2 = P.Dx * (ss - P.sb);
        tmp2 = tmp2 * tmp2;
        const double comp = exp(P.b * (tmp1 + tmp2));                 // :170-172
        const double arg = (ss - P.sb) * P.xb + (ts - P.tb) * P.yb;   // :189
        double sa, ca;
        sincos(arg, &sa, &ca);
        C2 o;
        o.x = static_cast<decltype(o.x)>((a0 * ca + a1 * sa) * comp);
        o.y = static_cast<decltype(o.x)>((a1 * ca - a0 * sa) * comp);
        F[k] = o;
    }
}

int cuda_status(cudaError_t e) {
    if (e == cudaSuccess) return NFFT2D_OK;
    return e == cudaErrorMemoryAllocation ? NFFT2D_ERR_OOM : NFFT2D_ERR_CUDA;
}

#define T3_CUDA(expr)                                   \
    do {                                                \
        const int st_ = cuda_status(expr);              \
        if (st_ != NFFT2D_OK) return st_;               \
    } while (0)

int minmax(const double *a, const double *b, long long n, unsigned long long *d_mm, cudaStream_t st, double out[4]) {
    const unsigned long long init[4] = {~0ull, 0ull, ~0ull, 0ull};
    T3_CUDA(cudaMemcpyAsync(d_mm, init, sizeof init, cudaMemcpyHostToDevice, st));
    const int blocks = static_cast<int>(std::max<long long>(1, std::min<long long>((n + 255) / 256, 1024)));
    k_minmax2<<<blocks, 256, 0, st>>>(a, b, n, d_mm);
    T3_CUDA(cudaGetLastError());
    unsigned long long h[4];
    T3_CUDA(cudaMemcpyAsync(h, d_mm, sizeof h, cudaMemcpyDeviceToHost, st));
    T3_CUDA(cudaStreamSynchronize(st));
    for (int i = 0; i < 4; ++i) out[i] = ord_value(h[i]);
    return NFFT2D_OK;
}

struct Scratch {
    cudaStream_t st;
    void *mm = nullptr, *grid = nullptr;
    cufftHandle plan = 0;
    bool plan_ok = false;
    ~Scratch() {
        if (plan_ok) cufftDestroy(plan);
        if (grid) cudaFreeAsync(grid, st);
        if (mm) cudaFreeAsync(mm, st);
    }
};

}  // namespace

extern "C" int nfft2d_nufft3_2d(const double *x, const double *y, const double *s, const double *t, const void *f,
                                void *F, double eps, long long len_in, long long len_out, int precision,
                                void *stream) {
    if (!x || !y || !s || !t || !f || !F || len_in < 1 || len_out < 1) return NFFT2D_ERR_INVALID_ARG;
    if (!(eps > 0 && eps < 1)) return NFFT2D_ERR_INVALID_ARG;
    if (precision != NFFT2D_F32 && precision != NFFT2D_F64) return NFFT2D_ERR_INVALID_ARG;
    if (len_in > (1LL << 40) || len_out > (1LL << 40)) return NFFT2D_ERR_INVALID_ARG;
    const cudaStream_t st = static_cast<cudaStream_t>(stream);
    Scratch S{st};
    T3_CUDA(cudaMallocAsync(&S.mm, 4 * sizeof(unsigned long long), st));
    double exy[4], est[4];
    int rc = minmax(x, y, len_in, static_cast<unsigned long long *>(S.mm), st, exy);
    if (rc != NFFT2D_OK) return rc;
    rc = minmax(s, t, len_out, static_cast<unsigned long long *>(S.mm), st, est);
    if (rc != NFFT2D_OK) return rc;
    for (double v : exy)
        if (!std::isfinite(v)) return NFFT2D_ERR_NONFINITE;
    for (double v : est)
        if (!std::isfinite(v)) return NFFT2D_ERR_NONFINITE;
    // :214-232 (the reductions start from -+FLT_MAX, which finite data within
    // range never leaves)
    double Max_x = exy[1], min_x = exy[0], Max_y = exy[3], min_y = exy[2];
    double Max_s = est[1], min_s = est[0], Max_t = est[3], min_t = est[2];
    double xb = (Max_x + min_x) / 2, X1 = std::fabs(Max_x - xb);
    double yb = (Max_y + min_y) / 2, Y1 = std::fabs(Max_y - yb);
    double sb = (Max_s + min_s) / 2, Sx = std::fabs(Max_s - sb);
    double tb = (Max_t + min_t) / 2, Ty = std::fabs(Max_t - tb);
    if (!(X1 > 0) || !(Y1 > 0)) return NFFT2D_ERR_INVALID_ARG;  // all points on one line: no scale
    const double R = 2.2;
    double msp = 2 + 2 * (R * R) * (-std::log(eps / 76)) / (kPi * (R * R - 2));  // :235
    const double mrx = 2 * std::ceil((X1 * Sx / kPi) * R * R + R * msp);         // :237-238
    const double mry = 2 * std::ceil((Y1 * Ty / kPi) * R * R + R * msp);
    if (!(mrx <= 65536) || !(mry <= 65536) || mrx * mry > 1.5e9) return NFFT2D_ERR_UNSUPPORTED;
    Params P{};
    P.Mrx = static_cast<int>(mrx);
    P.Mry = static_cast<int>(mry);
    P.Dx = 2 * kPi / P.Mrx;
    P.Dy = 2 * kPi / P.Mry;
    P.kx = X1 / (kPi / 2);
    P.ky = Y1 / (kPi / 2);
    Max_x = Max_x / P.kx;
    min_x = min_x / P.kx;
    P.xb = (Max_x + min_x) / 2;
    Max_s = Max_s * P.kx;
    min_s = min_s * P.kx;
    P.sb = (Max_s + min_s) / 2;
    Max_y = Max_y / P.ky;
    min_y = min_y / P.ky;
    P.yb = (Max_y + min_y) / 2;
    Max_t = Max_t * P.ky;
    min_t = min_t * P.ky;
    P.tb = (Max_t + min_t) / 2;
    P.b = (msp - 2) / (4 * kPi);
    P.t1 = 1 / (4 * P.b);
    msp = std::floor(msp - 2);
    P.ms = static_cast<int>(msp);
    const double f0 = 1. / (4. * kPi * P.b);
    P.fact = f0 * f0;

    const bool dbl = precision == NFFT2D_F64;
    const size_t cells = static_cast<size_t>(P.Mrx) * P.Mry;
    const size_t csz = dbl ? sizeof(double2) : sizeof(float2);
    T3_CUDA(cudaMallocAsync(&S.grid, cells * csz, st));
    T3_CUDA(cudaMemsetAsync(S.grid, 0, cells * csz, st));
    const unsigned blk_in = static_cast<unsigned>((len_in + kWarpsPerBlock - 1) / kWarpsPerBlock);
    const unsigned blk_out = static_cast<unsigned>((len_out + kWarpsPerBlock - 1) / kWarpsPerBlock);
    if (dbl)
        k_t3_spread<double2, double><<<blk_in, kWarpsPerBlock * 32, 0, st>>>(
            x, y, static_cast<const double2 *>(f), len_in, P, static_cast<double2 *>(S.grid));
    else
        k_t3_spread<float2, float><<<blk_in, kWarpsPerBlock * 32, 0, st>>>(
            x, y, static_cast<const float2 *>(f), len_in, P, static_cast<float2 *>(S.grid));
    T3_CUDA(cudaGetLastError());
    // :283-292 -- rows are Mry, the fast (column) dimension Mrx
    if (cufftPlan2d(&S.plan, P.Mry, P.Mrx, dbl ? CUFFT_Z2Z : CUFFT_C2C) != CUFFT_SUCCESS) return NFFT2D_ERR_CUFFT;
    S.plan_ok = true;
    if (cufftSetStream(S.plan, st) != CUFFT_SUCCESS) return NFFT2D_ERR_CUFFT;
    const cufftResult fr =
        dbl ? cufftExecZ2Z(S.plan, static_cast<cufftDoubleComplex *>(S.grid), static_cast<cufftDoubleComplex *>(S.grid),
                           CUFFT_FORWARD)
            : cufftExecC2C(S.plan, static_cast<cufftComplex *>(S.grid), static_cast<cufftComplex *>(S.grid),
                           CUFFT_FORWARD);
    if (fr != CUFFT_SUCCESS) return NFFT2D_ERR_CUFFT;
    if (dbl)
        k_t3_gather<double2><<<blk_out, kWarpsPerBlock * 32, 0, st>>>(s, t, len_out, P,
                                                                     static_cast<const double2 *>(S.grid),
                                                                     static_cast<double2 *>(F));
    else
        k_t3_gather<float2><<<blk_out, kWarpsPerBlock * 32, 0, st>>>(s, t, len_out, P,
                                                                    static_cast<const float2 *>(S.grid),
                                                                    static_cast<float2 *>(F));
    T3_CUDA(cudaGetLastError());
    return cuda_status(cudaStreamSynchronize(st));
}
