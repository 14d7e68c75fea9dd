// nfft2d_noalloc.cu -- a forward (type-2) transform for small grids that
// allocates no memory at all.
//
// Who needs it: code that must not call cudaMalloc (or anything that does,
// such as creating a cuFFT plan) while it runs.  Typical cases are a host
// application that owns every device allocation through its own pool and
// forbids extensions to allocate behind its back (a MATLAB MEX gateway working
// on gpuArray data is one), and latency-critical loops where cudaMalloc's
// implicit device synchronisation and unbounded run time are not acceptable.
//
// How: every work buffer -- the padded oversampled grid, the row-transform
// intermediate and the two deapodization tables -- lives in ONE file-scope
// `static __device__` array (kScratchBytes, about 1.12 MB; every GPU that
// loads the library holds it until the process exits).  The uniform-grid
// transform is a direct DFT by rows then columns in this file's own kernels,
// because a cuFFT plan cannot be created without allocating; that is cheap at
// these sizes (sigma*N <= 256).  Points are not binned: the gather reduces
// each coordinate itself and reads its taps straight from the grid.
//
// Host code cannot pass the array's name to a kernel (in host code it is a
// host-side stand-in, not a device address), so the device address is taken
// with cudaGetSymbolAddress once per device, on the first call made with that
// device current, and cached.  The cache lives as long as the process: a
// cudaDeviceReset (or any other teardown of the device's primary context)
// reloads the module and may move the array, after which this entry point
// must not be called again in the same process.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "nfft2d_device.cuh"
#include "nfft2d_internal.h"

namespace {

using nfft2d::kHalo;

constexpr int kMaxN = 128;                       // N1, N2 <= 128 (sigma = 2: grid <= 256)
constexpr int kMaxGrid = 2 * kMaxN;              // oversampled size
constexpr int kMaxPitch = kMaxGrid + 2 * kHalo;  // padded grid side, halo on both sides
constexpr size_t kGridElems = static_cast<size_t>(kMaxPitch) * kMaxPitch;
constexpr size_t kRowElems = static_cast<size_t>(kMaxGrid) * kMaxGrid;
constexpr size_t kTableElems = kMaxN;            // 2 * kMaxN floats, stored as float2 slots
constexpr size_t kScratchElems = kGridElems + kRowElems + kTableElems;
constexpr size_t kScratchBytes = kScratchElems * sizeof(float2);
constexpr double kSigma = 2.0;                   // the reference's c (NFFT2_2D.cu:20)
constexpr double kPi = 3.141592653589793238462643383279502884;

static __device__ __align__(256) float2 g_scratch[kScratchElems];

std::mutex g_mu;
constexpr int kMaxDevices = 64;
float2 *g_scratch_ptr[kMaxDevices] = {};

// Device address of g_scratch on the current device (looked up once per device).
int scratch_address(float2 **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return NFFT2D_ERR_CUDA;
    if (dev < 0 || dev >= kMaxDevices) return NFFT2D_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess || !p) return NFFT2D_ERR_CUDA;
        g_scratch_ptr[dev] = static_cast<float2 *>(p);
    }
    *out = g_scratch_ptr[dev];
    return NFFT2D_OK;
}

// Deapodization tables S / I0(K sqrt(alpha^2 - xi^2)), S = sinh(alpha K)/(pi K),
// xi = 2 pi k / (sigma N), in FP64 (the same values a plan computes on the host).
__global__ void k_na_deap(float *tab, int N1, int N2, int K, double alpha) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N1 + N2) return;
    const int N = i < N1 ? N1 : N2;
    const int k = (i < N1 ? i : i - N1) - N / 2;
    const double xi = 2.0 * kPi * k / (kSigma * N);
    const double x = K * sqrt(alpha * alpha - xi * xi);
    const double q = 0.25 * x * x;
    double term = 1.0, sum = 1.0;  // I0 power series (Abramowitz & Stegun 9.6.12)
    for (int j = 1; j < 200; ++j) {
        term *= q / (static_cast<double>(j) * j);
        sum += term;
        if (term < 1e-18 * sum) break;
    }
    const double S = sinh(alpha * K) / (kPi * K);
    tab[i] = static_cast<float>(S / sum);
}

// Zero-padded, deapodized coefficients on the grid interior: FFT index r holds
// frequency r (r < n/2) or r - n.  Every interior cell is written.
__global__ void k_na_pad(const float2 *__restrict__ F, float2 *__restrict__ grid, const float *__restrict__ tab,
                         int N1, int N2, int n1, int n2, int C) {
    const int r = blockIdx.y, c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n2) return;
    const int k1 = r < n1 / 2 ? r : r - n1, k2 = c < n2 / 2 ? c : c - n2;
    float2 v = make_float2(0.f, 0.f);
    if (k1 >= -N1 / 2 && k1 < N1 / 2 && k2 >= -N2 / 2 && k2 < N2 / 2) {
        const int i = k1 + N1 / 2, j = k2 + N2 / 2;
        const float s = tab[i] * tab[N1 + j];
        const float2 f = F[static_cast<size_t>(i) * N2 + j];
        v = make_float2(f.x * s, f.y * s);
    }
    grid[static_cast<size_t>(r + kHalo) * C + c + kHalo] = v;
}

// Row transform: V[r][c] = sum_j grid[r][j] exp(sign 2 pi i c j / n2) over the
// columns j that hold data (|k2| < N2/2).  One block per data row.
__global__ void k_na_dft_rows(const float2 *__restrict__ grid, float2 *__restrict__ V, int N1, int N2, int n1,
                              int n2, int C, float sign) {
    __shared__ float2 row[kMaxN];
    __shared__ float2 tw[kMaxGrid];
    const int br = blockIdx.x;                          // 0 .. N1-1
    const int r = br < N1 / 2 ? br : n1 - N1 + br;      // FFT row index of data row br
    for (int j = threadIdx.x; j < n2; j += blockDim.x) {
        float s, cth;
        sincospif(2.0f * static_cast<float>(j) / static_cast<float>(n2), &s, &cth);
        tw[j] = make_float2(cth, sign * s);
    }
    for (int jj = threadIdx.x; jj < N2; jj += blockDim.x) {
        const int j = jj < N2 / 2 ? jj : n2 - N2 + jj;
        row[jj] = grid[static_cast<size_t>(r + kHalo) * C + j + kHalo];
    }
    __syncthreads();
    for (int c = threadIdx.x; c < n2; c += blockDim.x) {
        float ax = 0.f, ay = 0.f;
        for (int jj = 0; jj < N2; ++jj) {
            const int j = jj < N2 / 2 ? jj : n2 - N2 + jj;
            const float2 w = tw[(c * j) % n2];
            const float2 u = row[jj];
            ax = fmaf(u.x, w.x, fmaf(-u.y, w.y, ax));
            ay = fmaf(u.x, w.y, fmaf(u.y, w.x, ay));
        }
        V[static_cast<size_t>(r) * n2 + c] = make_float2(ax, ay);
    }
}

// Column transform back onto the grid interior:
// grid[r][c] = sum_i V[i][c] exp(sign 2 pi i r i / n1) over the data rows i.
__global__ void k_na_dft_cols(const float2 *__restrict__ V, float2 *__restrict__ grid, int N1, int n1, int n2,
                              int C, float sign) {
    __shared__ float2 col[kMaxN];
    __shared__ float2 tw[kMaxGrid];
    const int c = blockIdx.x;
    for (int j = threadIdx.x; j < n1; j += blockDim.x) {
        float s, cth;
        sincospif(2.0f * static_cast<float>(j) / static_cast<float>(n1), &s, &cth);
        tw[j] = make_float2(cth, sign * s);
    }
    for (int ii = threadIdx.x; ii < N1; ii += blockDim.x) {
        const int i = ii < N1 / 2 ? ii : n1 - N1 + ii;
        col[ii] = V[static_cast<size_t>(i) * n2 + c];
    }
    __syncthreads();
    for (int r = threadIdx.x; r < n1; r += blockDim.x) {
        float ax = 0.f, ay = 0.f;
        for (int ii = 0; ii < N1; ++ii) {
            const int i = ii < N1 / 2 ? ii : n1 - N1 + ii;
            const float2 w = tw[(r * i) % n1];
            const float2 u = col[ii];
            ax = fmaf(u.x, w.x, fmaf(-u.y, w.y, ax));
            ay = fmaf(u.x, w.y, fmaf(u.y, w.x, ay));
        }
        grid[static_cast<size_t>(r + kHalo) * C + c + kHalo] = make_float2(ax, ay);
    }
}

// Periodic halo of width kHalo around the n1 x n2 interior (rows and columns
// of the padded square beyond the interior are copies of interior cells).
__global__ void k_na_halo(float2 *__restrict__ grid, int n1, int n2, int C) {
    const int R = n1 + 2 * kHalo, Cl = n2 + 2 * kHalo;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < R * Cl; idx += gridDim.x * blockDim.x) {
        const int r = idx / Cl, c = idx - r * Cl;
        if (r >= kHalo && r < kHalo + n1 && c >= kHalo && c < kHalo + n2) continue;
        int sr = (r - kHalo) % n1, sc = (c - kHalo) % n2;
        sr += sr < 0 ? n1 : 0;
        sc += sc < 0 ? n2 : 0;
        grid[static_cast<size_t>(r) * C + c] = grid[static_cast<size_t>(sr + kHalo) * C + sc + kHalo];
    }
}

// Gather without binning: each thread reduces its point's coordinates in FP64
// (v = s x, mu = rint(v) wrapped into [0, n), t = v - mu) and sums its
// (2K+1)^2 taps from the halo-padded grid: FMA row partials, the weighted row
// partials summed with TwoSum and the rounding errors carried in a second
// accumulator, as the plan's gathers do.  A non-finite coordinate yields NaN
// for that point and reads nothing.
template <int K>
__global__ void k_na_gather(const float *__restrict__ x1, const float *__restrict__ x2, int M, double s1,
                            double s2, const float2 *__restrict__ grid, int n1, int n2, int C, float alpha, float cn,
                            float kp, float2 *__restrict__ out) {
    constexpr int W = 2 * K + 1;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= M) return;
    double v1 = static_cast<double>(x1[p]) * s1, v2 = static_cast<double>(x2[p]) * s2;
    if (!isfinite(v1) || !isfinite(v2)) {  // no tap is read for a non-finite point
        out[p] = make_float2(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000));
        return;
    }
    if (fabs(v1) >= 1073741824.0) v1 -= static_cast<double>(n1) * floor(v1 / n1);  // keep rint in range
    if (fabs(v2) >= 1073741824.0) v2 -= static_cast<double>(n2) * floor(v2 / n2);
    const double m1 = rint(v1), m2 = rint(v2);
    long long i1 = static_cast<long long>(m1) % n1, i2 = static_cast<long long>(m2) % n2;
    i1 += i1 < 0 ? n1 : 0;
    i2 += i2 < 0 ? n2 : 0;
    float w1[W], w2[W];
    nfft2d::weights_f32<K>(static_cast<float>(v1 - m1), w1, alpha, cn, kp);
    nfft2d::weights_f32<K>(static_cast<float>(v2 - m2), w2, alpha, cn, kp);
    const float2 *base = grid + static_cast<size_t>(i1 + kHalo - K) * C + (i2 + kHalo - K);
    float sx = 0.f, sy = 0.f, ex = 0.f, ey = 0.f;
#pragma unroll
    for (int a = 0; a < W; ++a) {
        float rx = 0.f, ry = 0.f;
#pragma unroll
        for (int b = 0; b < W; ++b) {
            const float2 u = __ldg(base + static_cast<size_t>(a) * C + b);
            rx = fmaf(w2[b], u.x, rx);
            ry = fmaf(w2[b], u.y, ry);
        }
        float e;
        nfft2d::two_sum(sx, __fmul_rn(w1[a], rx), sx, e);
        ex = __fadd_rn(ex, e);
        nfft2d::two_sum(sy, __fmul_rn(w1[a], ry), sy, e);
        ey = __fadd_rn(ey, e);
    }
    out[p] = make_float2(sx + ex, sy + ey);
}

template <int K>
void launch_gather(const float *x1, const float *x2, int M, double s1, double s2, const float2 *grid, int n1,
                   int n2, int C, float alpha, float cn, float kp, float2 *out, cudaStream_t st) {
    k_na_gather<K><<<(M + 255) / 256, 256, 0, st>>>(x1, x2, M, s1, s2, grid, n1, n2, C, alpha, cn, kp, out);
}

}  // namespace

extern "C" int nfft2d_forward_small_noalloc(int N1, int N2, int K, long long M, const float *x1, const float *x2,
                                            int units, const void *F, void *f, void *stream) {
    if (N1 <= 0 || N2 <= 0 || (N1 & 1) || (N2 & 1)) return NFFT2D_ERR_INVALID_ARG;
    if (K < nfft2d::kMinK || K > nfft2d::kMaxK) return NFFT2D_ERR_INVALID_ARG;
    if (N1 > kMaxN || N2 > kMaxN) return NFFT2D_ERR_SCRATCH_LIMIT;
    const int n1 = static_cast<int>(kSigma * N1), n2 = static_cast<int>(kSigma * N2);
    if (n1 < 2 * K + 2 || n2 < 2 * K + 2) return NFFT2D_ERR_INVALID_ARG;
    if (M < 0 || M > 0x7fffffffLL) return NFFT2D_ERR_INVALID_ARG;
    if (units != NFFT2D_UNITS_GRID && units != NFFT2D_UNITS_UNIT && units != NFFT2D_UNITS_RADIANS)
        return NFFT2D_ERR_INVALID_ARG;
    if (!F || (M > 0 && (!x1 || !x2 || !f))) return NFFT2D_ERR_INVALID_ARG;
    float2 *scratch = nullptr;
    int st = scratch_address(&scratch);
    if (st != NFFT2D_OK) return st;
    if (M == 0) return NFFT2D_OK;

    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int C = n2 + 2 * kHalo;  // pitch of the padded grid inside the scratch
    float2 *grid = scratch;
    float2 *V = scratch + kGridElems;
    float *tab = reinterpret_cast<float *>(scratch + kGridElems + kRowElems);
    const double alpha = (2.0 - 1.0 / kSigma) * kPi - 0.01;  // NFFT1_2D.m:11
    const float cn = static_cast<float>(K / std::sinh(alpha * K));
    const float kp = static_cast<float>(K / (1.0 - std::exp(-2.0 * alpha * K)));
    double u1 = 1.0, u2 = 1.0;
    if (units == NFFT2D_UNITS_UNIT) {
        u1 = N1;
        u2 = N2;
    } else if (units == NFFT2D_UNITS_RADIANS) {
        u1 = N1 / (2.0 * kPi);
        u2 = N2 / (2.0 * kPi);
    }
    const float sign = -1.0f;  // the reference's forward sign (NFFT1_2D.m:55)

    k_na_deap<<<(N1 + N2 + 127) / 128, 128, 0, s>>>(tab, N1, N2, K, alpha);
    k_na_pad<<<dim3((n2 + 127) / 128, n1), 128, 0, s>>>(static_cast<const float2 *>(F), grid, tab, N1, N2, n1, n2, C);
    k_na_dft_rows<<<N1, 256, 0, s>>>(grid, V, N1, N2, n1, n2, C, sign);
    k_na_dft_cols<<<n2, 256, 0, s>>>(V, grid, N1, n1, n2, C, sign);
    k_na_halo<<<64, 256, 0, s>>>(grid, n1, n2, C);
    const int Mi = static_cast<int>(M);
    const double s1 = kSigma * u1, s2 = kSigma * u2;
    float2 *out = static_cast<float2 *>(f);
    switch (K) {
        case 2: launch_gather<2>(x1, x2, Mi, s1, s2, grid, n1, n2, C, static_cast<float>(alpha), cn, kp, out, s); break;
        case 3: launch_gather<3>(x1, x2, Mi, s1, s2, grid, n1, n2, C, static_cast<float>(alpha), cn, kp, out, s); break;
        case 4: launch_gather<4>(x1, x2, Mi, s1, s2, grid, n1, n2, C, static_cast<float>(alpha), cn, kp, out, s); break;
        case 5: launch_gather<5>(x1, x2, Mi, s1, s2, grid, n1, n2, C, static_cast<float>(alpha), cn, kp, out, s); break;
        case 6: launch_gather<6>(x1, x2, Mi, s1, s2, grid, n1, n2, C, static_cast<float>(alpha), cn, kp, out, s); break;
        case 7: launch_gather<7>(x1, x2, Mi, s1, s2, grid, n1, n2, C, static_cast<float>(alpha), cn, kp, out, s); break;
        default: launch_gather<8>(x1, x2, Mi, s1, s2, grid, n1, n2, C, static_cast<float>(alpha), cn, kp, out, s); break;
    }
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? NFFT2D_OK : NFFT2D_ERR_CUDA;
}
