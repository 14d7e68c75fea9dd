// nfft2d_plan.cu -- plan life cycle, point binning (counting sort by tile and
// cell with single-pass look-back scans), the small grid kernels (deapodize+
// pad, halo fill/fold, crop+deapodize: used around cuFFT) and the C ABI entry
// points of libnfft2d_gb300.so.  The oversampled FFT is the fused passes of
// nfft2d_fft.cu for FP32 plans on power-of-two grids below 2048 x 2048 cells
// (use_fused), cuFFT otherwise (run_fft).
//
// Reference path being replaced: NFFT/NFFT2_2D.cu:329-495 (NFFT2_2D_GPU:
// constants, Kernel_Bessel, malloc/memset, Interpolation_NFFT2_2D_GPUKernel,
// fftshift_2D + cufftExecC2C + fftshift_2D, Decimation_and_Scaling) and
// BP_FBP_FFBP/NFFT1_2D.m:1-69 (deapodize + zero-pad, fft2, gather).
#include <cuda.h>
#include <cuda_runtime.h>
#include <cufft.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <cstdlib>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "nfft2d_device.cuh"
#include "nfft2d_internal.h"

using namespace nfft2d;

// I0 by its power series (Abramowitz & Stegun 9.6.12); all terms positive.
double nfft2d::bessel_i0_host(double x) {
    const double q = 0.25 * x * x;
    double term = 1.0, sum = 1.0;
    for (int j = 1; j < 500; ++j) {
        term *= q / (static_cast<double>(j) * j);
        sum += term;
        if (term < 1e-18 * sum) break;
    }
    return sum;
}

// S / phi(xi_k) for k = i - N/2, i < N: S = sinh(alpha K)/(pi K) (the window
// normalisation), phi(xi) = I0(K sqrt(alpha^2 - xi^2)), xi_k = 2 pi k / n
// (NFFT1_2D.m:17-22, NFFT2_2D.cu:60-69).
void nfft2d::deapod_table_host(int N, int n, int K, double alpha, double *out) {
    const double pi = 3.141592653589793238462643383279502884;
    const double S = std::sinh(alpha * K) / (pi * K);
    for (int i = 0; i < N; ++i) {
        const double xi = 2.0 * pi * (i - N / 2) / n;
        out[i] = S / bessel_i0_host(K * std::sqrt(alpha * alpha - xi * xi));
    }
}

double nfft2d::fit_window_poly(double sigma, int K, WinPoly *out) {
    if (!out || K < kMinK || K > kMaxK || !(sigma >= 1.0) || !std::isfinite(sigma)) return -1.0;
    const double pi = 3.141592653589793238462643383279502884;
    const double alpha = (2.0 - 1.0 / sigma) * pi - 0.01;
    const double cn = K / std::sinh(alpha * K);
    // the normalised window, closed form with both branches
    auto win = [&](double u) {
        const double P = (K - u) * (K + u);
        const double s = std::sqrt(std::fabs(P));
        if (s == 0.0) return cn * alpha;
        return cn * (P > 0 ? std::sinh(alpha * s) : std::sin(alpha * s)) / s;
    };
    const int D = poly_degree(K), n = D + 1;
    std::memset(out, 0, sizeof(*out));
    double maxerr = 0.0;
    for (int a = 0; a <= 2 * K; ++a) {
        const int m = a - K;
        // interpolate at the Chebyshev nodes of [-1/2, 1/2]: Vandermonde
        // system, Gaussian elimination with partial pivoting
        double A[kPolyCoef][kPolyCoef + 1];
        for (int i = 0; i < n; ++i) {
            const double t = 0.5 * std::cos(pi * (i + 0.5) / n);
            double pw = 1.0;
            for (int j = 0; j < n; ++j) {
                A[i][j] = pw;
                pw *= t;
            }
            A[i][n] = win(t - m);
        }
        for (int col = 0; col < n; ++col) {
            int piv = col;
            for (int r = col + 1; r < n; ++r)
                if (std::fabs(A[r][col]) > std::fabs(A[piv][col])) piv = r;
            if (piv != col)
                for (int j = 0; j <= n; ++j) std::swap(A[col][j], A[piv][j]);
            for (int r = col + 1; r < n; ++r) {
                const double f = A[r][col] / A[col][col];
                for (int j = col; j <= n; ++j) A[r][j] -= f * A[col][j];
            }
        }
        double c[kPolyCoef];
        for (int i = n - 1; i >= 0; --i) {
            double v = A[i][n];
            for (int j = i + 1; j < n; ++j) v -= A[i][j] * c[j];
            c[i] = v / A[i][i];
        }
        for (int q = 0; q <= 1000; ++q) {
            const double t = -0.5 + q / 1000.0;
            double v = c[D];
            for (int d = D - 1; d >= 0; --d) v = v * t + c[d];
            maxerr = std::max(maxerr, std::fabs(v - win(t - m)));
        }
        for (int d = 0; d < n; ++d) out->c[d][a] = static_cast<float>(c[d]);
    }
    return maxerr;
}

namespace {
// The fitted window of every (sigma, K) a process has used: plans of the same
// window (every regridding of an FFBP image, every transform of a batch)
// share one fit instead of refitting on each plan creation.
struct PolyCacheEntry {
    double sigma;
    int K;
    double err;
    nfft2d::WinPoly poly;
};
std::mutex g_poly_mu;
std::vector<PolyCacheEntry> g_poly_cache;

double cached_window_poly(double sigma, int K, nfft2d::WinPoly *out) {
    {
        std::lock_guard<std::mutex> lock(g_poly_mu);
        for (const auto &e : g_poly_cache)
            if (e.sigma == sigma && e.K == K) {
                *out = e.poly;
                return e.err;
            }
    }
    const double err = nfft2d::fit_window_poly(sigma, K, out);
    if (err >= 0.0) {
        std::lock_guard<std::mutex> lock(g_poly_mu);
        if (g_poly_cache.size() < 64) g_poly_cache.push_back({sigma, K, err, *out});
    }
    return err;
}
}  // namespace

// Device allocations of a plan.  For tests of the host-side failure paths,
// NFFT2D_FAIL_ALLOC_AT=k makes the k-th allocation (counted from the moment
// the variable takes that value) report cudaErrorMemoryAllocation without
// allocating; unset, it is one getenv per allocation (plan creation and
// set_points only, never per transform).
// NFFT2D_FAIL_ALLOC_AT=k: the k-th plan allocation (device or pinned host,
// counted since the variable last changed) fails.
static bool injected_alloc_failure() {
    static std::mutex mu;
    static std::string seen;
    static long long count = 0;
    const char *v = std::getenv("NFFT2D_FAIL_ALLOC_AT");
    if (!v || !*v) return false;
    std::lock_guard<std::mutex> lock(mu);
    if (seen != v) {
        seen = v;
        count = 0;
    }
    return ++count == std::atoll(v);
}

// Plan buffers come from a process-wide cache of freed device blocks: a
// cudaMalloc / cudaFree pair costs ~0.06-0.09 ms on GB300 and cudaFree waits
// for the whole device, while callers that make and drop plans (the FFBP
// recursion: two plans and a regridder per node) reuse the same sizes.  A
// request takes the smallest cached block of at least its size and at most
// twice it, on the current device; freed blocks are kept up to 1 GiB, the
// oldest released first.
// Callers return a block only once no work of theirs that uses it is in
// flight (they synchronize the stream first).
namespace {
constexpr size_t kBlockCacheBytes = size_t(1) << 30;
struct CachedBlock {
    void *p;
    size_t bytes;
    int device;
    unsigned long long age;
};
std::mutex g_blk_mu;
std::vector<CachedBlock> g_blk_free;  // released blocks
std::vector<CachedBlock> g_blk_live;  // blocks handed out
size_t g_blk_free_bytes = 0;
unsigned long long g_blk_clock = 0;
}  // namespace

cudaError_t nfft2d::plan_malloc(void **ptr, size_t bytes) {
    if (injected_alloc_failure()) {
        *ptr = nullptr;
        return cudaErrorMemoryAllocation;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    {
        std::lock_guard<std::mutex> lock(g_blk_mu);
        size_t best = g_blk_free.size();
        for (size_t i = 0; i < g_blk_free.size(); ++i)
            if (g_blk_free[i].device == dev && g_blk_free[i].bytes >= bytes && g_blk_free[i].bytes <= 2 * bytes + 4096 &&
                (best == g_blk_free.size() || g_blk_free[i].bytes < g_blk_free[best].bytes))
                best = i;
        if (best < g_blk_free.size()) {
            const CachedBlock b = g_blk_free[best];
            g_blk_free.erase(g_blk_free.begin() + static_cast<long>(best));
            g_blk_free_bytes -= b.bytes;
            g_blk_live.push_back(b);
            *ptr = b.p;
            return cudaSuccess;
        }
    }
    const cudaError_t e = cudaMalloc(ptr, bytes);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(g_blk_mu);
    g_blk_live.push_back({*ptr, bytes, dev, 0});
    return cudaSuccess;
}

void nfft2d::plan_free(void *ptr) {
    if (!ptr) return;
    std::vector<void *> drop;
    {
        std::lock_guard<std::mutex> lock(g_blk_mu);
        size_t i = 0;
        while (i < g_blk_live.size() && g_blk_live[i].p != ptr) ++i;
        if (i == g_blk_live.size()) {
            drop.push_back(ptr);  // not from plan_malloc
        } else {
            CachedBlock b = g_blk_live[i];
            g_blk_live.erase(g_blk_live.begin() + static_cast<long>(i));
            b.age = ++g_blk_clock;
            g_blk_free.push_back(b);
            g_blk_free_bytes += b.bytes;
            while (g_blk_free_bytes > kBlockCacheBytes && !g_blk_free.empty()) {
                size_t old = 0;
                for (size_t j = 1; j < g_blk_free.size(); ++j)
                    if (g_blk_free[j].age < g_blk_free[old].age) old = j;
                drop.push_back(g_blk_free[old].p);
                g_blk_free_bytes -= g_blk_free[old].bytes;
                g_blk_free.erase(g_blk_free.begin() + static_cast<long>(old));
            }
        }
    }
    for (void *d : drop) cudaFree(d);
}

// Page-locked status words: 16-byte slots cut from 4 KB page-locked blocks
// that live as long as the process (a page-locked allocation costs ~0.25 ms
// on GB300; plans that come and go -- the FFBP recursion makes over a
// hundred per image -- take a slot instead).  Requests above one slot are
// plain page-locked allocations.
namespace {
constexpr size_t kSlotBytes = 16, kSlotBlock = 4096;
std::mutex g_slot_mu;
std::vector<void *> g_slot_free;
}  // namespace

cudaError_t nfft2d::plan_malloc_host(void **ptr, size_t bytes) {
    if (injected_alloc_failure()) {
        *ptr = nullptr;
        return cudaErrorMemoryAllocation;
    }
    if (bytes > kSlotBytes) return cudaMallocHost(ptr, bytes);
    std::lock_guard<std::mutex> lock(g_slot_mu);
    if (g_slot_free.empty()) {
        void *blk = nullptr;
        const cudaError_t e = cudaMallocHost(&blk, kSlotBlock);
        if (e != cudaSuccess) {
            *ptr = nullptr;
            return e;
        }
        for (size_t o = 0; o < kSlotBlock; o += kSlotBytes) g_slot_free.push_back(static_cast<char *>(blk) + o);
    }
    *ptr = g_slot_free.back();
    g_slot_free.pop_back();
    return cudaSuccess;
}

void nfft2d::plan_free_host(void *ptr, size_t bytes) {
    if (!ptr) return;
    if (bytes > kSlotBytes) {
        cudaFreeHost(ptr);
        return;
    }
    std::lock_guard<std::mutex> lock(g_slot_mu);
    g_slot_free.push_back(ptr);
}

namespace {

constexpr double kPi = 3.141592653589793238462643383279502884;

// The fused FFT passes (nfft2d_fft.cu) serve FP32 plans on power-of-two
// grids: by default below 2048 x 2048 oversampled cells, where they beat
// cuFFT with the separate pad / fill / fold / crop kernels on GB300 (both
// directions at 1024^2: 51 vs 71 us; 2048^2: 110 vs 108 us for the pruned
// cuFFT passes; 4096^2: 421 vs 292 us, the column passes then holding one
// column per CTA), or whenever fft_mode 2 asks for them.
bool use_fused(const nfft2d_plan_s *p) {
    if (!p->fused_ok) return false;
    if (p->fft_mode == 2) return true;
    return p->fft_mode < 0 && 1LL * p->g.n1 * p->g.n2 < 2048LL * 2048LL;
}

// The automatic FP32 gather: the direct 16-byte-load gather from 128 points
// per 16 x 16 tile or 2^18 points up, the TMA-tiled patches for small, thin
// point sets.  Measured on GB300: tiled for 4096 points on 64^2
// coefficients (the autotuner's pick, 64 points per tile); direct 13 %
// faster at 256 points per tile (polar raster, uniform and clustered sets)
// and 16 % faster for the Knab regridding's 4 M outputs at 64 per tile.
int auto_gather(const nfft2d_plan_s *p, long long M) {
    const long long tiles = static_cast<long long>(p->g.tiles1) * p->g.tiles2;
    return (M >= 128 * tiles || M >= (1LL << 18)) ? NFFT2D_VARIANT_DIRECT : NFFT2D_VARIANT_TILED;
}

int fft_mode_in_use(const nfft2d_plan_s *p) {
    if (use_fused(p)) return 2;
    const bool pruned = p->fft_mode == 1 || (p->fft_mode < 0 && 1LL * p->g.n1 * p->g.n2 >= 2048LL * 2048LL);
    return pruned && p->pruned_ok ? 1 : 0;
}

// ---------------------------------------------------------------------------
// host math (plan time, FP64)
// ---------------------------------------------------------------------------


int status_from_cuda(cudaError_t e) {
    if (e == cudaSuccess) return NFFT2D_OK;
    if (e == cudaErrorMemoryAllocation) return NFFT2D_ERR_OOM;
    return NFFT2D_ERR_CUDA;
}

int status_from_cufft(cufftResult r) {
    if (r == CUFFT_SUCCESS) return NFFT2D_OK;
    if (r == CUFFT_ALLOC_FAILED) return NFFT2D_ERR_OOM;
    return NFFT2D_ERR_CUFFT;
}

#define NFFT_TRY_CUDA(expr)                                  \
    do {                                                     \
        cudaError_t e_ = (expr);                             \
        if (e_ != cudaSuccess) return status_from_cuda(e_);  \
    } while (0)

size_t real_size(int precision) { return precision == NFFT2D_F64 ? sizeof(double) : sizeof(float); }
size_t cplx_size(int precision) { return 2 * real_size(precision); }
size_t rec_size(int precision) { return precision == NFFT2D_F64 ? sizeof(Rec64) : sizeof(Rec32); }

// ---------------------------------------------------------------------------
// stage timing
// ---------------------------------------------------------------------------
enum Stage { ST_SORT = 0, ST_PAD, ST_FFT2, ST_FILL, ST_GATHER, ST_SPREAD, ST_FOLD, ST_FFT1, ST_CROP, ST_COUNT };
static_assert(ST_COUNT == kStages, "stage count");

// Every stage is also an NVTX range on the host thread that enqueues it
// (nfft2d:<stage>), so a system trace shows the library's calls; without a
// tool attached the NVTX calls do nothing.
const char *const kStageNames[ST_COUNT] = {"nfft2d:sort", "nfft2d:pad", "nfft2d:fft_type2", "nfft2d:halo_fill",
                                           "nfft2d:gather", "nfft2d:spread", "nfft2d:fold", "nfft2d:fft_type1",
                                           "nfft2d:crop"};
void stage_begin(nfft2d_plan_s *p, Stage s) {
    p->timer.nvtx[s] = nvtxRangeStartA(kStageNames[s]);
    if (!p->timer.on) return;
    cudaEventRecord(p->timer.ev[2 * s], p->stream);
    p->timer.used[s] = true;
}
void stage_end(nfft2d_plan_s *p, Stage s) {
    nvtxRangeEnd(p->timer.nvtx[s]);
    if (!p->timer.on) return;
    cudaEventRecord(p->timer.ev[2 * s + 1], p->stream);
}
// Forget the stages a call of this kind is about to re-run.
enum CallKind { CALL_SORT, CALL_TYPE2, CALL_TYPE1 };
void timer_reset(nfft2d_plan_s *p, CallKind k) {
    static const Stage sort_st[] = {ST_SORT};
    static const Stage t2_st[] = {ST_PAD, ST_FFT2, ST_FILL, ST_GATHER};
    static const Stage t1_st[] = {ST_SPREAD, ST_FOLD, ST_FFT1, ST_CROP};
    if (k == CALL_SORT) for (Stage s : sort_st) p->timer.used[s] = false;
    if (k == CALL_TYPE2) for (Stage s : t2_st) p->timer.used[s] = false;
    if (k == CALL_TYPE1) for (Stage s : t1_st) p->timer.used[s] = false;
}

// ---------------------------------------------------------------------------
// TMA descriptor (driver entry point fetched through the runtime, so the
// library does not link libcuda directly)
// ---------------------------------------------------------------------------
using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn get_encode_tiled() {
    static EncodeTiledFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *ptr = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(ptr);
    }
    return fn;
}

// The padded grid seen as a 2D FP32 tensor: Ra rows, 2*C floats per row.  One
// box is a tile patch: PR rows x 2*PC floats; the allocation is a whole number
// of tiles plus the halo on each side, so every box lies inside it.
int make_tensor_map(nfft2d_plan_s *p) {
    EncodeTiledFn enc = get_encode_tiled();
    if (!enc) return NFFT2D_ERR_CUDA;
    const Geom &g = p->g;
    cuuint64_t dims[2] = {static_cast<cuuint64_t>(2 * g.C), static_cast<cuuint64_t>(g.Ra)};
    cuuint64_t strides[1] = {static_cast<cuuint64_t>(2 * g.C) * sizeof(float)};
    cuuint32_t box[2] = {static_cast<cuuint32_t>(2 * g.PC), static_cast<cuuint32_t>(g.PR)};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(&p->tmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, p->grid, dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return NFFT2D_ERR_CUDA;
    // the spread's strip patch: G lane columns (+2 for odd K, whose patch
    // starts one column early to keep the box on a 16-byte boundary)
    const int K = (g.PR - g.T) / 2;
    cuuint32_t sbox[2] = {static_cast<cuuint32_t>(2 * (spread_group_lanes(K) + 2 * (K & 1))),
                          static_cast<cuuint32_t>(g.PR)};
    r = enc(&p->tmap_spread, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, p->grid, dims, strides, sbox, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return NFFT2D_ERR_CUDA;
    p->tmap_ok = true;
    return NFFT2D_OK;
}

// ---------------------------------------------------------------------------
// device kernels: deapodize + zero-pad, crop + deapodize, halo fill / fold
// ---------------------------------------------------------------------------
template <typename Cx, typename Rl>
__global__ void k_pad(const Cx *__restrict__ F, Cx *__restrict__ grid, const Rl *__restrict__ d1,
                      const Rl *__restrict__ d2, int N1, int N2, int n1, int n2, int H, int C) {
    // One row r of the oversampled grid per blockIdx.y.  FFT index r holds
    // frequency k1 = r (r < n1/2) or r - n1: the ifftshift of NFFT1_2D.m:55
    // applied to the centered zero-padded block of NFFT1_2D.m:48-49.
    const int r = blockIdx.y;
    const int k1 = (r < n1 / 2) ? r : r - n1;
    const bool row_in = (k1 >= -N1 / 2) && (k1 < N1 / 2);
    const int i = k1 + N1 / 2;
    const Rl s1 = row_in ? d1[i] : Rl(0);
    Cx *dst = grid + static_cast<size_t>(r + H) * C + H;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n2; c += gridDim.x * blockDim.x) {
        const int k2 = (c < n2 / 2) ? c : c - n2;
        Cx v;
        v.x = Rl(0);
        v.y = Rl(0);
        if (row_in && k2 >= -N2 / 2 && k2 < N2 / 2) {
            const int j = k2 + N2 / 2;
            const Rl s = s1 * d2[j];
            const Cx f = F[static_cast<size_t>(i) * N2 + j];
            v.x = f.x * s;
            v.y = f.y * s;
        }
        dst[c] = v;
    }
}

// FP32 pad with two cells per thread and one 16-byte store (grid rows start
// on 16-byte boundaries: the pitch and the halo are even).  Same mapping as
// k_pad.
__global__ void k_pad_f32x2(const float2 *__restrict__ F, float2 *__restrict__ grid, const float *__restrict__ d1,
                            const float *__restrict__ d2, int N1, int N2, int n1, int n2, int H, int C) {
    const int r = blockIdx.y;
    const int k1 = (r < n1 / 2) ? r : r - n1;
    const bool row_in = (k1 >= -N1 / 2) && (k1 < N1 / 2);
    const int i = k1 + N1 / 2;
    const float s1 = row_in ? d1[i] : 0.f;
    const float2 *Fr = F + static_cast<size_t>(row_in ? i : 0) * N2;
    float4 *dst = reinterpret_cast<float4 *>(grid + static_cast<size_t>(r + H) * C + H);
    const int pairs = n2 >> 1;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < pairs; q += gridDim.x * blockDim.x) {
        float2 v[2];
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const int c = 2 * q + e;
            const int k2 = (c < n2 / 2) ? c : c - n2;
            v[e] = make_float2(0.f, 0.f);
            if (row_in && k2 >= -N2 / 2 && k2 < N2 / 2) {
                const int j = k2 + N2 / 2;
                const float s = s1 * d2[j];
                const float2 f = Fr[j];
                v[e] = make_float2(f.x * s, f.y * s);
            }
        }
        dst[q] = make_float4(v[0].x, v[0].y, v[1].x, v[1].y);
    }
}

template <typename Cx, typename Rl>
__global__ void k_crop(const Cx *__restrict__ grid, Cx *__restrict__ F, const Rl *__restrict__ d1,
                       const Rl *__restrict__ d2, int N1, int N2, int n1, int n2, int H, int C) {
    // Decimation_and_Scaling (NFFT2_2D.cu:74-100, NFFT2_2D.m:70): keep
    // frequencies [-N/2, N/2) and multiply by the deapodization table.  The
    // fftshift pair around the FFT (NFFT2_2D.cu:383,393) is folded into the
    // index map k -> k mod n.
    const int i = blockIdx.y;
    const int k1 = i - N1 / 2;
    const int r = k1 < 0 ? k1 + n1 : k1;
    const Rl s1 = d1[i];
    const Cx *src = grid + static_cast<size_t>(r + H) * C + H;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < N2; j += gridDim.x * blockDim.x) {
        const int k2 = j - N2 / 2;
        const int c = k2 < 0 ? k2 + n2 : k2;
        const Rl s = s1 * d2[j];
        const Cx g = src[c];
        Cx v;
        v.x = g.x * s;
        v.y = g.y * s;
        F[static_cast<size_t>(i) * N2 + j] = v;
    }
}

__device__ __forceinline__ int pmod(int a, int n) {
    int r = a % n;
    return r < 0 ? r + n : r;
}

// Fill the periodic halo of the padded grid from the interior (type 2, after
// the FFT), so a tile patch never needs index wrapping.
template <typename Cx>
__global__ void k_halo_fill(Cx *__restrict__ grid, int n1, int n2, int H, int C) {
    const long long top = 2LL * H * C;
    const long long side = 2LL * H * n1;
    for (long long idx = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; idx < top + side;
         idx += static_cast<long long>(gridDim.x) * blockDim.x) {
        int r, c;
        if (idx < top) {
            const int rr = static_cast<int>(idx / C);
            c = static_cast<int>(idx - static_cast<long long>(rr) * C);
            r = rr < H ? rr : rr + n1;
        } else {
            const long long j = idx - top;
            r = H + static_cast<int>(j / (2 * H));
            const int cc = static_cast<int>(j - static_cast<long long>(r - H) * 2 * H);
            c = cc < H ? cc : cc + n2;
        }
        const int sr = pmod(r - H, n1) + H, sc = pmod(c - H, n2) + H;
        grid[static_cast<size_t>(r) * C + c] = grid[static_cast<size_t>(sr) * C + sc];
    }
}

// Fold the halo back onto the interior (type 1, after spreading): every
// interior cell within H of an edge adds all of its periodic images that lie
// in the padded grid.  Each such cell is owned by one thread; halo cells are
// only read, so no atomics are needed.
template <typename Cx>
__global__ void k_halo_fold(Cx *__restrict__ grid, int n1, int n2, int H, int R, int Cl, int C) {
    const int rows_tb = (n1 <= 2 * H) ? n1 : 2 * H;
    const int cols_lr = (n2 <= 2 * H) ? n2 : 2 * H;
    const long long part1 = static_cast<long long>(rows_tb) * n2;
    const long long part2 = (n1 > 2 * H) ? static_cast<long long>(n1 - 2 * H) * cols_lr : 0;
    for (long long idx = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; idx < part1 + part2;
         idx += static_cast<long long>(gridDim.x) * blockDim.x) {
        int r, c;
        if (idx < part1) {
            const int rr = static_cast<int>(idx / n2);
            c = static_cast<int>(idx - static_cast<long long>(rr) * n2);
            r = (n1 <= 2 * H) ? rr : (rr < H ? rr : n1 - 2 * H + rr);
        } else {
            const long long j = idx - part1;
            const int rr = static_cast<int>(j / cols_lr);
            const int cc = static_cast<int>(j - static_cast<long long>(rr) * cols_lr);
            r = H + rr;
            c = (n2 <= 2 * H) ? cc : (cc < H ? cc : n2 - 2 * H + cc);
        }
        // images at padded (r + H + a*n1, c + H + b*n2), (a, b) != (0, 0)
        const int pr0 = r + H, pc0 = c + H;
        const int amin = -((pr0) / n1), amax = (R - 1 - pr0) / n1;
        const int bmin = -((pc0) / n2), bmax = (Cl - 1 - pc0) / n2;
        auto acc = grid[static_cast<size_t>(pr0) * C + pc0];
        for (int a = amin; a <= amax; ++a)
            for (int b = bmin; b <= bmax; ++b) {
                if (a == 0 && b == 0) continue;
                const auto v = grid[static_cast<size_t>(pr0 + a * n1) * C + (pc0 + b * n2)];
                acc.x += v.x;
                acc.y += v.y;
            }
        grid[static_cast<size_t>(pr0) * C + pc0] = acc;
    }
}

// ---------------------------------------------------------------------------
// binning: per point cell key, counting sort by key, work items per tile
// ---------------------------------------------------------------------------
// Wrap an integer-valued grid index into [0, n).
__device__ __forceinline__ int wrap_index(long long m, int n) {
    long long r = m % n;
    return static_cast<int>(r < 0 ? r + n : r);
}

// Reduction of one coordinate: v = (x - o) * s (s = sigma * unit scale, o an
// origin, 0 for the plain transforms), mu = rint(v) wrapped into [0, n),
// t = v - mu in [-1/2, 1/2] (NFFT2_2D.cu:167-173 does the same in the data
// precision).  FP32 coordinates with a power-of-two scale and no origin take
// an exact FP32 path (the product, rint and the difference are all exact);
// everything else -- including a finite coordinate whose FP32 product is too
// large for that path -- is reduced in FP64.  Only a non-finite coordinate is
// rejected.
template <typename CT, typename TT>
__device__ __forceinline__ bool reduce_coord(CT x, double o, double s, float sf, bool exact_f32, int n, int &mu,
                                             TT &t) {
    if (exact_f32) {
        const float v = static_cast<float>(x) * sf;
        if (isfinite(v) && fabsf(v) < 1073741824.0f) {
            const float m = rintf(v);
            t = static_cast<TT>(v - m);
            mu = wrap_index(static_cast<long long>(m), n);
            return true;
        }
    }
    double v = (static_cast<double>(x) - o) * s;
    if (!isfinite(v)) return false;
    if (fabs(v) >= 1073741824.0) v -= static_cast<double>(n) * floor(v / n);  // keep the integer part in range
    const double m = rint(v);
    t = static_cast<TT>(v - m);
    mu = wrap_index(static_cast<long long>(m), n);
    return true;
}

// Cell key of wrapped cell (mu1, mu2): tile, then strip, row and column
// within the strip (row-major within the tile when the strip width is the
// tile's).
__device__ __forceinline__ unsigned cell_key(const Geom &g, int mu1, int mu2) {
    const int tr = mu1 / g.T, tc = mu2 / g.T;
    const int lr = mu1 - tr * g.T, lc = mu2 - tc * g.T;
    const int st = lc / g.SW, sc = lc - st * g.SW;
    return static_cast<unsigned>(tr * g.tiles2 + tc) * static_cast<unsigned>(g.T * g.T) +
           static_cast<unsigned>((st * g.T + lr) * g.SW + sc);
}

// Loads and stores of arrays that each binning pass streams through once.
// STREAM (set when the binning's arrays exceed L2): evict-first hints, so
// that the tables the passes hit at random -- the cell counters and starts,
// the inverse permutation -- stay in L2; else plain accesses, so that what
// one pass writes is still in L2 for the next.
template <bool STREAM, typename T>
__device__ __forceinline__ T ld_once(const T *p) {
    if constexpr (STREAM) return __ldcs(p);
    else return *p;
}
template <bool STREAM, typename T>
__device__ __forceinline__ void st_once(T *p, const T &v) {
    if constexpr (STREAM) __stcs(p, v);
    else *p = v;
}
template <bool STREAM, typename RecT>
__device__ __forceinline__ void st_rec(RecT *p, const RecT &r) {
    if constexpr (STREAM && sizeof(RecT) == 16)
        __stcs(reinterpret_cast<int4 *>(p), *reinterpret_cast<const int4 *>(&r));
    else
        *p = r;
}

template <typename CT, typename RecT, bool STREAM>
__global__ void k_bin_pass1(const CT *__restrict__ x1, const CT *__restrict__ x2, int M, double o1, double o2,
                            double s1, double s2, float s1f, float s2f, int exact_f32, Geom g, RecT *__restrict__ tmp,
                            uint2 *__restrict__ keyrank, unsigned *__restrict__ cell_count,
                            int *__restrict__ status, unsigned long long *__restrict__ scan_state,
                            int scan_words) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    // the two scans that follow start from zeroed tickets and tile words
    for (int k = i; k < scan_words; k += gridDim.x * blockDim.x) scan_state[k] = 0ull;
    if (i >= M) return;
    RecT r;
    int mu1, mu2;
    const bool ok1 = reduce_coord(ld_once<STREAM>(x1 + i), o1, s1, s1f, exact_f32 != 0, g.n1, mu1, r.t1);
    const bool ok2 = reduce_coord(ld_once<STREAM>(x2 + i), o2, s2, s2f, exact_f32 != 0, g.n2, mu2, r.t2);
    if (!ok1 || !ok2) {
        // the error is reported; the point is still binned (at cell 0, t = 0)
        // so every sorted record stays in bounds for transforms that an
        // asynchronous set_points lets run before the status is read
        latch_error(status, kErrNonfinite);
        mu1 = mu2 = 0;
        r.t1 = r.t2 = 0;
    }
    const unsigned key = cell_key(g, mu1, mu2);
    const unsigned rank = atomicAdd(cell_count + key, 1u);
    r.mu = (mu1 << 16) | mu2;
    r.orig = i;
    st_rec<STREAM>(tmp + i, r);
    st_once<STREAM>(keyrank + i, make_uint2(key, rank));
}

// The sorted position of every point, inverted: src[cell_start[key] + rank]
// = i.  The 4-byte writes land in an array a quarter of the records' size,
// which stays in L2 where the writes merge into whole lines.
template <bool STREAM>
__global__ void k_bin_invert(const uint2 *__restrict__ keyrank, const unsigned *__restrict__ cell_start, int M,
                             int *__restrict__ src) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M) return;
    const uint2 kr = ld_once<STREAM>(keyrank + i);
    src[cell_start[kr.x] + kr.y] = i;
}

// recs[p] = tmp[src[p]]: the records move to their sorted positions as
// random reads and coalesced writes (a scatter of the 16-byte records would
// write half sectors at random addresses of an array larger than L2).
template <typename RecT, bool STREAM>
__global__ void k_bin_gather(const RecT *__restrict__ tmp, const int *__restrict__ src, int M,
                             RecT *__restrict__ recs) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= M) return;
    st_rec<STREAM>(recs + q, tmp[ld_once<STREAM>(src + q)]);
}

// ---------------------------------------------------------------------------
// Binning of many small point sets at once (the transforms of a batch): one
// 1024-thread CTA per transform does the whole counting sort with its cell
// counters in shared memory -- reduction, key and rank (shared atomics),
// scan, ordered records, work items -- so a batch of hundreds of small
// transforms bins in one launch instead of five launches and two memsets
// each.  Same records, keys and work items as the per-plan binning.
// ---------------------------------------------------------------------------
constexpr int kSmallBinThreads = 1024;

// Exclusive block-wide scan of one value per thread; *total gets the sum.
__device__ unsigned small_block_scan(unsigned v, unsigned *warp_sums, unsigned *total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        unsigned w = warp_sums[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned u = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += u;
        }
        warp_sums[lane] = w;
    }
    __syncthreads();
    const unsigned excl = (warp ? warp_sums[warp - 1] : 0u) + incl - v;
    if (total) *total = warp_sums[31];
    __syncthreads();  // warp_sums reusable
    return excl;
}

template <typename CT>
__global__ void __launch_bounds__(kSmallBinThreads, 1) k_bin_small(const SmallBinJob *__restrict__ jobs) {
    extern __shared__ unsigned sb_smem[];
    const SmallBinJob J = jobs[blockIdx.x];
    const Geom &g = J.g;
    const int ncells = g.tiles1 * g.tiles2 * g.T * g.T;
    unsigned *cnt = sb_smem;                 // ncells + 1 counters, then the exclusive starts
    unsigned *ws = sb_smem + ncells + 1;     // 32 warp sums
    const int tid = threadIdx.x;
    for (int i = tid; i <= ncells; i += kSmallBinThreads) cnt[i] = 0u;
    if (tid < 4) J.status[tid] = 0;  // a new point set: no work items, no error bits
    __syncthreads();
    const CT *x1 = static_cast<const CT *>(J.x1), *x2 = static_cast<const CT *>(J.x2);
    bool bad = false;
    for (int i = tid; i < J.M; i += kSmallBinThreads) {
        Rec32 r;
        int mu1, mu2;
        const bool ok1 = reduce_coord(x1[i], 0.0, J.s1, J.s1f, J.exact != 0, g.n1, mu1, r.t1);
        const bool ok2 = reduce_coord(x2[i], 0.0, J.s2, J.s2f, J.exact != 0, g.n2, mu2, r.t2);
        if (!ok1 || !ok2) {  // as k_bin_pass1: reported, and binned at cell 0 with t = 0
            bad = true;
            mu1 = mu2 = 0;
            r.t1 = r.t2 = 0.f;
        }
        const unsigned key = cell_key(g, mu1, mu2);
        r.mu = (mu1 << 16) | mu2;
        r.orig = i;
        J.tmp[i] = r;
        J.keyrank[i] = make_uint2(key, atomicAdd(cnt + key, 1u));
    }
    if (bad) atomicOr(J.status + 1, kErrNonfinite);
    __syncthreads();
    // exclusive scan of the counters: each thread sums a contiguous run
    const int per = (ncells + 1 + kSmallBinThreads - 1) / kSmallBinThreads;
    const int c0 = min(tid * per, ncells + 1), c1 = min(c0 + per, ncells + 1);
    unsigned run = 0;
    for (int c = c0; c < c1; ++c) run += cnt[c];
    unsigned base = small_block_scan(run, ws, nullptr);
    for (int c = c0; c < c1; ++c) {
        const unsigned v = cnt[c];
        cnt[c] = base;
        base += v;
    }
    __syncthreads();
    // records in cell order and the permutation
    for (int i = tid; i < J.M; i += kSmallBinThreads) {
        const uint2 kr = J.keyrank[i];
        const unsigned q = cnt[kr.x] + kr.y;
        J.recs[q] = J.tmp[i];
        J.src[q] = i;
    }
    // work items: per tile, ceil(count / chunk) items of at most chunk points
    const int ntiles = g.tiles1 * g.tiles2, cpt = g.T * g.T;
    unsigned items_before = 0;
    for (int t0 = 0; t0 < ntiles; t0 += kSmallBinThreads) {
        const int t = t0 + tid;
        unsigned start = 0, count = 0, items = 0;
        if (t < ntiles) {
            start = cnt[t * cpt];
            count = cnt[(t + 1) * cpt] - start;  // cnt[ncells] is M
            items = (count + J.chunk - 1) / J.chunk;
        }
        unsigned total = 0;
        const unsigned at = items_before + small_block_scan(items, ws, &total);
        for (unsigned c = 0; c < items; ++c) {
            const unsigned off = c * J.chunk;
            J.chunks[at + c] = make_int4(t, static_cast<int>(start + off),
                                         static_cast<int>(min(count - off, static_cast<unsigned>(J.chunk))), 0);
        }
        items_before += total;
    }
    if (tid == 0) {
        J.status[0] = static_cast<int>(items_before);
        J.out[0] = static_cast<int>(items_before);
    }
    __syncthreads();
    if (tid == 0) J.out[1] = J.status[1];
}

// ---------------------------------------------------------------------------
// single-pass exclusive scans (decoupled look-back)
// ---------------------------------------------------------------------------
// Blocks take tiles of consecutive counters in launch order from a ticket
// counter, scan them locally, publish the tile's aggregate, then look back
// over the predecessors' published words -- 32 at a time, one per lane of
// the first warp -- until one carries its inclusive prefix.  A tile only
// waits on tiles whose blocks took earlier tickets (already running), and
// every wait is bounded: a lane that gives up latches kErrTimeout and counts
// the missing value as 0, so the host sees an error status instead of a
// hang.  One launch replaces the three-phase reduce / scan-of-sums / apply
// sequence.
constexpr int kCellScanThreads = 512, kCellScanItems = 8;  // 4096 cell counters per tile
constexpr int kItemScanThreads = 128, kItemScanItems = 1;  // 128 bin tiles per tile
constexpr unsigned long long kTileAggregate = 1ull << 32;
constexpr unsigned long long kTilePrefix = 2ull << 32;

// Scan state for one scan over n counters in tiles of `tile_elems`: a ticket
// counter (as a 64-bit word) followed by one status word per tile.
size_t scan_state_words(size_t n, int tile_elems) { return 1 + (n + tile_elems - 1) / tile_elems; }

// The exclusive offset of this tile among all tiles; `agg` is the tile's own
// sum.  Called by all lanes of warp 0; the result is valid in every lane.
__device__ unsigned tile_lookback(unsigned long long *tile_word, int tile, unsigned agg, int *status) {
    const int lane = threadIdx.x & 31;
    if (tile == 0) {
        if (lane == 0) atomicExch(tile_word, kTilePrefix | agg);
        return 0u;
    }
    if (lane == 0) atomicExch(tile_word + tile, kTileAggregate | agg);
    unsigned excl = 0;
    for (int base = tile - 1;; base -= 32) {
        const int j = base - lane;  // lane 0: the nearest predecessor
        unsigned long long w = kTilePrefix;  // before tile 0: an inclusive prefix of 0
        if (j >= 0) {
            uint32_t spins = 0;
            for (;;) {
                w = *reinterpret_cast<volatile unsigned long long *>(tile_word + j);
                if (w >> 32) break;
                if (++spins >= kSpinLimit) break;
                if (spins > 16) __nanosleep(64);
            }
            if (!(w >> 32)) {
                latch_error(status, kErrTimeout);
                w = kTilePrefix;  // give up here: count it as a prefix of 0
            }
        }
        const unsigned prefix_lanes = __ballot_sync(0xffffffffu, (w >> 32) == (kTilePrefix >> 32));
        // the nearest prefix ends the walk: add lanes 0 .. k (k = its lane)
        const int k = prefix_lanes ? __ffs(prefix_lanes) - 1 : 31;
        unsigned v = lane <= k ? static_cast<unsigned>(w) : 0u;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        excl += v;
        if (prefix_lanes) break;
    }
    if (lane == 0) atomicExch(tile_word + tile, kTilePrefix | (excl + agg));
    return excl;
}

// Exclusive scan of the block's THREADS * ITEMS items (v: the thread's ITEMS
// consecutive values) across all tiles: returns the exclusive prefix of the
// thread's first item.  `state` is the scan's ticket + words.
template <int THREADS, int ITEMS>
__device__ unsigned block_scan_lookback(const unsigned (&v)[ITEMS], int tile, unsigned long long *state,
                                        int *status) {
    constexpr int WARPS = THREADS / 32;
    __shared__ unsigned warp_tot[WARPS];
    __shared__ unsigned block_agg, block_excl;
    unsigned tsum = 0;
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) tsum += v[k];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned incl = tsum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) warp_tot[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        const unsigned w = lane < WARPS ? warp_tot[lane] : 0u;
        unsigned wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += y;
        }
        if (lane < WARPS) warp_tot[lane] = wi - w;
        const unsigned agg = __shfl_sync(0xffffffffu, wi, 31);
        const unsigned ex = tile_lookback(state + 1, tile, agg, status);
        if (lane == 0) {
            block_agg = agg;
            block_excl = ex;
        }
    }
    __syncthreads();
    return block_excl + warp_tot[wid] + (incl - tsum);
}

__device__ __forceinline__ int scan_ticket(unsigned long long *state) {
    __shared__ int t;
    if (threadIdx.x == 0) t = static_cast<int>(atomicAdd(state, 1ull));
    __syncthreads();
    return t;
}

// In-place exclusive scan of n counters.
__global__ void __launch_bounds__(kCellScanThreads) k_scan_counts(unsigned *__restrict__ data, size_t n,
                                                                  unsigned long long *state, int *status) {
    constexpr int ITEMS = kCellScanItems;
    const int tile = scan_ticket(state);
    const size_t base = static_cast<size_t>(tile) * (kCellScanThreads * ITEMS) +
                        static_cast<size_t>(threadIdx.x) * ITEMS;
    unsigned v[ITEMS];
    if (base + ITEMS <= n) {
        const uint4 a = *reinterpret_cast<const uint4 *>(data + base);
        const uint4 b = *reinterpret_cast<const uint4 *>(data + base + 4);
        v[0] = a.x, v[1] = a.y, v[2] = a.z, v[3] = a.w, v[4] = b.x, v[5] = b.y, v[6] = b.z, v[7] = b.w;
    } else {
#pragma unroll
        for (int k = 0; k < ITEMS; ++k) v[k] = base + k < n ? data[base + k] : 0u;
    }
    unsigned run = block_scan_lookback<kCellScanThreads, ITEMS>(v, tile, state, status);
    if (base + ITEMS <= n) {
        uint4 a, b;
        a.x = run, run += v[0], a.y = run, run += v[1], a.z = run, run += v[2], a.w = run, run += v[3];
        b.x = run, run += v[4], b.y = run, run += v[5], b.z = run, run += v[6], b.w = run;
        *reinterpret_cast<uint4 *>(data + base) = a;
        *reinterpret_cast<uint4 *>(data + base + 4) = b;
    } else {
#pragma unroll
        for (int k = 0; k < ITEMS; ++k)
            if (base + k < n) {
                data[base + k] = run;
                run += v[k];
            }
    }
}

// Work items from the scanned cell starts: tile t (cells_per_tile cells from
// t * cells_per_tile) holds ceil(count / chunk) items of up to `chunk`
// points.  One scan over the per-tile item counts places every tile's items;
// the thread owning index ntiles stores the total in *total.
__global__ void __launch_bounds__(kItemScanThreads, 1) k_scan_emit_chunks(const unsigned *__restrict__ cell_start,
                                                                       int ntiles, int cells_per_tile, int chunk,
                                                                       int4 *__restrict__ chunks,
                                                                       unsigned long long *state, int *status,
                                                                       int *total) {
    static_assert(kItemScanItems == 1, "one bin tile per thread");
    const int tile = scan_ticket(state);
    const long long t = static_cast<long long>(tile) * kItemScanThreads + threadIdx.x;  // bin tile
    unsigned start = 0, cnt = 0;
    unsigned v[1] = {0u};
    if (t < ntiles) {
        start = cell_start[static_cast<size_t>(t) * cells_per_tile];
        cnt = cell_start[static_cast<size_t>(t + 1) * cells_per_tile] - start;
        v[0] = (cnt + chunk - 1) / chunk;
    }
    const unsigned run = block_scan_lookback<kItemScanThreads, 1>(v, tile, state, status);
    if (t == ntiles) *total = static_cast<int>(run);
    for (unsigned c = 0; c < v[0]; ++c) {
        const unsigned off = c * chunk;
        chunks[run + c] = make_int4(static_cast<int>(t), static_cast<int>(start + off),
                                    static_cast<int>(min(cnt - off, static_cast<unsigned>(chunk))), 0);
    }
}

// ---------------------------------------------------------------------------
// plan helpers
// ---------------------------------------------------------------------------
void free_points(nfft2d_plan_s *p) {
    if (p->recs || p->tmp_recs || p->keyrank || p->src || p->chunks || p->items)
        cudaStreamSynchronize(p->stream);  // no transform of the old points in flight
    plan_free(p->recs);
    plan_free(p->tmp_recs);
    plan_free(p->keyrank);
    plan_free(p->src);
    plan_free(p->chunks);
    plan_free(p->items);
    p->items = nullptr;
    p->items_cap = 0;
    p->recs = p->tmp_recs = nullptr;
    p->keyrank = nullptr;
    p->src = nullptr;
    p->chunks = nullptr;
    p->capM = 0;
    p->chunks_cap = 0;
}

// The plan's cuFFT handles back to the pool, once no transform of the plan
// is in flight (another stream may take a handle, and its work area, next).
void release_ffts(nfft2d_plan_s *p) {
    if (!p->fft_ok && !p->pruned_ok) return;
    cudaStreamSynchronize(p->stream);
    if (p->fft_ok) pooled_plan_release(p->fft);
    if (p->pruned_ok) {
        pooled_plan_release(p->fft_rows);
        pooled_plan_release(p->fft_cols);
    }
    p->fft_ok = p->pruned_ok = false;
}

void destroy_plan(nfft2d_plan_s *p) {
    if (!p) return;
    cudaStreamSynchronize(p->stream);  // its buffers go back to the cache: nothing of the plan in flight
    if (p->aux) {
        cudaStreamSynchronize(p->aux);
        cudaStreamDestroy(p->aux);
    }
    if (p->ev_fork) cudaEventDestroy(p->ev_fork);
    if (p->ev_join) cudaEventDestroy(p->ev_join);
    if (p->ev_coords) cudaEventDestroy(p->ev_coords);
    plan_free(p->F_stage);
    release_ffts(p);
    free_points(p);
    if (!p->grid_external) plan_free(p->grid);
    plan_free(p->deap1);
    plan_free(p->deap2);
    plan_free(p->d_status);
    plan_free_host(p->h_status, 4 * sizeof(int));
    plan_free(p->tw1);
    plan_free(p->tw2);
    plan_free(p->cell_count);
    plan_free(p->scan_tmp);
    for (auto &e : p->timer.ev)
        if (e) cudaEventDestroy(e);
    delete p;
}

long long chunks_capacity(const nfft2d_plan_s *p, long long M) {
    return static_cast<long long>(p->g.tiles1) * p->g.tiles2 + M / p->chunk + 1;
}

// Capacity of the spread's own work list (plans whose chunk exceeds
// kSpreadItemMax), 0 when the chunks serve the spread.
long long items_capacity(const nfft2d_plan_s *p, long long M) {
    if (p->chunk <= kSpreadItemMax) return 0;
    return static_cast<long long>(p->g.tiles1) * p->g.tiles2 + M / kSpreadItemMax + 1;
}

int ensure_points_capacity(nfft2d_plan_s *p, long long M) {
    const long long need_chunks = chunks_capacity(p, M);
    if (M <= p->capM && need_chunks <= p->chunks_cap && items_capacity(p, M) <= p->items_cap) return NFFT2D_OK;
    free_points(p);
    const long long cap = std::max<long long>(M, 1);
    const size_t rs = rec_size(p->precision);
    NFFT_TRY_CUDA(plan_malloc(reinterpret_cast<void **>(&p->recs), rs * cap));
    NFFT_TRY_CUDA(plan_malloc(reinterpret_cast<void **>(&p->tmp_recs), rs * cap));
    NFFT_TRY_CUDA(plan_malloc(reinterpret_cast<void **>(&p->keyrank), sizeof(uint2) * cap));
    NFFT_TRY_CUDA(plan_malloc(reinterpret_cast<void **>(&p->src), sizeof(int) * cap));
    const long long cc = chunks_capacity(p, cap);
    NFFT_TRY_CUDA(plan_malloc(reinterpret_cast<void **>(&p->chunks), sizeof(int4) * cc));
    const long long ic = items_capacity(p, cap);
    if (ic > 0) NFFT_TRY_CUDA(plan_malloc(reinterpret_cast<void **>(&p->items), sizeof(int4) * ic));
    p->capM = cap;
    p->chunks_cap = cc;
    p->items_cap = ic;
    return NFFT2D_OK;
}

size_t plan_workspace_bytes(const nfft2d_plan_s *p) {
    const size_t grid = cplx_size(p->precision) * static_cast<size_t>(p->g.Ra) * p->g.C;
    const size_t pts = static_cast<size_t>(p->capM) * (2 * rec_size(p->precision) + sizeof(uint2) + sizeof(int)) +
                       static_cast<size_t>(p->chunks_cap + p->items_cap) * sizeof(int4);
    const size_t bins = sizeof(unsigned) * (p->ncells + 1 + p->scan_tmp_elems);
    return grid + pts + bins + real_size(p->precision) * (p->N1 + p->N2);
}

int check_plan(nfft2d_plan_s *p) { return p ? NFFT2D_OK : NFFT2D_ERR_INVALID_ARG; }

// The cuFFT plans on the padded grid's interior (advanced layout) that the
// plan's FFT mode runs on, taken from the pool when missing: the 2D plan, or
// from 2048 x 2048 cells up (or fft_mode 1) the pruned pair -- n1 rows of n2
// points (contiguous, pitch C) and N2/2 columns of n1 points (stride C), run
// once per half of the band -- with the 2D plan as the fallback.  Nothing
// for the fused passes.  Plans for a batch's external grid are the batch's.
int ensure_ffts(nfft2d_plan_s *p) {
    if (p->grid_external || use_fused(p)) return NFFT2D_OK;
    const Geom &g = p->g;
    const cufftType t = p->precision == NFFT2D_F64 ? CUFFT_Z2Z : CUFFT_C2C;
    const bool pruned = p->fft_mode == 1 || (p->fft_mode < 0 && 1LL * g.n1 * g.n2 >= 2048LL * 2048LL);
    if (pruned && !p->pruned_ok) {
        const int nr[1] = {g.n2}, er[1] = {g.C};
        const int nc[1] = {g.n1}, ec[1] = {g.Ra};
        if (pooled_plan_many(&p->fft_rows, 1, nr, er, 1, g.C, er, 1, g.C, t, g.n1) == CUFFT_SUCCESS) {
            if (pooled_plan_many(&p->fft_cols, 1, nc, ec, g.C, 1, ec, g.C, 1, t, p->N2 / 2) == CUFFT_SUCCESS) {
                p->pruned_ok = cufftSetStream(p->fft_rows, p->stream) == CUFFT_SUCCESS &&
                               cufftSetStream(p->fft_cols, p->stream) == CUFFT_SUCCESS;
                if (!p->pruned_ok) {
                    pooled_plan_release(p->fft_rows);
                    pooled_plan_release(p->fft_cols);
                }
            } else {
                pooled_plan_release(p->fft_rows);
            }
        }
    }
    if ((!pruned || !p->pruned_ok) && !p->fft_ok) {
        const int n[2] = {g.n1, g.n2};
        const int emb[2] = {g.Ra, g.C};
        const int dist = g.Ra * g.C;
        cufftResult fr = pooled_plan_many(&p->fft, 2, n, emb, 1, dist, emb, 1, dist, t, 1);
        if (fr != CUFFT_SUCCESS) return status_from_cufft(fr);
        p->fft_ok = true;
        if ((fr = cufftSetStream(p->fft, p->stream)) != CUFFT_SUCCESS) return status_from_cufft(fr);
    }
    return NFFT2D_OK;
}

// (Re)allocate the padded grid for the current geometry, take the cuFFT
// plans its FFT mode needs and rebuild the TMA descriptor.
int setup_grid(nfft2d_plan_s *p) {
    const Geom &g = p->g;
    release_ffts(p);
    p->tmap_ok = false;
    if (!p->grid_external) {
        if (p->grid) cudaStreamSynchronize(p->stream);  // no transform on the old grid in flight
        plan_free(p->grid);
        p->grid = nullptr;
        // 256 zeroed bytes of slack after the grid: the 16-byte-load gather
        // may read one complex past the last row's end (with weight 0)
        const size_t bytes = cplx_size(p->precision) * static_cast<size_t>(g.Ra) * g.C + 256;
        NFFT_TRY_CUDA(plan_malloc(reinterpret_cast<void **>(&p->grid), bytes));
        NFFT_TRY_CUDA(cudaMemsetAsync(p->grid, 0, bytes, p->stream));
        const int st = setup_fused_fft(p);
        if (st != NFFT2D_OK) return st;
        // the cuFFT plans the current FFT mode runs on (none for the fused passes)
        const int sf = ensure_ffts(p);
        if (sf != NFFT2D_OK) return sf;
    }
    if (p->precision == NFFT2D_F32) return make_tensor_map(p);
    return NFFT2D_OK;
}

// (Re)allocate the bin counters for the current tile geometry.
int setup_bins(nfft2d_plan_s *p) {
    const Geom &g = p->g;
    if (p->cell_count || p->scan_tmp) cudaStreamSynchronize(p->stream);
    plan_free(p->cell_count);
    plan_free(p->scan_tmp);
    p->cell_count = p->scan_tmp = nullptr;
    p->ncells = static_cast<size_t>(g.tiles1) * g.tiles2 * g.T * g.T;
    const size_t ntiles = static_cast<size_t>(g.tiles1) * g.tiles2;
    // two 64-bit scan states (cells, work items), counted in 32-bit words
    // 64-bit state words of three scans: cells, work items, the spread's own items
    p->scan_tmp_elems = 2 * (scan_state_words(p->ncells + 1, kCellScanThreads * kCellScanItems) +
                             2 * scan_state_words(ntiles + 1, kItemScanThreads * kItemScanItems));
    NFFT_TRY_CUDA(plan_malloc(reinterpret_cast<void **>(&p->cell_count), sizeof(unsigned) * (p->ncells + 1)));
    NFFT_TRY_CUDA(plan_malloc(reinterpret_cast<void **>(&p->scan_tmp), sizeof(unsigned) * p->scan_tmp_elems));
    return NFFT2D_OK;
}


// Self-test of the bounded device-side wait: one thread waits on an
// mbarrier phase that nothing completes, gives up after `limit` polls (the
// same mbar_wait_bounded the tiled kernels use) and records the timeout.
__device__ int g_selftest_status;
__global__ void k_selftest_wait(uint32_t limit) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_proxy_async_smem();
        g_selftest_status = mbar_wait_bounded(&bar, 0, limit) ? 0 : kErrTimeout;
    }
}

}  // namespace

namespace nfft2d {
// The same bounded wait latching kErrTimeout into a plan's (or batch's)
// status word, as the tiled kernels do when their own wait runs out.
__global__ void k_selftest_latch(uint32_t limit, int *status) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_proxy_async_smem();
        if (!mbar_wait_bounded(&bar, 0, limit)) latch_error(status, kErrTimeout);
    }
}
}  // namespace nfft2d

namespace {

// Launch shape for the small elementwise kernels.
dim3 row_grid(int cols, int rows) {
    const int bx = std::max(1, std::min((cols + 255) / 256, 64));
    return dim3(bx, rows, 1);
}

}  // namespace

// ===========================================================================
// internal API used by the other translation units
// ===========================================================================
namespace nfft2d {

int compute_layout(int N1, int N2, double sigma, int K, int precision, int tile, Geom *g, int *n1o, int *n2o,
                   bool strips) {
    if (N1 <= 0 || N2 <= 0 || (N1 & 1) || (N2 & 1)) return NFFT2D_ERR_INVALID_ARG;
    if (K < kMinK || K > kMaxK) return NFFT2D_ERR_INVALID_ARG;
    if (precision != NFFT2D_F32 && precision != NFFT2D_F64) return NFFT2D_ERR_INVALID_ARG;
    if (!(sigma >= 1.25) || !std::isfinite(sigma)) return NFFT2D_ERR_INVALID_ARG;
    const double c1 = sigma * N1, c2 = sigma * N2;
    const long long n1 = std::llround(c1), n2 = std::llround(c2);
    if (std::fabs(c1 - n1) > 1e-9 || std::fabs(c2 - n2) > 1e-9) return NFFT2D_ERR_INVALID_ARG;
    if ((n1 & 1) || (n2 & 1)) return NFFT2D_ERR_INVALID_ARG;
    if (n1 < 2 * K + 2 || n2 < 2 * K + 2) return NFFT2D_ERR_INVALID_ARG;
    if (n1 > 46000 || n2 > 46000) return NFFT2D_ERR_INVALID_ARG;
    const int nmin = static_cast<int>(std::min(n1, n2));
    int T = tile;
    if (T == 0) {
        // 16 x 16 tiles: the register-resident spread needs them, and the
        // gather runs within a few percent of its best tile there
        T = 16;
        while (T > 8 && T > nmin) T >>= 1;
    }
    if (T != 8 && T != 16 && T != 32 && T != 64) return NFFT2D_ERR_INVALID_ARG;
    if (T > nmin) return NFFT2D_ERR_INVALID_ARG;
    g->n1 = static_cast<int>(n1);
    g->n2 = static_cast<int>(n2);
    g->H = kHalo;
    g->T = T;
    g->tiles1 = (g->n1 + T - 1) / T;
    g->tiles2 = (g->n2 + T - 1) / T;
    g->Ke = K + (K & 1);
    // strip-major cell order inside a tile where the register spread runs
    // (FP32, 16 x 16 tiles), plain row-major elsewhere
    g->SW = (strips && precision == NFFT2D_F32 && T == 16) ? spread_strip_width(K) : T;
    g->PR = T + 2 * K;
    // Patch row pitch: the T + 2Ke columns a tile needs, rounded up to 16
    // complex (128 bytes); with it a warp's reads of one tap spread over the
    // shared-memory banks with fewer conflicts (2.6 instead of 3.1 wavefronts
    // per 64-bit load on the polar and uniform point sets at T = 32, K = 6).
    g->PC = ((T + 2 * g->Ke + 15) / 16) * 16;
    // Strip-ordered tiles put a warp's consecutive points in SW columns and
    // many rows; a pitch of SW mod 16 complex shifts each patch row by 2 SW
    // banks, so the tiled gather's 8-byte tap loads of a half-warp (16
    // points, 16 / SW rows of SW columns) meet distinct banks.
    if (g->SW < T) g->PC += g->SW;
    g->R = g->n1 + 2 * kHalo;
    g->Cl = g->n2 + 2 * kHalo;
    // allocation: whole tiles + halo, plus the pitch padding of the last patch
    g->C = g->tiles2 * T + 2 * kHalo + (g->PC - T - 2 * g->Ke);
    g->Ra = g->tiles1 * T + 2 * kHalo;
    const unsigned long long ncells = 1ULL * g->tiles1 * g->tiles2 * T * T;
    if (ncells >= (1ULL << 31)) return NFFT2D_ERR_INVALID_ARG;
    if (n1o) *n1o = g->n1;
    if (n2o) *n2o = g->n2;
    return NFFT2D_OK;
}

int grid_blocks(const nfft2d_plan_s *p, const void *kernel, int threads, int smem) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    return per_sm * std::max(1, p->num_sms);
}

cudaError_t launch_pad(const nfft2d_plan_s *p, const void *F) {
    const Geom &g = p->g;
    const dim3 grid = row_grid(g.n2, g.n1);
    if (p->precision == NFFT2D_F64)
        k_pad<double2, double><<<grid, 256, 0, p->stream>>>(
            static_cast<const double2 *>(F), static_cast<double2 *>(p->grid), static_cast<const double *>(p->deap1),
            static_cast<const double *>(p->deap2), p->N1, p->N2, g.n1, g.n2, g.H, g.C);
    else
        k_pad_f32x2<<<row_grid(g.n2 / 2, g.n1), 256, 0, p->stream>>>(
            static_cast<const float2 *>(F), static_cast<float2 *>(p->grid), static_cast<const float *>(p->deap1),
            static_cast<const float *>(p->deap2), p->N1, p->N2, g.n1, g.n2, g.H, g.C);
    return cudaGetLastError();
}

cudaError_t launch_crop(const nfft2d_plan_s *p, void *F) {
    const Geom &g = p->g;
    const dim3 grid = row_grid(p->N2, p->N1);
    if (p->precision == NFFT2D_F64)
        k_crop<double2, double><<<grid, 256, 0, p->stream>>>(
            static_cast<const double2 *>(p->grid), static_cast<double2 *>(F), static_cast<const double *>(p->deap1),
            static_cast<const double *>(p->deap2), p->N1, p->N2, g.n1, g.n2, g.H, g.C);
    else
        k_crop<float2, float><<<grid, 256, 0, p->stream>>>(
            static_cast<const float2 *>(p->grid), static_cast<float2 *>(F), static_cast<const float *>(p->deap1),
            static_cast<const float *>(p->deap2), p->N1, p->N2, g.n1, g.n2, g.H, g.C);
    return cudaGetLastError();
}

cudaError_t launch_halo_fill(const nfft2d_plan_s *p) {
    const Geom &g = p->g;
    const long long n = 2LL * g.H * g.C + 2LL * g.H * g.n1;
    const int blocks = static_cast<int>(std::min<long long>((n + 255) / 256, 4LL * p->num_sms));
    if (p->precision == NFFT2D_F64)
        k_halo_fill<double2><<<blocks, 256, 0, p->stream>>>(static_cast<double2 *>(p->grid), g.n1, g.n2, g.H, g.C);
    else
        k_halo_fill<float2><<<blocks, 256, 0, p->stream>>>(static_cast<float2 *>(p->grid), g.n1, g.n2, g.H, g.C);
    return cudaGetLastError();
}

cudaError_t launch_halo_fold(const nfft2d_plan_s *p) {
    const Geom &g = p->g;
    const long long n = 2LL * g.H * (g.n1 + g.n2);
    const int blocks = static_cast<int>(std::min<long long>((n + 255) / 256, 4LL * p->num_sms));
    if (p->precision == NFFT2D_F64)
        k_halo_fold<double2><<<blocks, 256, 0, p->stream>>>(static_cast<double2 *>(p->grid), g.n1, g.n2, g.H, g.R, g.Cl, g.C);
    else
        k_halo_fold<float2><<<blocks, 256, 0, p->stream>>>(static_cast<float2 *>(p->grid), g.n1, g.n2, g.H, g.R, g.Cl, g.C);
    return cudaGetLastError();
}

}  // namespace nfft2d

// ===========================================================================
// C ABI
// ===========================================================================
namespace {

// One in-place C2C / Z2Z transform (a 1D batch or the full 2D plan) at
// element offset off of the grid.
cufftResult exec_at(const nfft2d_plan_s *p, cufftHandle h, size_t off, int dir) {
    if (p->precision == NFFT2D_F64) {
        cufftDoubleComplex *d = static_cast<cufftDoubleComplex *>(p->grid) + off;
        return cufftExecZ2Z(h, d, d, dir);
    }
    cufftComplex *d = static_cast<cufftComplex *>(p->grid) + off;
    return cufftExecC2C(h, d, d, dir);
}

// The oversampled FFT.  With the pruned plans the 2D transform runs as two
// 1D passes and the column pass covers only the columns that matter: for a
// type-2 transform (type2 = true) the padded coefficients are zero outside
// the band |k2| < N2/2, so only those columns are transformed (first), then
// every row; for a type-1 transform every row is transformed first and only
// the columns the crop keeps afterwards.  With sigma = 2 that is 1.5 passes
// over the grid instead of 2.
int run_fft(nfft2d_plan_s *p, int sign, bool type2) {
    const Geom &g = p->g;
    const int dir = sign < 0 ? CUFFT_FORWARD : CUFFT_INVERSE;
    const size_t off = static_cast<size_t>(g.H) * g.C + g.H;
    // by default the two passes run from 2048 x 2048 oversampled cells up:
    // below that cuFFT's single 2D plan is faster on GB300 (1024^2: 20 us
    // vs 30 us; 2048^2: 40 vs 35 us; 4096^2: 153 vs 112 us)
    const bool pruned = p->fft_mode == 1 || (p->fft_mode < 0 && 1LL * g.n1 * g.n2 >= 2048LL * 2048LL);
    if (!(pruned && p->pruned_ok) && !p->fft_ok) {  // a mode set on a plan made without its plans
        const int st = ensure_ffts(p);
        if (st != NFFT2D_OK) return st;
    }
    if (!(pruned && p->pruned_ok)) return status_from_cufft(exec_at(p, p->fft, off, dir));
    const size_t right = off + static_cast<size_t>(g.n2 - p->N2 / 2);  // first column of the negative band
    cufftResult r;
    if (type2) {
        if ((r = exec_at(p, p->fft_cols, off, dir)) != CUFFT_SUCCESS) return status_from_cufft(r);
        if ((r = exec_at(p, p->fft_cols, right, dir)) != CUFFT_SUCCESS) return status_from_cufft(r);
        return status_from_cufft(exec_at(p, p->fft_rows, off, dir));
    }
    if ((r = exec_at(p, p->fft_rows, off, dir)) != CUFFT_SUCCESS) return status_from_cufft(r);
    if ((r = exec_at(p, p->fft_cols, off, dir)) != CUFFT_SUCCESS) return status_from_cufft(r);
    return status_from_cufft(exec_at(p, p->fft_cols, right, dir));
}


int type2_prepare(nfft2d_plan_s *p, int sign, const void *F) {
    if (use_fused(p)) {  // pad + band-column FFT, then row FFT + halo fill
        stage_begin(p, ST_PAD);
        NFFT_TRY_CUDA(fused_type2_cols(p, sign, F));
        stage_end(p, ST_PAD);
        stage_begin(p, ST_FFT2);
        NFFT_TRY_CUDA(fused_type2_rows(p, sign));
        stage_end(p, ST_FFT2);
        return NFFT2D_OK;
    }
    stage_begin(p, ST_PAD);
    NFFT_TRY_CUDA(launch_pad(p, F));
    stage_end(p, ST_PAD);
    stage_begin(p, ST_FFT2);
    int st = run_fft(p, sign, true);
    if (st != NFFT2D_OK) return st;
    stage_end(p, ST_FFT2);
    stage_begin(p, ST_FILL);
    NFFT_TRY_CUDA(launch_halo_fill(p));
    stage_end(p, ST_FILL);
    return NFFT2D_OK;
}

}  // namespace

extern "C" {

const char *nfft2d_status_string(int s) {
    switch (s) {
        case NFFT2D_OK: return "ok";
        case NFFT2D_ERR_INVALID_ARG: return "invalid argument";
        case NFFT2D_ERR_OOM: return "out of memory";
        case NFFT2D_ERR_CUDA: return "CUDA runtime error";
        case NFFT2D_ERR_CUFFT: return "cuFFT error";
        case NFFT2D_ERR_NO_POINTS: return "no points set on the plan";
        case NFFT2D_ERR_NONFINITE: return "non-finite point coordinate";
        case NFFT2D_ERR_DEVICE_TIMEOUT: return "device-side wait timed out";
        case NFFT2D_ERR_DEVICE_BOUNDS: return "device-side bounds check failed";
        case NFFT2D_ERR_UNSUPPORTED: return "unsupported request";
        case NFFT2D_ERR_INTERNAL: return "internal error";
        case NFFT2D_ERR_SCRATCH_LIMIT: return "size exceeds the fixed scratch of the no-allocation entry point";
        default: return "unknown status";
    }
}

int nfft2d_selftest_wait_timeout(int spin_limit, void *stream) {
    if (spin_limit < 1) return NFFT2D_ERR_INVALID_ARG;
    const cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int init = -1;
    NFFT_TRY_CUDA(cudaMemcpyToSymbolAsync(g_selftest_status, &init, sizeof(int), 0, cudaMemcpyHostToDevice, st));
    k_selftest_wait<<<1, 32, 0, st>>>(static_cast<uint32_t>(spin_limit));
    NFFT_TRY_CUDA(cudaGetLastError());
    int h = -1;
    NFFT_TRY_CUDA(cudaMemcpyFromSymbolAsync(&h, g_selftest_status, sizeof(int), 0, cudaMemcpyDeviceToHost, st));
    NFFT_TRY_CUDA(cudaStreamSynchronize(st));
    if (h == kErrTimeout) return NFFT2D_ERR_DEVICE_TIMEOUT;
    return h == 0 ? NFFT2D_OK : NFFT2D_ERR_INTERNAL;
}

int nfft2d_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
    return n;
}

int nfft2d_layout_query(int N1, int N2, double sigma, int K, int precision, int tile, nfft2d_info *info) {
    if (!info) return NFFT2D_ERR_INVALID_ARG;
    Geom g{};
    int st = compute_layout(N1, N2, sigma, K, precision, tile, &g, nullptr, nullptr);
    if (st != NFFT2D_OK) return st;
    std::memset(info, 0, sizeof(*info));
    info->N1 = N1;
    info->N2 = N2;
    info->sigma = sigma;
    info->K = K;
    info->precision = precision;
    info->n1 = g.n1;
    info->n2 = g.n2;
    info->halo = g.H;
    info->rows = g.Ra;
    info->cols = g.C;
    info->tile = g.T;
    info->tiles1 = g.tiles1;
    info->tiles2 = g.tiles2;
    info->patch_rows = g.PR;
    info->patch_cols = g.PC;
    info->chunk = 256;
    info->gather_variant = precision == NFFT2D_F32 ? NFFT2D_VARIANT_TILED : NFFT2D_VARIANT_DIRECT;
    info->spread_variant = info->gather_variant;
    return NFFT2D_OK;
}

}  // extern "C"

namespace nfft2d {

int create_plan(nfft2d_plan_s **out, int N1, int N2, double sigma, int K, int precision, int tile,
                cudaStream_t stream, void *ext_grid, bool strips) {
    if (!out) return NFFT2D_ERR_INVALID_ARG;
    *out = nullptr;
    Geom g{};
    int st = compute_layout(N1, N2, sigma, K, precision, tile, &g, nullptr, nullptr, strips);
    if (st != NFFT2D_OK) return st;
    nfft2d_plan_s *p = new (std::nothrow) nfft2d_plan_s();
    if (!p) return NFFT2D_ERR_OOM;
    p->N1 = N1;
    p->N2 = N2;
    p->K = K;
    p->sigma = sigma;
    p->precision = precision;
    p->g = g;
    p->strips = strips;
    p->stream = stream;
    p->grid = ext_grid;
    p->grid_external = ext_grid != nullptr;
    if (precision == NFFT2D_F64) {
        p->gather_variant = NFFT2D_VARIANT_DIRECT;
        p->spread_variant = NFFT2D_VARIANT_DIRECT;
        p->gather_auto = false;
    }
    auto fail = [&](int s) {
        destroy_plan(p);
        return s;
    };
    if (cudaGetDevice(&p->device) != cudaSuccess) return fail(NFFT2D_ERR_CUDA);
    if (cudaDeviceGetAttribute(&p->num_sms, cudaDevAttrMultiProcessorCount, p->device) != cudaSuccess)
        return fail(NFFT2D_ERR_CUDA);
    if (cudaDeviceGetAttribute(&p->l2_bytes, cudaDevAttrL2CacheSize, p->device) != cudaSuccess)
        return fail(NFFT2D_ERR_CUDA);

    // window constants (FP64, plan time)
    const double alpha = (2.0 - 1.0 / sigma) * kPi - 0.01;
    p->w.alpha = alpha;
    p->w.cn = K / std::sinh(alpha * K);
    p->w.kp = K / (1.0 - std::exp(-2.0 * alpha * K));
    const double poly_err = cached_window_poly(sigma, K, &p->poly);
    if (!(poly_err >= 0.0 && poly_err < 1e-8)) return fail(NFFT2D_ERR_INTERNAL);

    const size_t rs = real_size(precision);
    cudaError_t e;
    if ((st = setup_grid(p)) != NFFT2D_OK) return fail(st);
    if ((st = setup_bins(p)) != NFFT2D_OK) return fail(st);
    if ((e = plan_malloc(reinterpret_cast<void **>(&p->deap1), rs * N1)) != cudaSuccess) return fail(status_from_cuda(e));
    if ((e = plan_malloc(reinterpret_cast<void **>(&p->deap2), rs * N2)) != cudaSuccess) return fail(status_from_cuda(e));
    if ((e = plan_malloc(reinterpret_cast<void **>(&p->d_status), 4 * sizeof(int))) != cudaSuccess) return fail(status_from_cuda(e));
    if ((e = plan_malloc_host(reinterpret_cast<void **>(&p->h_status), 4 * sizeof(int))) != cudaSuccess)
        return fail(status_from_cuda(e));
    if ((e = cudaMemsetAsync(p->d_status, 0, 4 * sizeof(int), p->stream)) != cudaSuccess)
        return fail(status_from_cuda(e));

    // Deapodization tables S / phi(xi_k), S = sinh(alpha K)/(pi K) (the
    // window normalisation), phi(xi) = I0(K sqrt(alpha^2 - xi^2)),
    // xi_k = 2 pi k / (sigma N)  (NFFT1_2D.m:17-22, NFFT2_2D.cu:60-69).
    for (int d = 0; d < 2; ++d) {
        const int N = d == 0 ? N1 : N2;
        std::vector<double> tab(N);
        deapod_table_host(N, d == 0 ? g.n1 : g.n2, K, alpha, tab.data());
        void *dst = d == 0 ? p->deap1 : p->deap2;
        if (precision == NFFT2D_F64) {
            e = cudaMemcpy(dst, tab.data(), sizeof(double) * N, cudaMemcpyHostToDevice);
        } else {
            std::vector<float> tf(tab.begin(), tab.end());
            e = cudaMemcpy(dst, tf.data(), sizeof(float) * N, cudaMemcpyHostToDevice);
        }
        if (e != cudaSuccess) return fail(status_from_cuda(e));
    }

    // the stage events are created when timing is first enabled
    if ((e = cudaStreamSynchronize(p->stream)) != cudaSuccess) return fail(status_from_cuda(e));
    p->workspace_bytes = plan_workspace_bytes(p);
    *out = p;
    return NFFT2D_OK;
}

void release_plan(nfft2d_plan_s *p) { destroy_plan(p); }

int tensor_map_for(nfft2d_plan_s *p) { return make_tensor_map(p); }

}  // namespace nfft2d

extern "C" {

int nfft2d_plan_create(nfft2d_plan *out, int N1, int N2, double sigma, int K, int precision, void *stream) {
    return nfft2d::create_plan(out, N1, N2, sigma, K, precision, 0, static_cast<cudaStream_t>(stream), nullptr);
}

int nfft2d_plan_destroy(nfft2d_plan p) {
    if (!p) return NFFT2D_ERR_INVALID_ARG;
    cudaStreamSynchronize(p->stream);
    destroy_plan(p);
    return NFFT2D_OK;
}

int nfft2d_set_stream(nfft2d_plan p, void *stream) {
    if (!p) return NFFT2D_ERR_INVALID_ARG;
    p->stream = static_cast<cudaStream_t>(stream);
    if (p->pruned_ok) {
        cufftResult r = cufftSetStream(p->fft_rows, p->stream);
        if (r == CUFFT_SUCCESS) r = cufftSetStream(p->fft_cols, p->stream);
        if (r != CUFFT_SUCCESS) return status_from_cufft(r);
    }
    return p->fft_ok ? status_from_cufft(cufftSetStream(p->fft, p->stream)) : NFFT2D_OK;
}

int nfft2d_set_tuning(nfft2d_plan p, const nfft2d_tuning *t) {
    if (!p || !t) return NFFT2D_ERR_INVALID_ARG;
    if (t->tile > 0 && t->tile != p->g.T) {
        Geom g{};
        int st = compute_layout(p->N1, p->N2, p->sigma, p->K, p->precision, t->tile, &g, nullptr, nullptr, p->strips);
        if (st != NFFT2D_OK) return st;
        cudaStreamSynchronize(p->stream);
        p->g = g;
        free_points(p);
        p->points_valid = false;
        p->M = 0;
        if ((st = setup_grid(p)) != NFFT2D_OK) return st;
        if ((st = setup_bins(p)) != NFFT2D_OK) return st;
    }
    if (t->chunk != 0 && t->chunk != -1) {
        if (t->chunk < 32 || t->chunk > (1 << 20)) return NFFT2D_ERR_INVALID_ARG;
        if (t->chunk != p->chunk) {
            p->chunk = t->chunk;
            p->points_valid = false;
            p->M = 0;
        }
    }
    for (int v : {t->gather_variant, t->spread_variant})
        if (v < -1 || v > NFFT2D_VARIANT_DIRECT) return NFFT2D_ERR_INVALID_ARG;
    const int auto_v = p->precision == NFFT2D_F32 ? NFFT2D_VARIANT_TILED : NFFT2D_VARIANT_DIRECT;
    if (t->gather_variant >= 0) {  // -1 keeps the current choice (automatic or fixed)
        const bool gauto = t->gather_variant == NFFT2D_VARIANT_AUTO && p->precision == NFFT2D_F32;
        const int gv = gauto ? auto_gather(p, p->points_valid ? p->M : 0)
                             : (t->gather_variant == NFFT2D_VARIANT_AUTO ? auto_v : t->gather_variant);
        if (p->precision == NFFT2D_F64 && gv == NFFT2D_VARIANT_TILED) return NFFT2D_ERR_UNSUPPORTED;
        p->gather_variant = gv;
        p->gather_auto = gauto;
    }
    if (t->spread_variant >= 0) {
        const int sv = t->spread_variant == NFFT2D_VARIANT_AUTO ? auto_v : t->spread_variant;
        if (p->precision == NFFT2D_F64 && sv == NFFT2D_VARIANT_TILED) return NFFT2D_ERR_UNSUPPORTED;
        p->spread_variant = sv;
    }
    if (t->compensated >= 0) p->compensated = t->compensated ? 1 : 0;
    if (t->io_order >= 0) {
        if (t->io_order != NFFT2D_ORDER_CALLER && t->io_order != NFFT2D_ORDER_BINNED) return NFFT2D_ERR_INVALID_ARG;
        p->binned_io = t->io_order == NFFT2D_ORDER_BINNED;
    }
    if (t->fft_mode > 2 || t->fft_mode < -1) return NFFT2D_ERR_INVALID_ARG;
    if (t->fft_mode == 2 && !p->fused_ok) return NFFT2D_ERR_UNSUPPORTED;
    if (t->fft_mode >= 0) {
        p->fft_mode = t->fft_mode;
        const int sf = ensure_ffts(p);  // the new mode's cuFFT plans now, not inside a transform
        if (sf != NFFT2D_OK) return sf;
    }
    p->workspace_bytes = plan_workspace_bytes(p);
    return NFFT2D_OK;
}

int nfft2d_get_info(nfft2d_plan p, nfft2d_info *info) {
    if (!p || !info) return NFFT2D_ERR_INVALID_ARG;
    std::memset(info, 0, sizeof(*info));
    info->N1 = p->N1;
    info->N2 = p->N2;
    info->sigma = p->sigma;
    info->K = p->K;
    info->precision = p->precision;
    info->n1 = p->g.n1;
    info->n2 = p->g.n2;
    info->halo = p->g.H;
    info->rows = p->g.Ra;
    info->cols = p->g.C;
    info->tile = p->g.T;
    info->tiles1 = p->g.tiles1;
    info->tiles2 = p->g.tiles2;
    info->patch_rows = p->g.PR;
    info->patch_cols = p->g.PC;
    info->chunk = p->chunk;
    info->gather_variant = p->gather_variant;
    info->spread_variant = p->spread_variant;
    info->M = p->points_valid ? p->M : 0;
    info->n_chunks = p->points_valid ? p->n_chunks : 0;
    info->workspace_bytes = p->workspace_bytes;
    info->fft_mode = fft_mode_in_use(p);
    return NFFT2D_OK;
}

static int nfft2d_set_points_impl(nfft2d_plan p, long long M, const void *x1, const void *x2, int coord_dtype, int units,
                                  bool async) {
    if (!p) return NFFT2D_ERR_INVALID_ARG;
    if (units != NFFT2D_UNITS_GRID && units != NFFT2D_UNITS_UNIT && units != NFFT2D_UNITS_RADIANS)
        return NFFT2D_ERR_INVALID_ARG;
    double u1 = 1.0, u2 = 1.0;
    if (units == NFFT2D_UNITS_UNIT) {
        u1 = p->N1;
        u2 = p->N2;
    } else if (units == NFFT2D_UNITS_RADIANS) {
        u1 = p->N1 / (2.0 * kPi);
        u2 = p->N2 / (2.0 * kPi);
    }
    return nfft2d::set_points_scaled(p, M, x1, x2, coord_dtype, u1, u2, 0.0, 0.0, async);
}

// The address the binning kernel reads coordinates through: device or
// managed memory as given; page-locked host memory (cudaHostAlloc,
// cudaHostRegister) through its device mapping, so the binning pass itself
// pulls the coordinates over the host link and no separate upload runs
// first; other host memory only where the device can read pageable memory
// (cudaDevAttrPageableMemoryAccess, e.g. a coherent CPU-GPU link), else
// INVALID_ARG instead of a faulting read.
static int coord_device_ptr(const nfft2d_plan_s *p, const void *x, const void **dx) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, x) != cudaSuccess) {
        cudaGetLastError();
        return NFFT2D_ERR_INVALID_ARG;
    }
    if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) {
        *dx = x;
        return NFFT2D_OK;
    }
    if (a.type == cudaMemoryTypeHost) {
        if (!a.devicePointer) return NFFT2D_ERR_INVALID_ARG;
        *dx = a.devicePointer;
        return NFFT2D_OK;
    }
    int pageable = 0;
    if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, p->device) != cudaSuccess || !pageable)
        return NFFT2D_ERR_INVALID_ARG;
    *dx = x;
    return NFFT2D_OK;
}

extern "C++" {
int nfft2d::bin_small_batch(nfft2d_plan_s *const *plans, const long long *M, const void *const *x1,
                             const void *const *x2, int coord_dtype, int units, int count, cudaStream_t stream) {
    if (count < 1 || (coord_dtype != NFFT2D_COORD_F32 && coord_dtype != NFFT2D_COORD_F64))
        return NFFT2D_ERR_INVALID_ARG;
    if (units != NFFT2D_UNITS_GRID && units != NFFT2D_UNITS_UNIT && units != NFFT2D_UNITS_RADIANS)
        return NFFT2D_ERR_INVALID_ARG;
    std::vector<SmallBinJob> jobs(static_cast<size_t>(count));
    size_t max_cells = 0;
    for (int i = 0; i < count; ++i) {
        nfft2d_plan_s *p = plans[i];
        if (!p || M[i] < 0 || M[i] > (1LL << 24) || p->precision != NFFT2D_F32) return NFFT2D_ERR_UNSUPPORTED;
        if (M[i] > 0 && (!x1[i] || !x2[i])) return NFFT2D_ERR_INVALID_ARG;
        max_cells = std::max(max_cells, p->ncells);
    }
    const size_t smem = sizeof(unsigned) * (max_cells + 1 + 32);
    if (smem > 200 * 1024) return NFFT2D_ERR_UNSUPPORTED;  // the counters must fit in shared memory
    int *d_out = nullptr;
    SmallBinJob *d_jobs = nullptr;
    for (int i = 0; i < count; ++i) {
        nfft2d_plan_s *p = plans[i];
        const void *dx1 = x1[i], *dx2 = x2[i];
        if (M[i] > 0) {
            int st = coord_device_ptr(p, x1[i], &dx1);
            if (st == NFFT2D_OK) st = coord_device_ptr(p, x2[i], &dx2);
            if (st != NFFT2D_OK) return st;
        }
        p->points_valid = false;
        p->M = 0;
        p->n_chunks = 0;
        const int st = ensure_points_capacity(p, std::max<long long>(M[i], 1));
        if (st != NFFT2D_OK) return st;
        p->workspace_bytes = plan_workspace_bytes(p);
        // the unit scales of nfft2d_set_points
        const double u1 = units == NFFT2D_UNITS_GRID ? 1.0 : (units == NFFT2D_UNITS_UNIT ? p->N1 : p->N1 / (2.0 * kPi));
        const double u2 = units == NFFT2D_UNITS_GRID ? 1.0 : (units == NFFT2D_UNITS_UNIT ? p->N2 : p->N2 / (2.0 * kPi));
        const double s1 = p->sigma * u1, s2 = p->sigma * u2;
        p->xscale1 = s1;
        p->xscale2 = s2;
        int e1 = 0, e2 = 0;
        const bool pow2 = std::frexp(s1, &e1) == 0.5 && std::frexp(s2, &e2) == 0.5;
        SmallBinJob &J = jobs[static_cast<size_t>(i)];
        J.x1 = dx1;
        J.x2 = dx2;
        J.M = static_cast<int>(M[i]);
        J.s1 = s1;
        J.s2 = s2;
        J.s1f = static_cast<float>(s1);
        J.s2f = static_cast<float>(s2);
        J.exact = (coord_dtype == NFFT2D_COORD_F32 && pow2) ? 1 : 0;
        J.g = p->g;
        J.tmp = static_cast<Rec32 *>(p->tmp_recs);
        J.keyrank = p->keyrank;
        J.recs = static_cast<Rec32 *>(p->recs);
        J.src = p->src;
        J.chunks = p->chunks;
        J.chunk = p->chunk;
        J.status = p->d_status;
        J.out = nullptr;  // set below
    }
    NFFT_TRY_CUDA(cudaMallocAsync(reinterpret_cast<void **>(&d_out), sizeof(int) * 2 * count, stream));
    for (int i = 0; i < count; ++i) jobs[static_cast<size_t>(i)].out = d_out + 2 * i;
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(&d_jobs), sizeof(SmallBinJob) * count, stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_jobs, jobs.data(), sizeof(SmallBinJob) * count, cudaMemcpyHostToDevice, stream);
    auto kernel = coord_dtype == NFFT2D_COORD_F64 ? k_bin_small<double> : k_bin_small<float>;
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e == cudaSuccess) {
        kernel<<<count, kSmallBinThreads, smem, stream>>>(d_jobs);
        e = cudaGetLastError();
    }
    std::vector<int> out(static_cast<size_t>(2 * count));
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out.data(), d_out, sizeof(int) * 2 * count, cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    cudaFreeAsync(d_jobs, stream);
    cudaFreeAsync(d_out, stream);
    if (e != cudaSuccess) return status_from_cuda(e);
    int status = NFFT2D_OK;
    for (int i = 0; i < count; ++i) {
        nfft2d_plan_s *p = plans[i];
        const int n_chunks = out[static_cast<size_t>(2 * i)], bits = out[static_cast<size_t>(2 * i + 1)];
        if (bits & kErrNonfinite) {
            status = NFFT2D_ERR_NONFINITE;
            continue;
        }
        if (n_chunks < 0 || n_chunks > p->chunks_cap) return NFFT2D_ERR_INTERNAL;
        p->M = M[i];
        p->n_chunks = n_chunks;
        p->points_valid = true;
        if (p->gather_auto) p->gather_variant = auto_gather(p, M[i]);
    }
    if (status != NFFT2D_OK)  // the error bits are reported here, not again by synchronize
        for (int i = 0; i < count; ++i) cudaMemsetAsync(plans[i]->d_status + 1, 0, sizeof(int), stream);
    return status;
}

int nfft2d::set_points_scaled(nfft2d_plan_s *p, long long M, const void *x1, const void *x2, int coord_dtype,
                              double u1, double u2, double o1, double o2, bool async, cudaEvent_t coords_read) {
    if (!p) return NFFT2D_ERR_INVALID_ARG;
    if (M < 0 || M > 0x7fffffffLL) return NFFT2D_ERR_INVALID_ARG;
    if (coord_dtype != NFFT2D_COORD_F32 && coord_dtype != NFFT2D_COORD_F64) return NFFT2D_ERR_INVALID_ARG;
    if (!(u1 > 0) || !(u2 > 0) || !std::isfinite(u1) || !std::isfinite(u2) || !std::isfinite(o1) ||
        !std::isfinite(o2))
        return NFFT2D_ERR_INVALID_ARG;
    if (M > 0 && (!x1 || !x2)) return NFFT2D_ERR_INVALID_ARG;
    if (M > 0) {
        int st = coord_device_ptr(p, x1, &x1);
        if (st == NFFT2D_OK) st = coord_device_ptr(p, x2, &x2);
        if (st != NFFT2D_OK) return st;
    }
    p->points_valid = false;
    p->M = 0;
    p->n_chunks = 0;
    timer_reset(p, CALL_SORT);
    int st = ensure_points_capacity(p, M);
    if (st != NFFT2D_OK) return st;
    p->workspace_bytes = plan_workspace_bytes(p);
    if (M == 0) {
        p->points_valid = true;
        if (coords_read) NFFT_TRY_CUDA(cudaEventRecord(coords_read, p->stream));
        return NFFT2D_OK;
    }
    const Geom &g = p->g;
    const double s1 = p->sigma * u1, s2 = p->sigma * u2;
    p->xscale1 = s1;
    p->xscale2 = s2;
    // exact FP32 reduction when both scales are powers of two and x is FP32
    int e1 = 0, e2 = 0;
    const bool pow2 = std::frexp(s1, &e1) == 0.5 && std::frexp(s2, &e2) == 0.5;
    const int exact = (coord_dtype == NFFT2D_COORD_F32 && pow2 && o1 == 0.0 && o2 == 0.0) ? 1 : 0;
    const float s1f = static_cast<float>(s1), s2f = static_cast<float>(s2);
    stage_begin(p, ST_SORT);
    NFFT_TRY_CUDA(cudaMemsetAsync(p->d_status, 0, 4 * sizeof(int), p->stream));
    NFFT_TRY_CUDA(cudaMemsetAsync(p->cell_count, 0, sizeof(unsigned) * (p->ncells + 1), p->stream));
    const int Mi = static_cast<int>(M);
    const int blocks = (Mi + 255) / 256;
    // ticket + tile words of the cell scan, then of the work-item scan
    unsigned long long *scan_state = reinterpret_cast<unsigned long long *>(p->scan_tmp);
    constexpr int kCellTile = kCellScanThreads * kCellScanItems, kItemTile = kItemScanThreads * kItemScanItems;
    const size_t item_words = scan_state_words(static_cast<size_t>(g.tiles1) * g.tiles2 + 1, kItemTile);
    const int scan_words = static_cast<int>(scan_state_words(p->ncells + 1, kCellTile) + 2 * item_words);
    // the binning's arrays against L2: coordinates, tmp records, keys and
    // ranks, the inverse permutation, sorted records, cell counters
    const size_t rec_bytes = p->precision == NFFT2D_F64 ? sizeof(Rec64) : sizeof(Rec32);
    const size_t bin_bytes = static_cast<size_t>(M) * ((coord_dtype == NFFT2D_COORD_F64 ? 16 : 8) + 2 * rec_bytes + 12) +
                             4 * (p->ncells + 1);
    const bool stream = bin_bytes > static_cast<size_t>(p->l2_bytes);
    auto bin = [&](auto ct, auto rt, auto st) -> cudaError_t {
        using CT = decltype(ct);
        using RecT = decltype(rt);
        constexpr bool S = decltype(st)::value;
        k_bin_pass1<CT, RecT, S><<<blocks, 256, 0, p->stream>>>(
            static_cast<const CT *>(x1), static_cast<const CT *>(x2), Mi, o1, o2, s1, s2, s1f, s2f, exact, g,
            static_cast<RecT *>(p->tmp_recs), p->keyrank, p->cell_count, p->d_status, scan_state, scan_words);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        if (coords_read && (e = cudaEventRecord(coords_read, p->stream)) != cudaSuccess) return e;  // coordinates read
        const size_t cells_n = p->ncells + 1;
        k_scan_counts<<<static_cast<unsigned>((cells_n + kCellTile - 1) / kCellTile), kCellScanThreads, 0,
                        p->stream>>>(p->cell_count, cells_n, scan_state, p->d_status);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        k_bin_invert<S><<<blocks, 256, 0, p->stream>>>(p->keyrank, p->cell_count, Mi, p->src);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        k_bin_gather<RecT, S><<<blocks, 256, 0, p->stream>>>(static_cast<const RecT *>(p->tmp_recs), p->src, Mi,
                                                              static_cast<RecT *>(p->recs));
        return cudaGetLastError();
    };
    using Yes = std::true_type;
    using No = std::false_type;
    cudaError_t be;
    if (p->precision == NFFT2D_F64) {
        if (coord_dtype == NFFT2D_COORD_F64)
            be = stream ? bin(double{}, Rec64{}, Yes{}) : bin(double{}, Rec64{}, No{});
        else
            be = stream ? bin(float{}, Rec64{}, Yes{}) : bin(float{}, Rec64{}, No{});
    } else {
        if (coord_dtype == NFFT2D_COORD_F64)
            be = stream ? bin(double{}, Rec32{}, Yes{}) : bin(double{}, Rec32{}, No{});
        else
            be = stream ? bin(float{}, Rec32{}, Yes{}) : bin(float{}, Rec32{}, No{});
    }
    NFFT_TRY_CUDA(be);
    const size_t cells_n = p->ncells + 1;
    const int ntiles = g.tiles1 * g.tiles2;
    const unsigned emit_blocks = static_cast<unsigned>((ntiles + 1 + kItemTile - 1) / kItemTile);
    unsigned long long *item_state = scan_state + scan_state_words(cells_n, kCellTile);
    k_scan_emit_chunks<<<emit_blocks, kItemScanThreads, 0, p->stream>>>(
        p->cell_count, ntiles, g.T * g.T, p->chunk, p->chunks, item_state, p->d_status, p->d_status);
    NFFT_TRY_CUDA(cudaGetLastError());
    if (p->chunk > kSpreadItemMax) {  // the spread's own work list, count in status[3]
        k_scan_emit_chunks<<<emit_blocks, kItemScanThreads, 0, p->stream>>>(
            p->cell_count, ntiles, g.T * g.T, kSpreadItemMax, p->items, item_state + item_words, p->d_status,
            p->d_status + 3);
        NFFT_TRY_CUDA(cudaGetLastError());
    }
    stage_end(p, ST_SORT);
    if (p->gather_auto) p->gather_variant = auto_gather(p, M);
    if (async) {
        // the work-item count stays on the device (status[0]); the kernels
        // read it there, nfft2d_synchronize fetches it and reports errors
        p->n_chunks = -1;
        p->M = M;
        p->points_valid = true;
        return NFFT2D_OK;
    }
    const int *hs = p->h_status;  // page-locked: the read-back is one small DMA
    NFFT_TRY_CUDA(cudaMemcpyAsync(p->h_status, p->d_status, 4 * sizeof(int), cudaMemcpyDeviceToHost, p->stream));
    NFFT_TRY_CUDA(cudaStreamSynchronize(p->stream));
    if (hs[1] & kErrNonfinite) return NFFT2D_ERR_NONFINITE;
    if (hs[1] & kErrTimeout) return NFFT2D_ERR_DEVICE_TIMEOUT;
    if (hs[0] < 0 || hs[0] > p->chunks_cap) return NFFT2D_ERR_INTERNAL;
    p->n_chunks = hs[0];
    p->M = M;
    p->points_valid = true;
    return NFFT2D_OK;
}
}  // extern "C++"

extern "C++" {
int nfft2d::type2_with_pad(nfft2d_plan_s *p, int sign, void *f, PadFn pad, const void *ctx) {
    if (!p || !pad) return NFFT2D_ERR_INVALID_ARG;
    if (sign != 1 && sign != -1) return NFFT2D_ERR_INVALID_ARG;
    if (!p->points_valid) return NFFT2D_ERR_NO_POINTS;
    timer_reset(p, CALL_TYPE2);
    if (p->M == 0) return NFFT2D_OK;
    stage_begin(p, ST_PAD);
    NFFT_TRY_CUDA(pad(p, ctx));
    stage_end(p, ST_PAD);
    stage_begin(p, ST_FFT2);
    int st = run_fft(p, sign, true);
    if (st != NFFT2D_OK) return st;
    stage_end(p, ST_FFT2);
    stage_begin(p, ST_FILL);
    NFFT_TRY_CUDA(launch_halo_fill(p));
    stage_end(p, ST_FILL);
    stage_begin(p, ST_GATHER);
    NFFT_TRY_CUDA(launch_gather(p, f));
    stage_end(p, ST_GATHER);
    return NFFT2D_OK;
}
}  // extern "C++"

static int nfft2d_type2_impl(nfft2d_plan p, int sign, const void *F, void *f) {
    if (!p) return NFFT2D_ERR_INVALID_ARG;
    if (sign != 1 && sign != -1) return NFFT2D_ERR_INVALID_ARG;
    if (!p->points_valid) return NFFT2D_ERR_NO_POINTS;
    if (!F || (p->M > 0 && !f)) return NFFT2D_ERR_INVALID_ARG;
    timer_reset(p, CALL_TYPE2);
    if (p->M == 0) return NFFT2D_OK;
    int st = type2_prepare(p, sign, F);
    if (st != NFFT2D_OK) return st;
    stage_begin(p, ST_GATHER);
    NFFT_TRY_CUDA(launch_gather(p, f));
    stage_end(p, ST_GATHER);
    return NFFT2D_OK;
}

static int nfft2d_type1_impl(nfft2d_plan p, int sign, const void *f, void *F) {
    if (!p) return NFFT2D_ERR_INVALID_ARG;
    if (sign != 1 && sign != -1) return NFFT2D_ERR_INVALID_ARG;
    if (!p->points_valid) return NFFT2D_ERR_NO_POINTS;
    if (!F || (p->M > 0 && !f)) return NFFT2D_ERR_INVALID_ARG;
    timer_reset(p, CALL_TYPE1);
    const Geom &g = p->g;
    if (p->M == 0) {
        NFFT_TRY_CUDA(cudaMemsetAsync(F, 0, cplx_size(p->precision) * p->N1 * p->N2, p->stream));
        return NFFT2D_OK;
    }
    stage_begin(p, ST_SPREAD);
    NFFT_TRY_CUDA(cudaMemsetAsync(p->grid, 0, cplx_size(p->precision) * static_cast<size_t>(g.Ra) * g.C, p->stream));
    NFFT_TRY_CUDA(launch_spread(p, f));
    stage_end(p, ST_SPREAD);
    if (use_fused(p)) {  // fold + row FFT, then band-column FFT + crop
        stage_begin(p, ST_FOLD);
        NFFT_TRY_CUDA(fused_type1_rows(p, sign));
        stage_end(p, ST_FOLD);
        stage_begin(p, ST_FFT1);
        NFFT_TRY_CUDA(fused_type1_cols(p, sign, F));
        stage_end(p, ST_FFT1);
        return NFFT2D_OK;
    }
    stage_begin(p, ST_FOLD);
    NFFT_TRY_CUDA(launch_halo_fold(p));
    stage_end(p, ST_FOLD);
    stage_begin(p, ST_FFT1);
    int st = run_fft(p, sign, false);
    if (st != NFFT2D_OK) return st;
    stage_end(p, ST_FFT1);
    stage_begin(p, ST_CROP);
    NFFT_TRY_CUDA(launch_crop(p, F));
    stage_end(p, ST_CROP);
    return NFFT2D_OK;
}

static int nfft2d_grad_x_impl(nfft2d_plan p, int sign, const void *F, const void *v, void *g1, void *g2);

int nfft2d_set_points(nfft2d_plan p, long long M, const void *x1, const void *x2, int coord_dtype, int units) {
    return nfft2d_set_points_impl(p, M, x1, x2, coord_dtype, units, false);
}

int nfft2d_set_points_async(nfft2d_plan p, long long M, const void *x1, const void *x2, int coord_dtype, int units) {
    return nfft2d_set_points_impl(p, M, x1, x2, coord_dtype, units, true);
}

// nfft2d_set_points_async + nfft2d_forward, with the forward's padding and
// FFT (which read only F and the grid) on a second stream, so they run while
// the binning's first pass reads the coordinates (over the host link, for
// page-locked host coordinates) and the rest of the binning runs; the gather
// waits for both.  F in device memory: the second stream starts at once.  F
// in page-locked host memory: it is copied into a staging buffer on the
// second stream once the coordinates have been read, so the two uploads do
// not share the link and F's copy overlaps the rest of the binning.
int nfft2d_bin_and_forward(nfft2d_plan p, long long M, const void *x1, const void *x2, int coord_dtype, int units,
                           const void *F, void *f, void *inputs_read_event) {
    if (!p || !F || (M > 0 && !f)) return NFFT2D_ERR_INVALID_ARG;
    if (units != NFFT2D_UNITS_GRID && units != NFFT2D_UNITS_UNIT && units != NFFT2D_UNITS_RADIANS)
        return NFFT2D_ERR_INVALID_ARG;
    if (p->grid_external) return NFFT2D_ERR_UNSUPPORTED;  // batch plans: the batch runs the FFTs
    cudaPointerAttributes fa;
    if (cudaPointerGetAttributes(&fa, F) != cudaSuccess) {
        cudaGetLastError();
        return NFFT2D_ERR_INVALID_ARG;
    }
    const bool F_host = fa.type == cudaMemoryTypeHost;
    if (!F_host && fa.type != cudaMemoryTypeDevice && fa.type != cudaMemoryTypeManaged)
        return NFFT2D_ERR_INVALID_ARG;  // pageable host memory
    const size_t F_bytes = static_cast<size_t>(p->N1) * p->N2 * (p->precision == NFFT2D_F64 ? 16 : 8);
    const double u1 = units == NFFT2D_UNITS_GRID ? 1.0 : (units == NFFT2D_UNITS_UNIT ? p->N1 : p->N1 / (2.0 * kPi));
    const double u2 = units == NFFT2D_UNITS_GRID ? 1.0 : (units == NFFT2D_UNITS_UNIT ? p->N2 : p->N2 / (2.0 * kPi));
    if (!p->aux) NFFT_TRY_CUDA(cudaStreamCreateWithFlags(&p->aux, cudaStreamNonBlocking));
    if (!p->ev_fork) NFFT_TRY_CUDA(cudaEventCreateWithFlags(&p->ev_fork, cudaEventDisableTiming));
    if (!p->ev_join) NFFT_TRY_CUDA(cudaEventCreateWithFlags(&p->ev_join, cudaEventDisableTiming));
    if (!p->ev_coords) NFFT_TRY_CUDA(cudaEventCreateWithFlags(&p->ev_coords, cudaEventDisableTiming));
    if (F_host && p->F_stage_bytes < F_bytes) {
        NFFT_TRY_CUDA(cudaStreamSynchronize(p->aux));  // the staging buffer's last reader
        plan_free(p->F_stage);
        p->F_stage = nullptr;
        p->F_stage_bytes = 0;
        NFFT_TRY_CUDA(plan_malloc(&p->F_stage, F_bytes));
        p->F_stage_bytes = F_bytes;
    }
    const cudaStream_t main = p->stream;
    NFFT_TRY_CUDA(cudaEventRecord(p->ev_fork, main));
    NFFT_TRY_CUDA(cudaStreamWaitEvent(p->aux, p->ev_fork, 0));
    // inputs_read_event marks the host inputs read: the coordinates, and F
    // too when it comes from the host (then recorded after F's copy)
    const cudaEvent_t user_ev = static_cast<cudaEvent_t>(inputs_read_event);
    const cudaEvent_t coords_read = (F_host || !user_ev) ? p->ev_coords : user_ev;
    timer_reset(p, CALL_TYPE2);
    int st = nfft2d::set_points_scaled(p, M, x1, x2, coord_dtype, u1, u2, 0.0, 0.0, true, coords_read);
    if (st != NFFT2D_OK) return st;
    // pad + FFT (+ halo fill) on the second stream: every launch of the
    // plan goes to p->stream, and the cuFFT plans to their bound stream
    auto bind = [&](cudaStream_t s) {
        p->stream = s;
        if (p->fft_ok) cufftSetStream(p->fft, s);
        if (p->pruned_ok) {
            cufftSetStream(p->fft_rows, s);
            cufftSetStream(p->fft_cols, s);
        }
    };
    const void *Fd = F;
    if (F_host) {
        NFFT_TRY_CUDA(cudaStreamWaitEvent(p->aux, coords_read, 0));
        NFFT_TRY_CUDA(cudaMemcpyAsync(p->F_stage, F, F_bytes, cudaMemcpyHostToDevice, p->aux));
        if (user_ev) NFFT_TRY_CUDA(cudaEventRecord(user_ev, p->aux));
        Fd = p->F_stage;
    }
    bind(p->aux);
    st = type2_prepare(p, -1, Fd);  // NFFT1_2D.m: exp(-i)
    bind(main);
    if (st != NFFT2D_OK) return st;
    NFFT_TRY_CUDA(cudaEventRecord(p->ev_join, p->aux));
    NFFT_TRY_CUDA(cudaStreamWaitEvent(main, p->ev_join, 0));
    if (M == 0) return NFFT2D_OK;
    stage_begin(p, ST_GATHER);
    NFFT_TRY_CUDA(launch_gather(p, f));
    stage_end(p, ST_GATHER);
    return NFFT2D_OK;
}

int nfft2d_type2(nfft2d_plan p, int sign, const void *F, void *f) {
    const int st = nfft2d_type2_impl(p, sign, F, f);
    return st;
}

int nfft2d_type1(nfft2d_plan p, int sign, const void *f, void *F) {
    const int st = nfft2d_type1_impl(p, sign, f, F);
    return st;
}

int nfft2d_grad_x(nfft2d_plan p, int sign, const void *F, const void *v, void *g1, void *g2) {
    const int st = nfft2d_grad_x_impl(p, sign, F, v, g1, g2);
    return st;
}

int nfft2d_forward(nfft2d_plan p, const void *F, void *f) { return nfft2d_type2(p, -1, F, f); }
int nfft2d_adjoint(nfft2d_plan p, const void *f, void *F) { return nfft2d_type1(p, +1, f, F); }
int nfft2d_spread_ref(nfft2d_plan p, const void *f, void *F) { return nfft2d_type1(p, -1, f, F); }

static int nfft2d_grad_x_impl(nfft2d_plan p, int sign, const void *F, const void *v, void *g1, void *g2) {
    if (!p) return NFFT2D_ERR_INVALID_ARG;
    if (sign != 1 && sign != -1) return NFFT2D_ERR_INVALID_ARG;
    if (!p->points_valid) return NFFT2D_ERR_NO_POINTS;
    if (!F || (p->M > 0 && (!v || !g1 || !g2))) return NFFT2D_ERR_INVALID_ARG;
    timer_reset(p, CALL_TYPE2);
    if (p->M == 0) return NFFT2D_OK;
    int st = type2_prepare(p, sign, F);
    if (st != NFFT2D_OK) return st;
    stage_begin(p, ST_GATHER);
    NFFT_TRY_CUDA(launch_grad(p, v, g1, g2));
    stage_end(p, ST_GATHER);
    return NFFT2D_OK;
}

int nfft2d_synchronize(nfft2d_plan p) {
    if (!p) return NFFT2D_ERR_INVALID_ARG;
    NFFT_TRY_CUDA(cudaMemcpyAsync(p->h_status, p->d_status, 4 * sizeof(int), cudaMemcpyDeviceToHost, p->stream));
    NFFT_TRY_CUDA(cudaStreamSynchronize(p->stream));
    NFFT_TRY_CUDA(cudaGetLastError());
    return nfft2d::apply_status(p);
}
}  // extern "C"

// The status words already copied to p->h_status (the stream idle since):
// completes an asynchronous set_points and reports (then clears) the
// device-side error bits.
int nfft2d::apply_status(nfft2d_plan_s *p) {
    const int *hs = p->h_status;
    if (p->points_valid && p->n_chunks < 0) {  // points set by nfft2d_set_points_async
        if (hs[1] & kErrNonfinite) {
            p->points_valid = false;
            p->M = 0;
            p->n_chunks = 0;
            return NFFT2D_ERR_NONFINITE;
        }
        if (hs[0] < 0 || hs[0] > p->chunks_cap) return NFFT2D_ERR_INTERNAL;
        p->n_chunks = hs[0];
    }
    // a device-side error is reported once: the bits are cleared after
    // they are read (the stream is idle here)
    const int bits = hs[1];
    if (bits) NFFT_TRY_CUDA(cudaMemsetAsync(p->d_status + 1, 0, sizeof(int), p->stream));
    if (bits & kErrTimeout) return NFFT2D_ERR_DEVICE_TIMEOUT;
    if (bits & kErrBounds) return NFFT2D_ERR_DEVICE_BOUNDS;
    return NFFT2D_OK;
}

extern "C" {
int nfft2d_get_permutation(nfft2d_plan p, int *perm) {
    if (!p || !perm) return NFFT2D_ERR_INVALID_ARG;
    if (!p->points_valid) return NFFT2D_ERR_NO_POINTS;
    if (p->M == 0) return NFFT2D_OK;
    // the binning's inverse permutation is exactly this array
    NFFT_TRY_CUDA(cudaMemcpyAsync(perm, p->src, sizeof(int) * static_cast<size_t>(p->M), cudaMemcpyDeviceToDevice,
                                  p->stream));
    return NFFT2D_OK;
}

int nfft2d_plan_selftest_wait_timeout(nfft2d_plan p, int spin_limit) {
    if (!p || spin_limit < 1) return NFFT2D_ERR_INVALID_ARG;
    nfft2d::k_selftest_latch<<<1, 32, 0, p->stream>>>(static_cast<uint32_t>(spin_limit), p->d_status);
    NFFT_TRY_CUDA(cudaGetLastError());
    return NFFT2D_OK;
}

int nfft2d_enable_timing(nfft2d_plan p, int on) {
    if (!p) return NFFT2D_ERR_INVALID_ARG;
    if (on)
        for (auto &ev : p->timer.ev)
            if (!ev) NFFT_TRY_CUDA(cudaEventCreate(&ev));
    p->timer.on = on != 0;
    for (bool &u : p->timer.used) u = false;
    return NFFT2D_OK;
}

int nfft2d_get_timings(nfft2d_plan p, nfft2d_timings *t) {
    if (!p || !t) return NFFT2D_ERR_INVALID_ARG;
    std::memset(t, 0, sizeof(*t));
    if (!p->timer.on) return NFFT2D_OK;
    NFFT_TRY_CUDA(cudaStreamSynchronize(p->stream));
    float *fields[ST_COUNT] = {&t->sort_ms,   &t->pad_ms,  &t->fft_type2_ms, &t->halo_fill_ms, &t->gather_ms,
                               &t->spread_ms, &t->fold_ms, &t->fft_type1_ms, &t->crop_ms};
    for (int s = 0; s < ST_COUNT; ++s) {
        if (!p->timer.used[s]) continue;
        float ms = 0;
        NFFT_TRY_CUDA(cudaEventElapsedTime(&ms, p->timer.ev[2 * s], p->timer.ev[2 * s + 1]));
        *fields[s] = ms;
    }
    return NFFT2D_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// cuFFT plan pool
// ---------------------------------------------------------------------------
namespace {
struct FftKey {
    int v[20];
    bool operator==(const FftKey &o) const { return std::memcmp(v, o.v, sizeof v) == 0; }
};
struct FftEntry {
    FftKey key;
    cufftHandle h;
    size_t bytes;
};
constexpr size_t kFftPoolPlans = 256;
constexpr size_t kFftPoolBytes = size_t(1) << 30;
std::mutex g_fft_mu;
std::vector<FftEntry> g_fft_free;  // released plans, oldest first
std::vector<FftEntry> g_fft_live;  // plans handed out
size_t g_fft_free_bytes = 0;

FftKey fft_key(int rank, const int *n, const int *inembed, int istride, int idist, const int *onembed, int ostride,
               int odist, cufftType type, int batch) {
    FftKey k;
    std::memset(k.v, 0, sizeof k.v);
    int dev = 0;
    cudaGetDevice(&dev);
    k.v[0] = dev;
    k.v[1] = rank;
    k.v[2] = static_cast<int>(type);
    k.v[3] = batch;
    k.v[4] = inembed ? 1 : 0;
    k.v[5] = onembed ? 1 : 0;
    k.v[6] = istride;
    k.v[7] = idist;
    k.v[8] = ostride;
    k.v[9] = odist;
    for (int d = 0; d < rank && d < 3; ++d) {
        k.v[10 + d] = n[d];
        k.v[13 + d] = inembed ? inembed[d] : 0;
        k.v[16 + d] = onembed ? onembed[d] : 0;
    }
    return k;
}
}  // namespace

cufftResult nfft2d::pooled_plan_many(cufftHandle *out, int rank, const int *n, const int *inembed, int istride,
                                     int idist, const int *onembed, int ostride, int odist, cufftType type,
                                     int batch) {
    if (rank < 1 || rank > 3) return CUFFT_INVALID_VALUE;
    const FftKey key = fft_key(rank, n, inembed, istride, idist, onembed, ostride, odist, type, batch);
    {
        std::lock_guard<std::mutex> lock(g_fft_mu);
        for (size_t i = g_fft_free.size(); i-- > 0;)
            if (g_fft_free[i].key == key) {
                const FftEntry e = g_fft_free[i];
                g_fft_free.erase(g_fft_free.begin() + static_cast<long>(i));
                g_fft_free_bytes -= e.bytes;
                g_fft_live.push_back(e);
                *out = e.h;
                return CUFFT_SUCCESS;
            }
    }
    cufftHandle h;
    cufftResult r = cufftPlanMany(&h, rank, const_cast<int *>(n), const_cast<int *>(inembed), istride, idist,
                                  const_cast<int *>(onembed), ostride, odist, type, batch);
    if (r != CUFFT_SUCCESS) return r;
    size_t bytes = 0;
    if (cufftGetSize(h, &bytes) != CUFFT_SUCCESS) bytes = 0;
    std::lock_guard<std::mutex> lock(g_fft_mu);
    g_fft_live.push_back({key, h, bytes});
    *out = h;
    return CUFFT_SUCCESS;
}

cufftResult nfft2d::pooled_plan_2d(cufftHandle *out, int nx, int ny, cufftType type) {
    const int n[2] = {nx, ny};
    return pooled_plan_many(out, 2, n, nullptr, 1, 0, nullptr, 1, 0, type, 1);
}

void nfft2d::pooled_plan_release(cufftHandle h) {
    std::vector<cufftHandle> drop;
    {
        std::lock_guard<std::mutex> lock(g_fft_mu);
        size_t i = 0;
        while (i < g_fft_live.size() && g_fft_live[i].h != h) ++i;
        if (i == g_fft_live.size()) {
            drop.push_back(h);  // not from the pool
        } else {
            const FftEntry e = g_fft_live[i];
            g_fft_live.erase(g_fft_live.begin() + static_cast<long>(i));
            g_fft_free.push_back(e);
            g_fft_free_bytes += e.bytes;
            while (!g_fft_free.empty() &&
                   (g_fft_free.size() > kFftPoolPlans || g_fft_free_bytes > kFftPoolBytes)) {
                drop.push_back(g_fft_free.front().h);
                g_fft_free_bytes -= g_fft_free.front().bytes;
                g_fft_free.erase(g_fft_free.begin());
            }
        }
    }
    for (cufftHandle d : drop) cufftDestroy(d);
}

