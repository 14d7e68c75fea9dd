// nfft2d_internal.h -- plan object and launcher declarations shared by the
// translation units of libnfft2d_gb300.so (host side, C++17).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <cufft.h>
#include <stdint.h>

#include "../../include/nfft2d_gb300.h"

namespace nfft2d {

constexpr int kHalo = 8;          // periodic halo around the oversampled grid (>= K rounded up to even)
constexpr int kMinK = 2;
constexpr int kMaxK = 8;

// Device-side error bits latched in Plan::d_status[1].
constexpr int kErrTimeout = 1;
constexpr int kErrBounds = 2;
constexpr int kErrNonfinite = 4;

// One binned point, FP32 plans: fractional offsets t = sigma*x_grid - mu in
// [-1/2, 1/2], packed wrapped cell (mu1 << 16 | mu2) and the caller's index.
struct __align__(16) Rec32 {
    float t1, t2;
    int mu;
    int orig;
};
// FP64 plans keep the offsets in double.
struct __align__(8) Rec64 {
    double t1, t2;
    int mu;
    int orig;
};

// The FP32 window as polynomials: tap a (grid offset m = a - K) of a point
// with fractional offset t in [-1/2, 1/2] is w(t - m) = sum_d c[d][a] t^d,
// degree kPolyDegree(K); fitted in FP64 at plan time (Chebyshev nodes), max
// error < 1e-9 against the closed form for every sigma >= 1.25, 2 <= K <= 8.
// The kernels evaluate all taps by Horner steps on FP32 FMAs, no special
// functions (piecewise-polynomial kernel evaluation, as published for
// FINUFFT by Barnett, Magland and af Klinteberg, SIAM J. Sci. Comput. 2019).
constexpr int kPolyCoef = 11;
__host__ __device__ constexpr int poly_degree(int K) { return K <= 3 ? 10 : 9; }
struct __align__(8) WinPoly {
    float c[kPolyCoef][2 * kMaxK + 2];  // rows padded to an even length: tap pairs are 8-byte aligned
};

// Fit the polynomials of the window for (sigma, K); returns the max abs
// error of the FP64 fit on a dense grid (negative on invalid arguments).
double fit_window_poly(double sigma, int K, WinPoly *out);

// Window constants of one plan (both precisions are filled).
struct WinConst {
    double alpha;   // (2 - 1/sigma) pi - 0.01  (NFFT1_2D.m:11, NFFT2_2D.cu:27)
    double cn;      // K / sinh(alpha K): normalises phi_hat to 1 at t = 0
    double kp;      // K / (1 - exp(-2 alpha K)) = cn * exp(alpha K) / 2
};

// The FP32 tiled spread splits each 16 x 16 tile into vertical strips of SW
// columns; a group of G lanes owns the G patch columns a strip's windows can
// touch (SW + 2K <= G), and 32 / G groups add different points of one strip
// at once.  The binning orders a tile's cells strip by strip (row-major
// within a strip) so that a strip's points are contiguous and row-sorted.
__host__ __device__ constexpr int spread_group_lanes(int K) { return K <= 3 ? 8 : (K <= 7 ? 16 : 32); }
__host__ __device__ constexpr int pow2_floor(int v) {
    int p = 1;
    while (p * 2 <= v) p *= 2;
    return p;
}
__host__ __device__ constexpr int spread_strip_width(int K) { return pow2_floor(spread_group_lanes(K) - 2 * K); }
// Largest work item of the tiled spread: plans with larger chunks (which the
// tiled gather prefers) get a second work list cut at this size.
constexpr int kSpreadItemMax = 512;

// Geometry shared by kernels.
struct Geom {
    int n1, n2;         // oversampled grid
    int H;              // halo
    int R, C;           // padded grid: logical rows n1+2H, row pitch tiles2*T+2H (complex elements)
    int Ra;             // allocated rows tiles1*T+2H: every tile patch box lies inside the allocation
    int Cl;             // logical columns n2+2H
    int T;              // tile edge
    int tiles1, tiles2;
    int PR, PC;         // patch rows / cols (complex elements)
    int Ke;             // K rounded up to even (column halo of a patch)
    int SW;             // strip width of the in-tile cell order (T: plain row-major)
};

// Per-stage CUDA events on the plan's stream: ev[2s], ev[2s+1] bracket stage s.
constexpr int kStages = 9;
struct Timer {
    bool on = false;
    cudaEvent_t ev[2 * kStages] = {};
    bool used[kStages] = {};
    uint64_t nvtx[kStages] = {};  // open NVTX range of each stage (host-side trace)
};

}  // namespace nfft2d

struct nfft2d_plan_s {
    int N1 = 0, N2 = 0, K = 0, precision = 0;
    double sigma = 2.0;
    nfft2d::Geom g{};
    nfft2d::WinConst w{};
    nfft2d::WinPoly poly{};      // FP32 window polynomials
    int chunk = 256;
    int gather_variant = NFFT2D_VARIANT_TILED;
    bool gather_auto = true;     // FP32: pick the gather by bin density at set_points
    int spread_variant = NFFT2D_VARIANT_TILED;
    int compensated = 1;
    int binned_io = 0;           // per-point arrays (f, v, g) in binned order, see nfft2d_tuning.io_order
    int device = 0;
    int num_sms = 0;
    int l2_bytes = 0;
    cudaStream_t stream = nullptr;

    // device buffers owned by the plan
    void *grid = nullptr;        // R*C complex, the padded oversampled grid
    bool grid_external = false;  // grid owned by a batch (no free, no own cuFFT plan)
    void *deap1 = nullptr;       // N1 reals: S / phi(xi_k1), plan precision
    void *deap2 = nullptr;       // N2 reals
    int *d_status = nullptr;     // [0] n_chunks, [1] error bits
    int *h_status = nullptr;     // page-locked host copy of d_status
    unsigned *cell_count = nullptr;  // ncells + 1 counters / starts
    size_t ncells = 0;
    unsigned *scan_tmp = nullptr;
    size_t scan_tmp_elems = 0;

    // points
    long long M = 0;             // points set (0: none)
    bool points_valid = false;
    long long capM = 0;
    void *recs = nullptr;        // sorted Rec32/Rec64
    void *tmp_recs = nullptr;    // unsorted records (caller order)
    uint2 *keyrank = nullptr;    // per point: cell key, rank within the cell
    int *src = nullptr;          // per sorted position: the caller index
    int4 *chunks = nullptr;
    long long chunks_cap = 0;
    // the tiled spread's work items when chunk > kSpreadItemMax: the same
    // tiles cut into items of kSpreadItemMax points (count in d_status[3])
    int4 *items = nullptr;
    long long items_cap = 0;
    long long n_chunks = 0;
    double xscale1 = 1.0, xscale2 = 1.0;  // dt/dx for the units given to set_points

    bool strips = true;  // strip-major cell order (false: row-major, a gather-only plan)
    cudaStream_t aux = nullptr;                         // second stream of nfft2d_bin_and_forward
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;   // its fork and join
    cudaEvent_t ev_coords = nullptr;                    // its coordinates-read mark
    void *F_stage = nullptr;                            // its device copy of a host F
    size_t F_stage_bytes = 0;
    cufftHandle fft = 0;
    bool fft_ok = false;
    cufftHandle fft_rows = 0, fft_cols = 0;  // pruned 1D passes (see run_fft)
    bool pruned_ok = false;
    int fft_mode = -1;                       // -1 auto, 0 2D plan, 1 pruned passes, 2 fused passes
    bool fused_ok = false;                   // twiddle tables of the fused passes are set up
    float2 *tw1 = nullptr, *tw2 = nullptr;   // exp(-2 pi i m / n1), exp(-2 pi i m / n2)
    CUtensorMap tmap;  // 64-byte aligned by its own declaration
    CUtensorMap tmap_spread;  // box of one strip patch of the FP32 tiled spread
    bool tmap_ok = false;

    nfft2d::Timer timer;
    nfft2d_timings last{};
    size_t workspace_bytes = 0;
};

namespace nfft2d {

// ---- launchers (defined in the .cu files) --------------------------------
// plan.cu
cudaError_t launch_pad(const nfft2d_plan_s *p, const void *F);
cudaError_t launch_crop(const nfft2d_plan_s *p, void *F);
cudaError_t launch_halo_fill(const nfft2d_plan_s *p);
cudaError_t launch_halo_fold(const nfft2d_plan_s *p);

// gather.cu
cudaError_t launch_gather(const nfft2d_plan_s *p, void *f);
cudaError_t launch_grad(const nfft2d_plan_s *p, const void *v, void *g1, void *g2);
int gather_smem_bytes(const nfft2d_plan_s *p);

// spread.cu
cudaError_t launch_spread(const nfft2d_plan_s *p, const void *f);

// Geometry for given parameters; returns NFFT2D_OK or an error status.
// strips = false bins a tile's cells row by row (strip width = tile): for
// plans that only gather, whose warps then read fewer distinct rows; their
// spreads take the direct kernel.
int compute_layout(int N1, int N2, double sigma, int K, int precision, int tile, Geom *g, int *n1, int *n2,
                   bool strips = true);

int grid_blocks(const nfft2d_plan_s *p, const void *kernel, int threads, int smem);

// Plan creation shared by nfft2d_plan_create and batches.  With ext_grid set
// the plan works on that (zeroed, Ra x C) grid instead of allocating one and
// creates no cuFFT plan of its own (the batch runs the FFTs); tile = 0 picks
// the default tile.
int create_plan(nfft2d_plan_s **out, int N1, int N2, double sigma, int K, int precision, int tile,
                cudaStream_t stream, void *ext_grid, bool strips = true);
void release_plan(nfft2d_plan_s *p);
int tensor_map_for(nfft2d_plan_s *p);

// Bin points whose grid-unit coordinates are (x - o) * u per dimension (the
// public set_points uses o = 0 and u from its units argument).  async: return
// after enqueuing; the work-item count stays on the device (n_chunks = -1)
// until nfft2d_synchronize reads it back with the error bits.  coords_read,
// if given, is recorded once the coordinates have been read (their buffers
// and the host link are free from there).
int set_points_scaled(nfft2d_plan_s *p, long long M, const void *x1, const void *x2, int coord_dtype, double u1,
                      double u2, double o1, double o2, bool async = false, cudaEvent_t coords_read = nullptr);

// cuFFT plans from a process-wide pool keyed by the device and every plan
// parameter: creating a plan of an awkward size costs milliseconds (a
// Bluestein length: 1.4 ms at 98 x 485, 6 ms at 552 x 970 on GB300), and
// callers that build and drop plans of recurring shapes (the FFBP
// recursion's regriddings, repeated type-3 calls, batches) take a released
// one back instead.  A handle is owned by one caller between acquire and
// release (cuFFT plans are not shareable between concurrent executions);
// released handles are kept up to 256 plans / 1 GiB of work area, oldest
// destroyed first.  inembed/onembed may be NULL (the basic layout).
cufftResult pooled_plan_many(cufftHandle *out, int rank, const int *n, const int *inembed, int istride, int idist,
                             const int *onembed, int ostride, int odist, cufftType type, int batch);
cufftResult pooled_plan_2d(cufftHandle *out, int nx, int ny, cufftType type);
void pooled_plan_release(cufftHandle h);

// One transform's binning job for bin_small_batch (device copy).
struct SmallBinJob {
    const void *x1, *x2;  // DEVICE coordinates (FP32 or FP64 as the batch's call)
    int M;
    double s1, s2;        // sigma * unit scale per dimension
    float s1f, s2f;
    int exact;            // exact FP32 reduction (power-of-two scales, FP32 data)
    Geom g;
    Rec32 *tmp;           // the plan's buffers
    uint2 *keyrank;
    Rec32 *recs;
    int *src;
    int4 *chunks;
    int chunk;
    int *status;          // the plan's status words ([0] work items, [1] error bits)
    int *out;             // work items and error bits, read back by the host
};

// Bin the points of `count` FP32 plans (a batch's transforms) with one
// launch: one CTA per transform with its cell counters in shared memory.
// Same result as nfft2d_set_points on each plan (units: NFFT2D_UNITS_*);
// synchronizes once.  NFFT2D_ERR_UNSUPPORTED when a plan's cells
// do not fit in shared memory or a transform has more than 2^24 points
// (the caller bins those per plan).
int bin_small_batch(nfft2d_plan_s *const *plans, const long long *M, const void *const *x1,
                    const void *const *x2, int coord_dtype, int units, int count, cudaStream_t stream);

// After the plan's status words were copied to p->h_status and its stream
// went idle: completes a set_points enqueued by nfft2d_set_points_async
// (the work-item count) and reports, then clears, the latched device-side
// error bits -- the tail of nfft2d_synchronize, for callers that fetch
// many plans' status words with one synchronisation.
int apply_status(nfft2d_plan_s *p);

// A type-2 transform whose deapodized, zero-padded coefficients are written
// into the grid interior by `pad` (launched on the plan's stream, timed as
// the pad stage) instead of by the plan's own pad kernel; then FFT, halo
// fill and gather as nfft2d_type2.
typedef cudaError_t (*PadFn)(const nfft2d_plan_s *p, const void *ctx);
int type2_with_pad(nfft2d_plan_s *p, int sign, void *f, PadFn pad, const void *ctx);

// Device and page-locked allocations of plan buffers (cached, see
// nfft2d_plan.cu), with the host-side allocation-failure hook used by the
// tests (NFFT2D_FAIL_ALLOC_AT).
cudaError_t plan_malloc(void **ptr, size_t bytes);
cudaError_t plan_malloc_host(void **ptr, size_t bytes);
void plan_free_host(void *ptr, size_t bytes);  // the counterpart of plan_malloc_host (same size)
// The counterpart of plan_malloc: the block goes back to the cache (the
// caller has no work on it in flight).  Any other device pointer is freed.
void plan_free(void *ptr);

// The fused FFT passes (nfft2d_fft.cu): eligibility, per-plan twiddle tables,
// type 2 = deapodize/pad + band-column FFT, then row FFT + halo fill;
// type 1 = halo fold + row FFT, then band-column FFT + crop/deapodize.
bool fused_fft_eligible(int precision, int n1, int n2);
int setup_fused_fft(nfft2d_plan_s *p);
cudaError_t fused_type2_cols(const nfft2d_plan_s *p, int sign, const void *F);
cudaError_t fused_type2_rows(const nfft2d_plan_s *p, int sign);
cudaError_t fused_type1_rows(const nfft2d_plan_s *p, int sign);
cudaError_t fused_type1_cols(const nfft2d_plan_s *p, int sign, void *F);

// One thread waits on an mbarrier phase that nothing completes, gives up
// after `limit` polls and latches kErrTimeout in status[1] (the self-tests of
// nfft2d_plan_selftest_wait_timeout / nfft2d_batch_selftest_wait_timeout).
__global__ void k_selftest_latch(uint32_t limit, int *status);

// Host FP64 helpers shared by the plan and the Knab regridder.
double bessel_i0_host(double x);
void deapod_table_host(int N, int n, int K, double alpha, double *out);

}  // namespace nfft2d
