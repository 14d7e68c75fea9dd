// nfft2d_batch.cu -- many independent 2D NFFTs of uneven size in one go.
//
// Layout: one plan per transform (its own binning, records and work list),
// but every padded grid lives in ONE allocation, grouped by size, so the
// FFTs of a size group run as one batched cuFFT call.  Each stage then covers
// all transforms with a single launch: deapodize + pad, halo fill / fold and
// crop walk (transform, row) pairs; the gather runs one thread per binned
// point of all transforms (the transform found by the point's global index,
// taps read straight from its grid, as the single-plan direct gather); the
// spread is a persistent warp kernel over the concatenated work items of all
// transforms (register-resident patches, one TMA reduce-add per item).  Per-transform descriptors -- the
// TMA tensor map, geometry, record and work-item pointers -- sit in device
// memory; the per-call input/output pointers go to a small device table
// copied before each run.  The stage sequence is captured once into a CUDA
// graph and replayed, so a batch costs one graph launch plus that copy.
//
// No reference counterpart: the reference runs one NFFT2_2D_GPU per PSO
// particle in a host loop (Synthesis/PSO/PSO.cu:348, Synthesis.cu:395).
#include <cuda.h>
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <tuple>
#include <new>
#include <vector>

#include "nfft2d_device.cuh"
#include "nfft2d_internal.h"
#include "nfft2d_kargs.cuh"
#include "nfft2d_tile_ops.cuh"

using namespace nfft2d;

namespace {

constexpr int kThreads = 256;
constexpr int kSpreadWarps = 4;

// One transform of a batch, device resident (the tensor map needs 64-byte
// alignment; the struct keeps it first and the array is allocated aligned).
struct alignas(128) BatchDesc {
    CUtensorMap tmap;   // the grid with the spread's strip-patch box
    const Rec32 *recs;
    const int4 *chunks;
    float2 *grid;
    const float *deap1, *deap2;
    Geom g;
    int N1, N2;
    int n_chunks;
    int chunk_base;     // first global work item of this transform
    int row_base;       // first global oversampled row (pad / halo kernels)
    int crop_base;      // first global output row (crop)
    int chunk;          // maximum points per work item
    int point_base;     // first global point of this transform (direct gather)
};

struct BatchIO {
    const float2 *in;  // type 2: F (N1*N2); type 1: f (M)
    float2 *out;       // type 2: f (M);     type 1: F (N1*N2)
};

// Index of the transform whose [base, next base) holds key (bases ascending).
template <int FIELD>
__device__ __forceinline__ int find_transform(const BatchDesc *__restrict__ d, int n, int key) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        const int b = FIELD == 0   ? __ldg(&d[mid].chunk_base)
                      : FIELD == 1 ? __ldg(&d[mid].row_base)
                      : FIELD == 2 ? __ldg(&d[mid].crop_base)
                                   : __ldg(&d[mid].point_base);
        if (b <= key)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// ---- per-row stages over all transforms ------------------------------------
__global__ void k_batch_pad(const BatchDesc *__restrict__ d, int n, const BatchIO *__restrict__ io) {
    const int t = find_transform<1>(d, n, blockIdx.x);
    const BatchDesc &D = d[t];
    const int r = blockIdx.x - D.row_base;
    const int n1 = D.g.n1, n2 = D.g.n2, N1 = D.N1, N2 = D.N2;
    const int k1 = (r < n1 / 2) ? r : r - n1;
    const bool row_in = k1 >= -N1 / 2 && k1 < N1 / 2;
    const int i = k1 + N1 / 2;
    const float s1 = row_in ? D.deap1[i] : 0.f;
    const float2 *F = io[t].in;
    float2 *dst = D.grid + static_cast<size_t>(r + D.g.H) * D.g.C + D.g.H;
    for (int c = threadIdx.x; c < n2; c += blockDim.x) {
        const int k2 = (c < n2 / 2) ? c : c - n2;
        float2 v = make_float2(0.f, 0.f);
        if (row_in && k2 >= -N2 / 2 && k2 < N2 / 2) {
            const int j = k2 + N2 / 2;
            const float s = s1 * D.deap2[j];
            const float2 f = F[static_cast<size_t>(i) * N2 + j];
            v = make_float2(f.x * s, f.y * s);
        }
        dst[c] = v;
    }
}

__global__ void k_batch_crop(const BatchDesc *__restrict__ d, int n, const BatchIO *__restrict__ io) {
    const int t = find_transform<2>(d, n, blockIdx.x);
    const BatchDesc &D = d[t];
    const int i = blockIdx.x - D.crop_base;
    const int N1 = D.N1, N2 = D.N2, n1 = D.g.n1, n2 = D.g.n2;
    const int k1 = i - N1 / 2;
    const int r = k1 < 0 ? k1 + n1 : k1;
    const float s1 = D.deap1[i];
    const float2 *src = D.grid + static_cast<size_t>(r + D.g.H) * D.g.C + D.g.H;
    float2 *F = io[t].out;
    for (int j = threadIdx.x; j < N2; j += blockDim.x) {
        const int k2 = j - N2 / 2;
        const int c = k2 < 0 ? k2 + n2 : k2;
        const float s = s1 * D.deap2[j];
        const float2 g = src[c];
        F[static_cast<size_t>(i) * N2 + j] = make_float2(g.x * s, g.y * s);
    }
}

__device__ __forceinline__ int pmod(int a, int n) {
    int r = a % n;
    return r < 0 ? r + n : r;
}

// Periodic halo fill (type 2) of transform blockIdx.y.
__global__ void k_batch_fill(const BatchDesc *__restrict__ d) {
    const BatchDesc &D = d[blockIdx.y];
    const int n1 = D.g.n1, n2 = D.g.n2, H = D.g.H, C = D.g.C;
    float2 *grid = D.grid;
    const long long top = 2LL * H * C, side = 2LL * H * n1;
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
        grid[static_cast<size_t>(r) * C + c] = grid[static_cast<size_t>(pmod(r - H, n1) + H) * C + pmod(c - H, n2) + H];
    }
}

// Halo fold (type 1) of transform blockIdx.y: each interior cell within H of
// an edge adds its periodic images.
__global__ void k_batch_fold(const BatchDesc *__restrict__ d) {
    const BatchDesc &D = d[blockIdx.y];
    const int n1 = D.g.n1, n2 = D.g.n2, H = D.g.H, C = D.g.C, R = D.g.R, Cl = D.g.Cl;
    float2 *grid = D.grid;
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
        const int pr0 = r + H, pc0 = c + H;
        const int amin = -(pr0 / n1), amax = (R - 1 - pr0) / n1;
        const int bmin = -(pc0 / n2), bmax = (Cl - 1 - pc0) / n2;
        float2 acc = grid[static_cast<size_t>(pr0) * C + pc0];
        for (int a = amin; a <= amax; ++a)
            for (int b = bmin; b <= bmax; ++b) {
                if (a == 0 && b == 0) continue;
                const float2 v = grid[static_cast<size_t>(pr0 + a * n1) * C + (pc0 + b * n2)];
                acc.x += v.x;
                acc.y += v.y;
            }
        grid[static_cast<size_t>(pr0) * C + pc0] = acc;
    }
}

// ---- gather over the points of all transforms --------------------------
// Direct gather over all transforms: one thread per binned point, the
// transform found by its global point index; taps read straight from that
// transform's padded grid (the single-plan FP32 direct gather).
// One launch per window width: transforms [first, first + n) of the batch's
// internal order share K and hold global points [point0, point0 + npoints).
template <int K>
__global__ void __launch_bounds__(kThreads, K <= 6 ? 4 : 3)  // as the single-plan FP32 gather
    k_batch_gather_direct(const BatchDesc *__restrict__ d, int first, int n, const BatchIO *__restrict__ io,
                          int point0, int npoints, const __grid_constant__ WinPoly wp, int *status) {
    const int i = point0 + blockIdx.x * kThreads + threadIdx.x;
    if (i >= point0 + npoints) return;
    const int t = first + find_transform<3>(d + first, n, i);
    const BatchDesc &D = d[t];
    const int4 raw = __ldg(reinterpret_cast<const int4 *>(D.recs) + (i - D.point_base));
    const int mu1 = static_cast<int>(static_cast<unsigned>(raw.z) >> 16), mu2 = raw.z & 0xFFFF;
    const int n1 = __ldg(&D.g.n1), n2 = __ldg(&D.g.n2);
    if (mu1 >= n1 || mu2 >= n2) {
        latch_error(status, kErrBounds);
        return;
    }
    io[t].out[raw.w] = gather_direct_f32<K, true>(D.grid, __ldg(&D.g.H), __ldg(&D.g.C), mu1, mu2, __int_as_float(raw.x),
                                            __int_as_float(raw.y), wp);
}

// ---- persistent spread over the work items of all transforms --------------
// One launch per window width: transforms [first, first + n) hold the global
// work items [chunk0, chunk0 + total).
template <int K>
__global__ void __launch_bounds__(kSpreadWarps * 32)
    k_batch_spread(const BatchDesc *__restrict__ d, int first, int n, const BatchIO *__restrict__ io, int chunk0,
                   int total, Geom g0, const __grid_constant__ WinPoly wp, int *work, int *status) {
    extern __shared__ unsigned char smem_raw[];
    using S = SpreadGeo<K>;
    unsigned char *base = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) &
                                                            ~uintptr_t(127));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float2 *bufs = reinterpret_cast<float2 *>(base) + warp * S::NBUF * S::PATCH;
    float *scr = reinterpret_cast<float *>(reinterpret_cast<float2 *>(base) + kSpreadWarps * S::NBUF * S::PATCH) +
                 warp * S::ROWS * S::SP;
    StripFlush fs{nullptr, bufs, g0.H, 0};
    strip_flush_init<K>(fs, scr);
    for (;;) {  // a warp's work item is one whole chunk, as in the single-plan spread
        int gl = 0;
        if (lane == 0) gl = atomicAdd(work, 1);
        gl = __shfl_sync(0xffffffffu, gl, 0);
        if (gl >= total) break;
        const int gc = chunk0 + gl;
        const int t = first + find_transform<0>(d + first, n, gc);
        const BatchDesc &D = d[t];
        const int4 ch = __ldg(&D.chunks[gc - D.chunk_base]);
        const int tr = ch.x / D.g.tiles2, tc = ch.x - tr * D.g.tiles2;
        fs.map = &D.tmap;  // this transform's grid (strip-patch box)
        spread_item<K>(D.recs, ch.y, ch.z, tr * kRegTile, tc * kRegTile, io[t].in, 0, scr, fs, wp, status);
    }
    if (lane == 0) bulk_wait_all();
}

}  // namespace

// ---------------------------------------------------------------------------
// host object
// ---------------------------------------------------------------------------
struct nfft2d_batch_s {
    int count = 0;
    double sigma = 2.0;
    // transforms are kept in an internal order sorted by (K, N1, N2): each
    // window width and each cuFFT size group is a contiguous range.
    // order[i] is the caller's index of internal transform i.
    std::vector<int> order;
    cudaStream_t user_stream = nullptr;
    cudaStream_t stream = nullptr;  // the batch's own stream (captured into graphs)
    std::vector<nfft2d_plan_s *> plans;
    void *grids = nullptr;
    size_t grid_bytes = 0;
    struct Group {
        int K, N1, N2;
        std::vector<int> members;  // transform indices, contiguous in `grids`
        size_t first_elem = 0;     // element offset of the first member's grid
        cufftHandle fft = 0;
        bool fft_ok = false;
    };
    std::vector<Group> groups;
    BatchDesc *d_desc = nullptr;
    BatchIO *d_io = nullptr;
    BatchIO *h_io = nullptr;  // pinned
    int *d_work = nullptr;    // spread work counter
    int *d_status = nullptr;  // [1] error bits (shared by the batched kernels)
    int total_chunks = 0, total_rows = 0, total_crop = 0, total_points = 0;
    bool points_valid = false;
    bool use_graph = true;
    cudaGraphExec_t graph[3] = {nullptr, nullptr, nullptr};  // type-2 forward, type-1 adjoint, type-1 sign -1
    cudaEvent_t ev_in = nullptr, ev_out = nullptr, ev_io = nullptr;
    bool io_pending = false;
    // transforms [first, first + n) of the internal order share the window
    // width K: one gather and one spread launch each
    struct KGroup {
        int K = 6, first = 0, n = 0;
        int chunk0 = 0, total_chunks = 0;  // their global work items
        int point0 = 0, total_points = 0;  // their global points
        Geom g0{};                         // patch geometry of the width
        WinPoly poly{};                    // window polynomials of the width
    };
    std::vector<KGroup> kgroups;
};

namespace {

void batch_free(nfft2d_batch_s *b) {
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    for (auto &gx : b->graph)
        if (gx) cudaGraphExecDestroy(gx);
    for (auto &gr : b->groups)
        if (gr.fft_ok) pooled_plan_release(gr.fft);
    for (auto *p : b->plans) release_plan(p);
    cudaFree(b->grids);
    cudaFree(b->d_desc);
    cudaFree(b->d_io);
    cudaFreeHost(b->h_io);
    cudaFree(b->d_work);
    cudaFree(b->d_status);
    for (auto e : {b->ev_in, b->ev_out, b->ev_io})
        if (e) cudaEventDestroy(e);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

int status_of(cudaError_t e) {
    if (e == cudaSuccess) return NFFT2D_OK;
    return e == cudaErrorMemoryAllocation ? NFFT2D_ERR_OOM : NFFT2D_ERR_CUDA;
}

#define B_TRY(expr)                                   \
    do {                                              \
        cudaError_t e_ = (expr);                      \
        if (e_ != cudaSuccess) return status_of(e_);  \
    } while (0)

void drop_graphs(nfft2d_batch_s *b) {
    for (auto &gx : b->graph)
        if (gx) {
            cudaGraphExecDestroy(gx);
            gx = nullptr;
        }
}

int run_ffts(nfft2d_batch_s *b, int dir) {
    for (auto &gr : b->groups) {
        const Geom &g = b->plans[gr.members[0]]->g;
        cufftComplex *base = static_cast<cufftComplex *>(b->grids) + gr.first_elem + static_cast<size_t>(g.H) * g.C + g.H;
        if (cufftExecC2C(gr.fft, base, base, dir) != CUFFT_SUCCESS) return NFFT2D_ERR_CUFFT;
    }
    return NFFT2D_OK;
}

template <int K>
int launch_gather(nfft2d_batch_s *b, const nfft2d_batch_s::KGroup &kg) {
    if (kg.total_points == 0) return NFFT2D_OK;
    k_batch_gather_direct<K><<<(kg.total_points + kThreads - 1) / kThreads, kThreads, 0, b->stream>>>(
        b->d_desc, kg.first, kg.n, b->d_io, kg.point0, kg.total_points, kg.poly, b->d_status);
    B_TRY(cudaGetLastError());
    return NFFT2D_OK;
}

template <int K>
int launch_spread(nfft2d_batch_s *b, const nfft2d_batch_s::KGroup &kg, int sms) {
    if (kg.total_chunks == 0) return NFFT2D_OK;
    const int smem = kSpreadWarps * spread_warp_smem_bytes<K>() + 128;
    auto kernel = k_batch_spread<K>;
    if (smem > 48 * 1024) B_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    int per_sm = 0;
    B_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kSpreadWarps * 32, smem));
    const long long items = kg.total_chunks;
    const int blocks = static_cast<int>(std::max(1LL, std::min<long long>((items + kSpreadWarps - 1) / kSpreadWarps,
                                                                    std::max(per_sm, 1) * sms)));
    B_TRY(cudaMemsetAsync(b->d_work, 0, sizeof(int), b->stream));
    kernel<<<blocks, kSpreadWarps * 32, smem, b->stream>>>(b->d_desc, kg.first, kg.n, b->d_io, kg.chunk0,
                                                           kg.total_chunks, kg.g0, kg.poly, b->d_work,
                                                           b->d_status);
    B_TRY(cudaGetLastError());
    return NFFT2D_OK;
}

int launch_gather_k(nfft2d_batch_s *b, const nfft2d_batch_s::KGroup &kg) {
    switch (kg.K) {
        case 2: return launch_gather<2>(b, kg);
        case 3: return launch_gather<3>(b, kg);
        case 4: return launch_gather<4>(b, kg);
        case 5: return launch_gather<5>(b, kg);
        case 6: return launch_gather<6>(b, kg);
        case 7: return launch_gather<7>(b, kg);
        case 8: return launch_gather<8>(b, kg);
        default: return NFFT2D_ERR_INVALID_ARG;
    }
}

int launch_spread_k(nfft2d_batch_s *b, const nfft2d_batch_s::KGroup &kg, int sms) {
    switch (kg.K) {
        case 2: return launch_spread<2>(b, kg, sms);
        case 3: return launch_spread<3>(b, kg, sms);
        case 4: return launch_spread<4>(b, kg, sms);
        case 5: return launch_spread<5>(b, kg, sms);
        case 6: return launch_spread<6>(b, kg, sms);
        case 7: return launch_spread<7>(b, kg, sms);
        case 8: return launch_spread<8>(b, kg, sms);
        default: return NFFT2D_ERR_INVALID_ARG;
    }
}

// type 2: forward (type 2, sign -1); type 1: adjoint (type 1, sign +1);
// type -1: the reference's spreading NFFT2_2D (type 1, sign -1).  The
// elementwise stages and each size group's FFT cover all transforms at once;
// the gather and the spread run once per window width.
int enqueue(nfft2d_batch_s *b, int type) {
    const int n = b->count;
    int sms = 0, dev = 0;
    B_TRY(cudaGetDevice(&dev));
    B_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    if (type == 2) {
        k_batch_pad<<<b->total_rows, kThreads, 0, b->stream>>>(b->d_desc, n, b->d_io);
        B_TRY(cudaGetLastError());
        int st = run_ffts(b, CUFFT_FORWARD);
        if (st != NFFT2D_OK) return st;
        k_batch_fill<<<dim3(16, n), kThreads, 0, b->stream>>>(b->d_desc);
        B_TRY(cudaGetLastError());
        for (const auto &kg : b->kgroups)
            if ((st = launch_gather_k(b, kg)) != NFFT2D_OK) return st;
    } else {
        B_TRY(cudaMemsetAsync(b->grids, 0, b->grid_bytes, b->stream));
        int st;
        for (const auto &kg : b->kgroups)
            if ((st = launch_spread_k(b, kg, sms)) != NFFT2D_OK) return st;
        k_batch_fold<<<dim3(16, n), kThreads, 0, b->stream>>>(b->d_desc);
        B_TRY(cudaGetLastError());
        st = run_ffts(b, type == 1 ? CUFFT_INVERSE : CUFFT_FORWARD);
        if (st != NFFT2D_OK) return st;
        k_batch_crop<<<b->total_crop, kThreads, 0, b->stream>>>(b->d_desc, n, b->d_io);
        B_TRY(cudaGetLastError());
    }
    return NFFT2D_OK;
}

int run(nfft2d_batch_s *b, int type, const void *const *in, void *const *out) {
    if (!b || !in || !out) return NFFT2D_ERR_INVALID_ARG;
    if (!b->points_valid) return NFFT2D_ERR_NO_POINTS;
    // the point-side array of a transform with no points may be null
    for (int i = 0; i < b->count; ++i) {
        const int t = b->order[i];
        const bool empty = b->plans[i]->M == 0;
        const void *coef = type == 2 ? in[t] : out[t];
        const void *pts = type == 2 ? out[t] : in[t];
        if (!coef || (!pts && !empty)) return NFFT2D_ERR_INVALID_ARG;
    }
    // the previous copy of the pointer table must have left the pinned buffer
    if (b->io_pending) B_TRY(cudaEventSynchronize(b->ev_io));
    for (int i = 0; i < b->count; ++i) {  // the table is in the internal order
        b->h_io[i].in = static_cast<const float2 *>(in[b->order[i]]);
        b->h_io[i].out = static_cast<float2 *>(out[b->order[i]]);
    }
    B_TRY(cudaEventRecord(b->ev_in, b->user_stream));
    B_TRY(cudaStreamWaitEvent(b->stream, b->ev_in, 0));
    B_TRY(cudaMemcpyAsync(b->d_io, b->h_io, sizeof(BatchIO) * b->count, cudaMemcpyHostToDevice, b->stream));
    B_TRY(cudaEventRecord(b->ev_io, b->stream));
    b->io_pending = true;
    const int gi = type == 2 ? 0 : (type == 1 ? 1 : 2);
    if (b->use_graph) {
        if (!b->graph[gi]) {
            cudaGraph_t graph = nullptr;
            B_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
            const int st = enqueue(b, type);
            const cudaError_t ec = cudaStreamEndCapture(b->stream, &graph);
            if (st != NFFT2D_OK) {
                if (graph) cudaGraphDestroy(graph);
                return st;
            }
            B_TRY(ec);
            const cudaError_t ei = cudaGraphInstantiate(&b->graph[gi], graph, 0);
            cudaGraphDestroy(graph);
            B_TRY(ei);
        }
        B_TRY(cudaGraphLaunch(b->graph[gi], b->stream));
    } else {
        const int st = enqueue(b, type);
        if (st != NFFT2D_OK) return st;
    }
    B_TRY(cudaEventRecord(b->ev_out, b->stream));
    B_TRY(cudaStreamWaitEvent(b->user_stream, b->ev_out, 0));
    return NFFT2D_OK;
}

}  // namespace

// Far-field step of the reflectarray PSO synthesis, for every particle of a
// batch: the FP32 coordinate scaling of Synthesis/PSO/Synthesis.cu:388-389,
// the reference-sign spread of :395 and the filter of :402.
namespace {
__global__ void k_scale_points(const float *const *__restrict__ X, const float *const *__restrict__ Y, long long M,
                               float sx, float sy, float *__restrict__ xs, float *__restrict__ ys) {
    const int t = blockIdx.y;
    const float *x = X[t], *y = Y[t];
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < M;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        xs[t * M + i] = x[i] * sx;  // vectorMulConstant<float>
        ys[t * M + i] = y[i] * sy;
    }
}
__global__ void k_filter(float2 *const *__restrict__ F, const float *__restrict__ filt, long long n) {
    float2 *f = F[blockIdx.y];
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const float w = filt[i];
        f[i] = make_float2(w * f[i].x, w * f[i].y);  // farFieldFiltering
    }
}
}  // namespace

extern "C" {

int nfft2d_batch_create_k(nfft2d_batch *out, int count, const int *N1, const int *N2, const int *K, double sigma,
                          void *stream) {
    if (!out || count <= 0 || !N1 || !N2 || !K) return NFFT2D_ERR_INVALID_ARG;
    *out = nullptr;
    for (int t = 0; t < count; ++t) {
        Geom g{};
        const int st = compute_layout(N1[t], N2[t], sigma, K[t], NFFT2D_F32, kRegTile, &g, nullptr, nullptr);
        if (st != NFFT2D_OK) return st;
    }
    nfft2d_batch_s *b = new (std::nothrow) nfft2d_batch_s();
    if (!b) return NFFT2D_ERR_OOM;
    auto fail = [&](int s) {
        batch_free(b);
        return s;
    };
    b->count = count;
    b->sigma = sigma;
    b->user_stream = static_cast<cudaStream_t>(stream);
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(NFFT2D_ERR_CUDA);
    for (auto *e : {&b->ev_in, &b->ev_out, &b->ev_io})
        if (cudaEventCreateWithFlags(e, cudaEventDisableTiming) != cudaSuccess) return fail(NFFT2D_ERR_CUDA);

    // internal order by (K, N1, N2); the grid pitch depends on K (the patch
    // padding), so cuFFT size groups are (K, N1, N2) groups, laid out group by
    // group in one allocation
    b->order.resize(count);
    for (int t = 0; t < count; ++t) b->order[t] = t;
    std::stable_sort(b->order.begin(), b->order.end(), [&](int a, int c) {
        return std::make_tuple(K[a], N1[a], N2[a]) < std::make_tuple(K[c], N1[c], N2[c]);
    });
    std::vector<size_t> offset(count);
    size_t elems = 0;
    for (int i = 0; i < count; ++i) {
        const int t = b->order[i];
        if (b->groups.empty() || b->groups.back().K != K[t] || b->groups.back().N1 != N1[t] ||
            b->groups.back().N2 != N2[t]) {
            nfft2d_batch_s::Group gr;
            gr.K = K[t];
            gr.N1 = N1[t];
            gr.N2 = N2[t];
            gr.first_elem = elems;
            b->groups.push_back(gr);
        }
        b->groups.back().members.push_back(i);
        Geom g{};
        compute_layout(N1[t], N2[t], sigma, K[t], NFFT2D_F32, kRegTile, &g, nullptr, nullptr);
        offset[i] = elems;
        elems += static_cast<size_t>(g.Ra) * g.C;
    }
    b->grid_bytes = elems * sizeof(float2);
    // 256 zeroed bytes of slack after the last grid: the direct gather may
    // read one complex past a grid's last row (with weight 0)
    if (cudaMalloc(&b->grids, b->grid_bytes + 256) != cudaSuccess) return fail(NFFT2D_ERR_OOM);
    if (cudaMemsetAsync(b->grids, 0, b->grid_bytes + 256, b->stream) != cudaSuccess) return fail(NFFT2D_ERR_CUDA);
    b->plans.assign(count, nullptr);
    for (int i = 0; i < count; ++i) {
        const int t = b->order[i];
        const int st = create_plan(&b->plans[i], N1[t], N2[t], sigma, K[t], NFFT2D_F32, kRegTile, b->stream,
                                   static_cast<float2 *>(b->grids) + offset[i]);
        if (st != NFFT2D_OK) return fail(st);
    }
    for (auto &gr : b->groups) {
        const Geom &g = b->plans[gr.members[0]]->g;
        int nn[2] = {g.n1, g.n2}, emb[2] = {g.Ra, g.C};
        const int dist = g.Ra * g.C;
        if (pooled_plan_many(&gr.fft, 2, nn, emb, 1, dist, emb, 1, dist, CUFFT_C2C,
                             static_cast<int>(gr.members.size())) != CUFFT_SUCCESS)
            return fail(NFFT2D_ERR_CUFFT);
        gr.fft_ok = true;
        if (cufftSetStream(gr.fft, b->stream) != CUFFT_SUCCESS) return fail(NFFT2D_ERR_CUFFT);
    }
    // window-width groups: contiguous in the internal order
    for (int i = 0; i < count; ++i) {
        const int k = b->plans[i]->K;
        if (b->kgroups.empty() || b->kgroups.back().K != k) {
            nfft2d_batch_s::KGroup kg;
            kg.K = k;
            kg.first = i;
            kg.g0 = b->plans[i]->g;
            kg.poly = b->plans[i]->poly;
            b->kgroups.push_back(kg);
        }
        ++b->kgroups.back().n;
    }
    if (cudaMalloc(&b->d_desc, sizeof(BatchDesc) * count) != cudaSuccess) return fail(NFFT2D_ERR_OOM);
    if (cudaMalloc(&b->d_io, sizeof(BatchIO) * count) != cudaSuccess) return fail(NFFT2D_ERR_OOM);
    if (cudaMallocHost(&b->h_io, sizeof(BatchIO) * count) != cudaSuccess) return fail(NFFT2D_ERR_OOM);
    if (cudaMalloc(&b->d_work, sizeof(int)) != cudaSuccess) return fail(NFFT2D_ERR_OOM);
    if (cudaMalloc(&b->d_status, 4 * sizeof(int)) != cudaSuccess) return fail(NFFT2D_ERR_OOM);
    if (cudaMemsetAsync(b->d_status, 0, 4 * sizeof(int), b->stream) != cudaSuccess) return fail(NFFT2D_ERR_CUDA);
    if (cudaStreamSynchronize(b->stream) != cudaSuccess) return fail(NFFT2D_ERR_CUDA);
    *out = b;
    return NFFT2D_OK;
}

int nfft2d_batch_create(nfft2d_batch *out, int count, const int *N1, const int *N2, double sigma, int K,
                        void *stream) {
    if (count <= 0) return NFFT2D_ERR_INVALID_ARG;
    const std::vector<int> Ks(static_cast<size_t>(count), K);
    return nfft2d_batch_create_k(out, count, N1, N2, Ks.data(), sigma, stream);
}

int nfft2d_batch_destroy(nfft2d_batch b) {
    if (!b) return NFFT2D_ERR_INVALID_ARG;
    batch_free(b);
    return NFFT2D_OK;
}

int nfft2d_batch_set_points(nfft2d_batch b, const long long *M, const void *const *x1, const void *const *x2,
                            int coord_dtype, int units) {
    if (!b || !M || !x1 || !x2) return NFFT2D_ERR_INVALID_ARG;
    b->points_valid = false;
    drop_graphs(b);
    B_TRY(cudaStreamSynchronize(b->stream));
    // one launch bins every transform when their cell counters fit in shared
    // memory (one CTA per transform); otherwise every transform's binning is
    // enqueued without a host round trip and the status words (work-item
    // counts, errors) of all of them come back with one synchronisation
    {
        std::vector<long long> Mi(b->count);
        std::vector<const void *> px(b->count), py(b->count);
        for (int i = 0; i < b->count; ++i) {  // internal order; the arguments are in the caller's
            const int t = b->order[i];
            Mi[i] = M[t];
            px[i] = x1[t];
            py[i] = x2[t];
        }
        int st = bin_small_batch(b->plans.data(), Mi.data(), px.data(), py.data(), coord_dtype, units, b->count,
                                 b->stream);
        if (st == NFFT2D_ERR_UNSUPPORTED) {
            for (int i = 0; i < b->count; ++i) {
                st = nfft2d_set_points_async(b->plans[i], Mi[i], px[i], py[i], coord_dtype, units);
                if (st != NFFT2D_OK) return st;
            }
            for (int i = 0; i < b->count; ++i)
                B_TRY(cudaMemcpyAsync(b->plans[i]->h_status, b->plans[i]->d_status, 4 * sizeof(int),
                                      cudaMemcpyDeviceToHost, b->stream));
            B_TRY(cudaStreamSynchronize(b->stream));
            for (int i = 0; i < b->count; ++i)
                if ((st = apply_status(b->plans[i])) != NFFT2D_OK) return st;
        } else if (st != NFFT2D_OK) {
            return st;
        }
    }
    std::vector<BatchDesc> h(b->count);
    int chunks = 0, rows = 0, crop = 0;
    long long points = 0;
    for (int i = 0; i < b->count; ++i) {
        nfft2d_plan_s *p = b->plans[i];
        BatchDesc &D = h[i];
        std::memset(&D, 0, sizeof(D));
        std::memcpy(&D.tmap, &p->tmap_spread, sizeof(CUtensorMap));
        D.recs = static_cast<const Rec32 *>(p->recs);
        D.chunks = p->chunks;
        D.grid = static_cast<float2 *>(p->grid);
        D.deap1 = static_cast<const float *>(p->deap1);
        D.deap2 = static_cast<const float *>(p->deap2);
        D.g = p->g;
        D.N1 = p->N1;
        D.N2 = p->N2;
        D.n_chunks = static_cast<int>(p->n_chunks);
        D.chunk_base = chunks;
        D.row_base = rows;
        D.crop_base = crop;
        D.chunk = p->chunk;
        D.point_base = static_cast<int>(points);
        points += p->M;
        chunks += D.n_chunks;
        rows += p->g.n1;
        crop += p->N1;
    }
    B_TRY(cudaMemcpy(b->d_desc, h.data(), sizeof(BatchDesc) * b->count, cudaMemcpyHostToDevice));
    if (points > 0x7fffffffLL) return NFFT2D_ERR_INVALID_ARG;  // global point indices are int
    for (auto &kg : b->kgroups) {
        kg.chunk0 = h[kg.first].chunk_base;
        kg.point0 = h[kg.first].point_base;
        const int last = kg.first + kg.n - 1;
        kg.total_chunks = h[last].chunk_base + h[last].n_chunks - kg.chunk0;
        kg.total_points = static_cast<int>(h[last].point_base + b->plans[last]->M - kg.point0);
    }
    b->total_chunks = chunks;
    b->total_points = static_cast<int>(points);
    b->total_rows = rows;
    b->total_crop = crop;
    b->points_valid = true;
    return NFFT2D_OK;
}

int nfft2d_batch_forward(nfft2d_batch b, const void *const *F, void *const *f) { return run(b, 2, F, f); }

int nfft2d_batch_adjoint(nfft2d_batch b, const void *const *f, void *const *F) { return run(b, 1, f, F); }

int nfft2d_batch_spread_ref(nfft2d_batch b, const void *const *f, void *const *F) { return run(b, -1, f, F); }

int nfft2d_batch_far_field(nfft2d_batch b, long long M, const float *const *X, const float *const *Y, float scale_x,
                           float scale_y, const void *const *excitations, const float *filter,
                           void *const *far_field) {
    if (!b || !X || !Y || !excitations || !far_field || M < 0 || M > 0x7fffffffLL) return NFFT2D_ERR_INVALID_ARG;
    const int n = b->count;
    long long cells = -1;
    for (int i = 0; i < n; ++i) {
        const long long c = static_cast<long long>(b->plans[i]->N1) * b->plans[i]->N2;
        if (cells >= 0 && c != cells && filter) return NFFT2D_ERR_INVALID_ARG;  // one filter for one grid size
        cells = c;
        if (M > 0 && (!X[i] || !Y[i])) return NFFT2D_ERR_INVALID_ARG;
    }
    // the caller's coordinates were written on its stream
    B_TRY(cudaEventRecord(b->ev_in, b->user_stream));
    B_TRY(cudaStreamWaitEvent(b->stream, b->ev_in, 0));
    float *xs = nullptr, *ys = nullptr;
    const float **dxy = nullptr;
    const size_t pts = static_cast<size_t>(n) * static_cast<size_t>(M);
    B_TRY(cudaMallocAsync(&xs, sizeof(float) * pts + 16, b->stream));
    B_TRY(cudaMallocAsync(&ys, sizeof(float) * pts + 16, b->stream));
    B_TRY(cudaMallocAsync(&dxy, sizeof(float *) * 2 * n, b->stream));
    std::vector<const float *> hxy(2 * static_cast<size_t>(n));
    for (int i = 0; i < n; ++i) {
        hxy[i] = X[i];
        hxy[n + i] = Y[i];
    }
    int st = NFFT2D_OK;
    if (cudaMemcpyAsync(dxy, hxy.data(), sizeof(float *) * 2 * n, cudaMemcpyHostToDevice, b->stream) != cudaSuccess)
        st = NFFT2D_ERR_CUDA;
    if (st == NFFT2D_OK && M > 0) {
        const dim3 grid(static_cast<unsigned>(std::min<long long>((M + 255) / 256, 64)), static_cast<unsigned>(n));
        k_scale_points<<<grid, 256, 0, b->stream>>>(dxy, dxy + n, M, scale_x, scale_y, xs, ys);
        if (cudaGetLastError() != cudaSuccess) st = NFFT2D_ERR_CUDA;
    }
    if (st == NFFT2D_OK) {
        std::vector<long long> Ms(static_cast<size_t>(n), M);
        std::vector<const void *> px(static_cast<size_t>(n)), py(static_cast<size_t>(n));
        for (int i = 0; i < n; ++i) {
            px[i] = xs + static_cast<size_t>(i) * M;
            py[i] = ys + static_cast<size_t>(i) * M;
        }
        st = nfft2d_batch_set_points(b, Ms.data(), px.data(), py.data(), NFFT2D_COORD_F32, NFFT2D_UNITS_GRID);
    }
    cudaFreeAsync(xs, b->stream);
    cudaFreeAsync(ys, b->stream);
    cudaFreeAsync(dxy, b->stream);
    if (st != NFFT2D_OK) return st;
    if ((st = run(b, -1, excitations, far_field)) != NFFT2D_OK) return st;  // NFFT2_2D_GPU for every particle
    if (filter && cells > 0) {
        float2 **dF = nullptr;
        B_TRY(cudaMallocAsync(&dF, sizeof(float2 *) * n, b->user_stream));
        std::vector<float2 *> hF(static_cast<size_t>(n));
        for (int i = 0; i < n; ++i) hF[i] = static_cast<float2 *>(far_field[i]);
        const cudaError_t e = cudaMemcpyAsync(dF, hF.data(), sizeof(float2 *) * n, cudaMemcpyHostToDevice,
                                              b->user_stream);
        if (e == cudaSuccess) {
            const dim3 grid(static_cast<unsigned>(std::min<long long>((cells + 255) / 256, 64)),
                            static_cast<unsigned>(n));
            k_filter<<<grid, 256, 0, b->user_stream>>>(dF, filter, cells);
        }
        cudaFreeAsync(dF, b->user_stream);
        B_TRY(e);
        B_TRY(cudaGetLastError());
    }
    return NFFT2D_OK;
}

int nfft2d_batch_set_graph(nfft2d_batch b, int on) {
    if (!b) return NFFT2D_ERR_INVALID_ARG;
    b->use_graph = on != 0;
    if (!b->use_graph) drop_graphs(b);
    return NFFT2D_OK;
}

int nfft2d_batch_synchronize(nfft2d_batch b) {
    if (!b) return NFFT2D_ERR_INVALID_ARG;
    int hs[4] = {0, 0, 0, 0};
    B_TRY(cudaStreamSynchronize(b->stream));
    B_TRY(cudaMemcpy(hs, b->d_status, sizeof(hs), cudaMemcpyDeviceToHost));
    // a device-side error is reported once: cleared after it is read
    if (hs[1]) {
        B_TRY(cudaMemsetAsync(b->d_status + 1, 0, sizeof(int), b->stream));
        B_TRY(cudaStreamSynchronize(b->stream));
    }
    if (hs[1] & kErrTimeout) return NFFT2D_ERR_DEVICE_TIMEOUT;
    if (hs[1] & kErrBounds) return NFFT2D_ERR_DEVICE_BOUNDS;
    return NFFT2D_OK;
}

int nfft2d_batch_selftest_wait_timeout(nfft2d_batch b, int spin_limit) {
    if (!b || spin_limit < 1) return NFFT2D_ERR_INVALID_ARG;
    k_selftest_latch<<<1, 32, 0, b->stream>>>(static_cast<uint32_t>(spin_limit), b->d_status);
    B_TRY(cudaGetLastError());
    return NFFT2D_OK;
}

}  // extern "C"
