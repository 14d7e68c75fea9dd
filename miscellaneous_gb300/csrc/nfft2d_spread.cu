// nfft2d_spread.cu -- type-1 windowed spreading of the nonuniform data onto
// the oversampled grid (NFFT/NFFT2/Matlab/NFFT2_2D.m:47-56; the reference GPU
// kernel is Interpolation_NFFT2_2D_GPUKernel + series_terms,
// NFFT/NFFT2_2D.cu:105-276, which launches one 13x13 child grid per point and
// issues 338 global float atomics per point).
//
// TILED variant (FP32 plans, 16 x 16 tiles): a warp pulls work items
// (tile, point range) from a global counter.  The binning orders a tile's
// points by vertical strip (SW columns, 4 at K = 6) and by row within a
// strip; the warp splits into groups of G lanes (16 at K = 6) whose lane l
// owns column l of the strip's patch -- every column the strip's windows
// can touch -- IN REGISTERS, one float2 per patch row.  The groups add
// different points of one row run at once with packed FP32x2 FMAs
// (static register indices: the run's row is warp-uniform), so 2K+1 of G
// lanes do useful work.  No shared-memory or global atomics: when the strip
// changes, each group's patch leaves through shared memory as one TMA tensor
// reduction (cp.reduce.async.bulk.tensor.2d ... .add, f32) into the padded
// grid, which runs while the warp walks the next strip.  The halo of the
// padded grid is folded back onto the interior afterwards (k_halo_fold), so
// no kernel wraps indices.
//
// Why not shared-memory atomics: on this GPU a float atomicAdd to shared
// memory runs as a compare-and-swap loop (measured ~470 instructions per
// point, 0.95 ms for 2^20 uniform points), and clustered points (the polar
// raster's centre holds hundreds of points per cell) serialise it further.
// Here clustered points cost the same as spread-out ones.
//
// DIRECT variant (both precisions): one thread per sorted point, global
// atomics into the padded grid.
#include <cuda.h>
#include <cuda_runtime.h>

#include "nfft2d_device.cuh"
#include "nfft2d_internal.h"
#include "nfft2d_kargs.cuh"
#include "nfft2d_tile_ops.cuh"

namespace nfft2d {
namespace {

constexpr int kThreads = 256;

constexpr int kSpreadWarps = 4;  // warps per CTA of the tiled spread

template <int K>
__global__ void __launch_bounds__(kSpreadWarps * 32) k_spread_tiled(const __grid_constant__ CUtensorMap tmap,
                                                                    const Rec32 *__restrict__ recs,
                                                                    const int4 *__restrict__ chunks, int n_host,
                                                                    const int *__restrict__ n_dev,
                                                                    const float2 *__restrict__ f,
                                                                    const __grid_constant__ KArgs a) {
    extern __shared__ unsigned char smem_raw[];
    using S = SpreadGeo<K>;
    const Geom g = a.g;  // g.T == kRegTile, g.SW == S::SW
    // TMA shared-memory operands: 128-byte aligned (the launch adds 128 bytes of slack)
    unsigned char *base = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) &
                                                            ~uintptr_t(127));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float2 *bufs = reinterpret_cast<float2 *>(base) + warp * S::NBUF * S::PATCH;
    float *scr = reinterpret_cast<float *>(reinterpret_cast<float2 *>(base) + kSpreadWarps * S::NBUF * S::PATCH) +
                 warp * S::ROWS * S::SP;
    const int n = n_host >= 0 ? n_host : *n_dev;  // < 0: counted on the device only
    int *work = a.status + 2;  // work-item counter, zeroed before the launch
    StripFlush fs{&tmap, bufs, g.H, 0};
    strip_flush_init<K>(fs, scr);

    // A warp's work item is one whole entry of the work list: the plan's
    // chunks (up to `chunk` points of one tile), or for chunks above
    // kSpreadItemMax the binning's second list cut at that size.  Splitting
    // chunks into fixed-size parts instead left parts empty wherever a chunk
    // held fewer points, and split one tile's strips between warps (each
    // flushing them) -- 1.08 against 0.97 ms at 2^24 clustered points and
    // 256-point chunks.
    for (;;) {
        int c = 0;
        if (lane == 0) c = atomicAdd(work, 1);
        c = __shfl_sync(0xffffffffu, c, 0);
        if (c >= n) break;
        const int4 ch = __ldg(&chunks[c]);
        const int tr = ch.x / g.tiles2, tc = ch.x - tr * g.tiles2;
        spread_item<K>(recs, ch.y, ch.z, tr * kRegTile, tc * kRegTile, f, a.binned_io, scr, fs, a.poly, a.status);
    }
    if (lane == 0) bulk_wait_all();
}

template <int K, typename Real, typename RecT>
__global__ void __launch_bounds__(kThreads) k_spread_direct(Real *__restrict__ grid, const RecT *__restrict__ recs,
                                                            const Real *__restrict__ f,
                                                            const __grid_constant__ KArgs a) {
    constexpr int W = 2 * K + 1;
    const int i = blockIdx.x * kThreads + threadIdx.x;
    if (i >= a.M) return;
    const RecT r = recs[i];
    const int mu1 = static_cast<int>(static_cast<unsigned>(r.mu) >> 16), mu2 = r.mu & 0xFFFF;
    const Geom g = a.g;
    if (mu1 >= g.n1 || mu2 >= g.n2) {
        latch_error(a.status, kErrBounds);
        return;
    }
    const size_t io = a.binned_io ? static_cast<size_t>(i) : static_cast<size_t>(r.orig);
    const Real vx = f[2 * io], vy = f[2 * io + 1];
    Real w1[W], w2[W];
    if constexpr (sizeof(Real) == 4) {
        weights_poly<K>(r.t1, w1, a.poly);
        weights_poly<K>(r.t2, w2, a.poly);
    } else {
        weights_f64<K>(r.t1, w1, a.alpha_d, a.cn_d);
        weights_f64<K>(r.t2, w2, a.alpha_d, a.cn_d);
    }
    Real *base = grid + 2 * (static_cast<size_t>(mu1 + g.H - K) * g.C + (mu2 + g.H - K));
#pragma unroll
    for (int rr = 0; rr < W; ++rr) {
        const Real ax = vx * w1[rr], ay = vy * w1[rr];
        Real *row = base + 2 * static_cast<size_t>(rr) * g.C;
#pragma unroll
        for (int q = 0; q < W; ++q) {
            atomicAdd(row + 2 * q, ax * w2[q]);
            atomicAdd(row + 2 * q + 1, ay * w2[q]);
        }
    }
}

template <int K>
cudaError_t launch_K(const nfft2d_plan_s *p, const void *f) {
    const KArgs a = make_kargs(p);
    if (p->precision == NFFT2D_F32 && p->spread_variant == NFFT2D_VARIANT_TILED && p->g.T == kRegTile &&
        p->g.SW == SpreadGeo<K>::SW) {
        if (p->n_chunks == 0) return cudaSuccess;
        const int smem = kSpreadWarps * spread_warp_smem_bytes<K>() + 128;
        auto kernel = k_spread_tiled<K>;
        if (smem > 48 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
            if (e != cudaSuccess) return e;
        }
        cudaError_t e = cudaMemsetAsync(p->d_status + 2, 0, sizeof(int), p->stream);
        if (e != cudaSuccess) return e;
        int blocks = grid_blocks(p, reinterpret_cast<const void *>(kernel), kSpreadWarps * 32, smem);
        const bool own_list = p->chunk > kSpreadItemMax;  // its count stays on the device (status[3])
        const int n_host = own_list ? -1 : static_cast<int>(p->n_chunks);
        if (n_host >= 0) {  // else the count is on the device: the full persistent grid
            const int need = (n_host + kSpreadWarps - 1) / kSpreadWarps;
            if (blocks > need) blocks = need;
        }
        kernel<<<blocks, kSpreadWarps * 32, smem, p->stream>>>(
            p->tmap_spread, static_cast<const Rec32 *>(p->recs), own_list ? p->items : p->chunks, n_host,
            p->d_status + (own_list ? 3 : 0), static_cast<const float2 *>(f), a);
        return cudaGetLastError();
    }
    const int blocks = static_cast<int>((p->M + kThreads - 1) / kThreads);
    if (blocks == 0) return cudaSuccess;
    if (p->precision == NFFT2D_F64)
        k_spread_direct<K, double, Rec64><<<blocks, kThreads, 0, p->stream>>>(
            static_cast<double *>(p->grid), static_cast<const Rec64 *>(p->recs), static_cast<const double *>(f), a);
    else
        k_spread_direct<K, float, Rec32><<<blocks, kThreads, 0, p->stream>>>(
            static_cast<float *>(p->grid), static_cast<const Rec32 *>(p->recs), static_cast<const float *>(f), a);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_spread(const nfft2d_plan_s *p, const void *f) {
    switch (p->K) {
        case 2: return launch_K<2>(p, f);
        case 3: return launch_K<3>(p, f);
        case 4: return launch_K<4>(p, f);
        case 5: return launch_K<5>(p, f);
        case 6: return launch_K<6>(p, f);
        case 7: return launch_K<7>(p, f);
        case 8: return launch_K<8>(p, f);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace nfft2d
