// nfft2d_gather.cu -- type-2 windowed gather at the nonuniform points (the
// hot loop of BP_FBP_FFBP/NFFT1_2D.m:61-67) and its derivative w.r.t. the
// point coordinates.
//
// TILED variant (FP32 plans): points are binned into T x T tiles of the
// oversampled grid and sorted row-major by cell inside each tile.  A
// persistent CTA walks work items (tile, point range); for each it stages the
// tile's (T+2K) x (T+2Ke) patch of the padded grid into shared memory with
// one TMA load (cp.async.bulk.tensor.2d, completion on an mbarrier),
// double-buffered so the next patch streams in while the current one is
// consumed.  Each thread evaluates the 2(2K+1) separable window weights of
// its point once and sums the (2K+1)^2 taps from shared memory; adjacent
// lanes hold adjacent cells, so a warp's reads of one tap hit consecutive
// addresses.  Row partial sums use FMA; the sum over rows is compensated
// (TwoSum) when enabled.
//
// DIRECT variant (both precisions): one thread per sorted point reads its
// taps straight from the padded grid (L1/L2), no shared memory.  FP32 plans
// use k_gather_direct_f32 / k_grad_direct_f32 (two taps per 16-byte load,
// bounded registers, compensated row sum in the gather); FP64 plans the
// generic k_gather_direct.
#include <cuda.h>
#include <cuda_runtime.h>

#include "nfft2d_device.cuh"
#include "nfft2d_internal.h"
#include "nfft2d_kargs.cuh"
#include "nfft2d_tile_ops.cuh"

namespace nfft2d {
namespace {

constexpr int kThreads = 256;

template <int K>
__device__ __forceinline__ void issue_patch(const CUtensorMap *map, const int4 *__restrict__ chunks, int c,
                                            float2 *dst, uint64_t *bar, const Geom &g) {
    const int tile = __ldg(&chunks[c].x);
    const int tr = tile / g.tiles2, tc = tile - tr * g.tiles2;
    const int x = 2 * (g.H + tc * g.T - g.Ke);  // FP32 element index, multiple of 4 (16 bytes)
    const int y = g.H + tr * g.T - K;
    mbar_arrive_expect_tx(bar, static_cast<uint32_t>(g.PR * g.PC * sizeof(float2)));
    tma_load_2d(dst, map, bar, x, y);
}

// MODE 0: f = gather(grid);  MODE 1: coordinate gradient contracted with vin.
// CPC > 0 fixes the patch pitch at compile time (all tap loads then use
// immediate offsets); CPC = 0 reads it from the geometry.
template <int K, bool COMP, int MODE, int CPC>
__global__ void __launch_bounds__(kThreads, MODE == 0 ? 4 : 2) k_gather_tiled(const __grid_constant__ CUtensorMap tmap,
                                                           const Rec32 *__restrict__ recs,
                                                           const int4 *__restrict__ chunks, float2 *__restrict__ out,
                                                           const float2 *__restrict__ vin, float *__restrict__ g1,
                                                           float *__restrict__ g2,
                                                           const __grid_constant__ KArgs a) {
    extern __shared__ unsigned char smem_raw[];
    // full[b]: the TMA of patch buffer b landed (one arrival + its bytes);
    // empty[b]: every warp is done with buffer b (one arrival per warp)
    __shared__ __align__(8) uint64_t full[2], empty[2];
    constexpr int kWarps = kThreads / 32;
    constexpr int W = 2 * K + 1;
    const Geom g = a.g;
    const int PC = CPC > 0 ? CPC : g.PC;
    const int pstride = patch_stride_elems(g);
    // TMA shared-memory operands: 128-byte aligned (the launch adds 128 bytes of slack)
    float2 *bufs = reinterpret_cast<float2 *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    const int n = a.n_chunks >= 0 ? a.n_chunks : a.status[0];  // < 0: counted on the device only
    const int lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        mbar_init(&full[0], 1);
        mbar_init(&full[1], 1);
        mbar_init(&empty[0], kWarps);
        mbar_init(&empty[1], kWarps);
        fence_proxy_async_smem();
    }
    __syncthreads();  // the only CTA-wide barrier: the mbarriers are initialised
    if (threadIdx.x == 0 && static_cast<int>(blockIdx.x) < n) issue_patch<K>(&tmap, chunks, blockIdx.x, bufs, &full[0], g);

    int it = 0;
    int pending = static_cast<int>(blockIdx.x) < n ? 0 : -1;  // thread 0: buffer of the last TMA issued
    for (int c = blockIdx.x; c < n; c += gridDim.x, ++it) {
        const int b = it & 1;
        const int cnext = c + gridDim.x;
        bool ok = true;
        if (threadIdx.x == 0 && cnext < n) {
            // the next patch goes to buffer b^1 once every warp is done with
            // its previous use (iteration it - 1)
            if (it >= 1 && !mbar_wait_bounded(&empty[b ^ 1], ((it - 1) >> 1) & 1u)) {
                ok = false;
            } else {
                fence_proxy_async_smem();
                issue_patch<K>(&tmap, chunks, cnext, bufs + (b ^ 1) * pstride, &full[b ^ 1], g);
                pending = b ^ 1;
            }
        }
        // this iteration's patch has landed (each thread acquires it itself)
        if (ok && !mbar_wait_bounded(&full[b], (it >> 1) & 1u)) ok = false;
        // a wait that ran out ends the whole warp at once (no lane is left
        // at a warp barrier); the other warps' own bounded waits then run
        // out in turn
        if (!__all_sync(0xffffffffu, ok)) {
            if (lane == 0) latch_error(a.status, kErrTimeout);
            // never leave with a copy into this CTA's shared memory in flight
            if (threadIdx.x == 0 && pending == (b ^ 1) && cnext < n)
                (void)mbar_wait_bounded(&full[b ^ 1], ((it + 1) >> 1) & 1u);
            return;
        }

        const int4 ch = __ldg(&chunks[c]);
        const int tr = ch.x / g.tiles2, tc = ch.x - tr * g.tiles2;
        const int r0 = tr * g.T, c0 = tc * g.T;
        const float2 *patch = bufs + b * pstride;
        for (int i = threadIdx.x; i < ch.z; i += kThreads) {
            const int4 raw = __ldg(reinterpret_cast<const int4 *>(recs) + ch.y + i);
            const float t1 = __int_as_float(raw.x), t2 = __int_as_float(raw.y);
            const int mu1 = static_cast<int>(static_cast<unsigned>(raw.z) >> 16), mu2 = raw.z & 0xFFFF;
            const int lr = mu1 - r0, lc = mu2 - c0;
            if (static_cast<unsigned>(lr) >= static_cast<unsigned>(g.T) ||
                static_cast<unsigned>(lc) >= static_cast<unsigned>(g.T)) {
                latch_error(a.status, kErrBounds);
                continue;
            }
            const int io = a.binned_io ? ch.y + i : raw.w;  // caller's index or binned position
            if (MODE == 0) {
                out[io] = gather_point<K, COMP>(patch, PC, g.Ke, lr, lc, t1, t2, a.poly);
            } else {
                float w1[W], w2[W], d1[W], d2[W];
                weights_poly_d<K>(t1, w1, d1, a.poly);
                weights_poly_d<K>(t2, w2, d2, a.poly);
                const float2 *base = patch + lr * PC + lc + (g.Ke - K);
                float ax = 0.f, ay = 0.f, bx = 0.f, by = 0.f;
#pragma unroll
                for (int r = 0; r < W; ++r) {
                    const float2 *row = base + r * PC;
                    float rx = 0.f, ry = 0.f, qx = 0.f, qy = 0.f;
#pragma unroll
                    for (int q = 0; q < W; ++q) {
                        const float2 v = row[q];
                        rx = fmaf(w2[q], v.x, rx);
                        ry = fmaf(w2[q], v.y, ry);
                        qx = fmaf(d2[q], v.x, qx);
                        qy = fmaf(d2[q], v.y, qy);
                    }
                    ax = fmaf(d1[r], rx, ax);
                    ay = fmaf(d1[r], ry, ay);
                    bx = fmaf(w1[r], qx, bx);
                    by = fmaf(w1[r], qy, by);
                }
                const float2 v = __ldg(&vin[io]);
                g1[io] = a.ds1 * (v.x * ax + v.y * ay);
                g2[io] = a.ds2 * (v.x * bx + v.y * by);
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[b]);  // this warp is done with buffer b
    }
}

template <typename Real>
struct CxOf;
template <>
struct CxOf<float> {
    using type = float2;
};
template <>
struct CxOf<double> {
    using type = double2;
};

template <int K, typename Real>
__device__ __forceinline__ void weights_any(Real t, Real (&w)[2 * K + 1], const KArgs &a) {
    if constexpr (sizeof(Real) == 4)
        weights_poly<K>(t, w, a.poly);
    else
        weights_f64<K>(t, w, a.alpha_d, a.cn_d);
}

// Slopes dw/dt of the taps; the FP32 path re-evaluates w with them (the
// same Horner steps, so w is unchanged).
template <int K, typename Real>
__device__ __forceinline__ void dweights_any(Real t, Real (&w)[2 * K + 1], Real (&dw)[2 * K + 1], const KArgs &a) {
    if constexpr (sizeof(Real) == 4)
        weights_poly_d<K>(t, w, dw, a.poly);
    else
        dweights_f64<K>(t, dw, a.alpha_d, a.cn_d);
}

template <int K, typename Real, typename RecT, int MODE>
__global__ void __launch_bounds__(kThreads) k_gather_direct(const typename CxOf<Real>::type *__restrict__ grid,
                                                            const RecT *__restrict__ recs,
                                                            typename CxOf<Real>::type *__restrict__ out,
                                                            const typename CxOf<Real>::type *__restrict__ vin,
                                                            Real *__restrict__ g1, Real *__restrict__ g2,
                                                            const __grid_constant__ KArgs a) {
    using Cx = typename CxOf<Real>::type;
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
    const Cx *base = grid + static_cast<size_t>(mu1 + g.H - K) * g.C + (mu2 + g.H - K);
    Real w1[W], w2[W];
    weights_any<K, Real>(static_cast<Real>(r.t1), w1, a);
    weights_any<K, Real>(static_cast<Real>(r.t2), w2, a);
    if constexpr (MODE == 0) {
        Real sx = 0, sy = 0;
#pragma unroll
        for (int rr = 0; rr < W; ++rr) {
            const Cx *row = base + static_cast<size_t>(rr) * g.C;
            Real rx = 0, ry = 0;
#pragma unroll
            for (int q = 0; q < W; ++q) {
                const Cx v = __ldg(row + q);
                rx += w2[q] * v.x;
                ry += w2[q] * v.y;
            }
            sx += w1[rr] * rx;
            sy += w1[rr] * ry;
        }
        Cx o;
        o.x = sx;
        o.y = sy;
        out[a.binned_io ? i : r.orig] = o;
    } else {
        Real d1[W], d2[W];
        dweights_any<K, Real>(static_cast<Real>(r.t1), w1, d1, a);
        dweights_any<K, Real>(static_cast<Real>(r.t2), w2, d2, a);
        Real ax = 0, ay = 0, bx = 0, by = 0;
#pragma unroll
        for (int rr = 0; rr < W; ++rr) {
            const Cx *row = base + static_cast<size_t>(rr) * g.C;
            Real rx = 0, ry = 0, qx = 0, qy = 0;
#pragma unroll
            for (int q = 0; q < W; ++q) {
                const Cx v = __ldg(row + q);
                rx += w2[q] * v.x;
                ry += w2[q] * v.y;
                qx += d2[q] * v.x;
                qy += d2[q] * v.y;
            }
            ax += d1[rr] * rx;
            ay += d1[rr] * ry;
            bx += w1[rr] * qx;
            by += w1[rr] * qy;
        }
        const int io = a.binned_io ? i : r.orig;
        const Cx v = __ldg(&vin[io]);
        if constexpr (sizeof(Real) == 4) {
            g1[io] = a.ds1 * (v.x * ax + v.y * ay);
            g2[io] = a.ds2 * (v.x * bx + v.y * by);
        } else {
            g1[io] = a.ds1_d * (v.x * ax + v.y * ay);
            g2[io] = a.ds2_d * (v.x * bx + v.y * by);
        }
    }
}

// The FP32 forward gather on its own: bounded to 64 registers (K <= 6) or
// 80 (K = 7, 8) so that four or three CTAs share an SM.  Its L1 loads are
// latency-bound, and the compiler's own choice (54 registers at K = 6, with
// fewer loads in flight) measured 9 % slower on GB300 (polar 65.5 -> 59.4 us,
// uniform 67.5 -> 61.3 us at K = 6).
template <int K>
__global__ void __launch_bounds__(kThreads, K <= 6 ? 4 : 3)
    k_gather_direct_f32(const float2 *__restrict__ grid, const Rec32 *__restrict__ recs, float2 *__restrict__ out,
                        const __grid_constant__ KArgs a) {
    const int i = blockIdx.x * kThreads + threadIdx.x;
    if (i >= a.M) return;
    const Rec32 r = recs[i];
    const int mu1 = static_cast<int>(static_cast<unsigned>(r.mu) >> 16), mu2 = r.mu & 0xFFFF;
    const Geom g = a.g;
    if (mu1 >= g.n1 || mu2 >= g.n2) {
        latch_error(a.status, kErrBounds);
        return;
    }
    out[a.binned_io ? i : r.orig] = a.compensated ? gather_direct_f32<K, true>(grid, g.H, g.C, mu1, mu2, r.t1, r.t2, a.poly)
                                : gather_direct_f32<K, false>(grid, g.H, g.C, mu1, mu2, r.t1, r.t2, a.poly);
}

// The FP32 coordinate gradient with the forward gather's 16-byte row loads:
// per row the value and slope column weights (shifted by one for odd starts,
// as in gather_direct_f32) give the partials r = sum w2 v and q = sum dw2 v;
// then d f/d t1 = sum dw1 r and d f/d t2 = sum w1 q.
template <int K>
__global__ void __launch_bounds__(kThreads, K <= 6 ? 3 : 2)
    k_grad_direct_f32(const float2 *__restrict__ grid, const Rec32 *__restrict__ recs,
                      const float2 *__restrict__ vin, float *__restrict__ g1, float *__restrict__ g2,
                      const __grid_constant__ KArgs a) {
    constexpr int W = 2 * K + 1;
    constexpr int V = K + 1;  // float4 loads per row
    const int i = blockIdx.x * kThreads + threadIdx.x;
    if (i >= a.M) return;
    const Rec32 r = recs[i];
    const int mu1 = static_cast<int>(static_cast<unsigned>(r.mu) >> 16), mu2 = r.mu & 0xFFFF;
    const Geom g = a.g;
    if (mu1 >= g.n1 || mu2 >= g.n2) {
        latch_error(a.status, kErrBounds);
        return;
    }
    float w1[W], d1[W], w2[W], d2[W];
    weights_poly_d<K>(r.t1, w1, d1, a.poly);
    weights_poly_d<K>(r.t2, w2, d2, a.poly);
    const int col0 = mu2 + g.H - K;
    const int odd = col0 & 1;
    float ws[2 * V], ds[2 * V];
#pragma unroll
    for (int q = 0; q < 2 * V; ++q) {
        const bool lo_in = q < W, hi_in = q >= 1 && q - 1 < W;
        ws[q] = odd ? (hi_in ? w2[q - 1] : 0.f) : (lo_in ? w2[q] : 0.f);
        ds[q] = odd ? (hi_in ? d2[q - 1] : 0.f) : (lo_in ? d2[q] : 0.f);
    }
    const float4 *rb = reinterpret_cast<const float4 *>(grid + static_cast<size_t>(mu1 + g.H - K) * g.C + (col0 - odd));
    const int pitch4 = g.C >> 1;
    float ax = 0.f, ay = 0.f, bx = 0.f, by = 0.f;
#pragma unroll
    for (int rr = 0; rr < W; ++rr) {
        const float4 *row = rb + rr * pitch4;
        float rx = 0.f, ry = 0.f, qx = 0.f, qy = 0.f;
#pragma unroll
        for (int q = 0; q < V; ++q) {
            const float4 v = __ldg(row + q);
            rx = fmaf(ws[2 * q], v.x, rx);
            ry = fmaf(ws[2 * q], v.y, ry);
            qx = fmaf(ds[2 * q], v.x, qx);
            qy = fmaf(ds[2 * q], v.y, qy);
            rx = fmaf(ws[2 * q + 1], v.z, rx);
            ry = fmaf(ws[2 * q + 1], v.w, ry);
            qx = fmaf(ds[2 * q + 1], v.z, qx);
            qy = fmaf(ds[2 * q + 1], v.w, qy);
        }
        ax = fmaf(d1[rr], rx, ax);
        ay = fmaf(d1[rr], ry, ay);
        bx = fmaf(w1[rr], qx, bx);
        by = fmaf(w1[rr], qy, by);
    }
    const int io = a.binned_io ? i : r.orig;
    const float2 v = __ldg(&vin[io]);
    g1[io] = a.ds1 * (v.x * ax + v.y * ay);
    g2[io] = a.ds2 * (v.x * bx + v.y * by);
}

template <typename KernelT>
cudaError_t prepare_smem(KernelT kernel, int smem) {
    if (smem > 48 * 1024) return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    return cudaSuccess;
}

template <int K, int MODE>
cudaError_t launch_K(const nfft2d_plan_s *p, void *f, const void *v, void *g1, void *g2) {
    const KArgs a = make_kargs(p);
    if (p->precision == NFFT2D_F32 && p->gather_variant == NFFT2D_VARIANT_TILED) {
        if (p->n_chunks == 0) return cudaSuccess;
        const int smem = 2 * patch_stride_elems(p->g) * static_cast<int>(sizeof(float2)) + 128;
        auto kernel = p->g.PC == 32
                          ? (p->compensated ? k_gather_tiled<K, true, MODE, 32> : k_gather_tiled<K, false, MODE, 32>)
                          : p->g.PC == 36
                                ? (p->compensated ? k_gather_tiled<K, true, MODE, 36> : k_gather_tiled<K, false, MODE, 36>)
                                : (p->compensated ? k_gather_tiled<K, true, MODE, 0> : k_gather_tiled<K, false, MODE, 0>);
        cudaError_t e = prepare_smem(kernel, smem);
        if (e != cudaSuccess) return e;
        int blocks = grid_blocks(p, reinterpret_cast<const void *>(kernel), kThreads, smem);
        if (p->n_chunks >= 0 && blocks > p->n_chunks) blocks = static_cast<int>(p->n_chunks);
        kernel<<<blocks, kThreads, smem, p->stream>>>(p->tmap, static_cast<const Rec32 *>(p->recs), p->chunks,
                                                      static_cast<float2 *>(f), static_cast<const float2 *>(v),
                                                      static_cast<float *>(g1), static_cast<float *>(g2), a);
        return cudaGetLastError();
    }
    const int blocks = static_cast<int>((p->M + kThreads - 1) / kThreads);
    if (blocks == 0) return cudaSuccess;
    if (p->precision == NFFT2D_F64) {
        k_gather_direct<K, double, Rec64, MODE><<<blocks, kThreads, 0, p->stream>>>(
            static_cast<const double2 *>(p->grid), static_cast<const Rec64 *>(p->recs), static_cast<double2 *>(f),
            static_cast<const double2 *>(v), static_cast<double *>(g1), static_cast<double *>(g2), a);
    } else if constexpr (MODE == 0) {
        k_gather_direct_f32<K><<<blocks, kThreads, 0, p->stream>>>(
            static_cast<const float2 *>(p->grid), static_cast<const Rec32 *>(p->recs), static_cast<float2 *>(f), a);
    } else {
        static_assert(MODE == 0 || MODE == 1, "gather (0) or coordinate gradient (1)");
        k_grad_direct_f32<K><<<blocks, kThreads, 0, p->stream>>>(
            static_cast<const float2 *>(p->grid), static_cast<const Rec32 *>(p->recs), static_cast<const float2 *>(v),
            static_cast<float *>(g1), static_cast<float *>(g2), a);
    }
    return cudaGetLastError();
}

template <int MODE>
cudaError_t dispatch(const nfft2d_plan_s *p, void *f, const void *v, void *g1, void *g2) {
    switch (p->K) {
        case 2: return launch_K<2, MODE>(p, f, v, g1, g2);
        case 3: return launch_K<3, MODE>(p, f, v, g1, g2);
        case 4: return launch_K<4, MODE>(p, f, v, g1, g2);
        case 5: return launch_K<5, MODE>(p, f, v, g1, g2);
        case 6: return launch_K<6, MODE>(p, f, v, g1, g2);
        case 7: return launch_K<7, MODE>(p, f, v, g1, g2);
        case 8: return launch_K<8, MODE>(p, f, v, g1, g2);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace

cudaError_t launch_gather(const nfft2d_plan_s *p, void *f) { return dispatch<0>(p, f, nullptr, nullptr, nullptr); }

cudaError_t launch_grad(const nfft2d_plan_s *p, const void *v, void *g1, void *g2) {
    return dispatch<1>(p, nullptr, v, g1, g2);
}

int gather_smem_bytes(const nfft2d_plan_s *p) { return 2 * patch_stride_elems(p->g) * static_cast<int>(sizeof(float2)) + 128; }

}  // namespace nfft2d
