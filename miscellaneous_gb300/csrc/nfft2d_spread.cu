// nfft2d_spread.cu -- type-1 windowed spreading of the nonuniform data onto
// the oversampled grid (NFFT/NFFT2/Matlab/NFFT2_2D.m:47-56; the reference GPU
// kernel is Interpolation_NFFT2_2D_GPUKernel + series_terms,
// NFFT/NFFT2_2D.cu:105-276, which launches one 13x13 child grid per point and
// issues 338 global float atomics per point).
//
// TILED variant (FP32 plans): a persistent CTA walks work items (tile, point
// range).  For each it zeroes a (T+2K) x (T+2Ke) shared-memory patch, every
// thread adds the (2K+1)^2 weighted contributions of its points with
// shared-memory atomics (adjacent lanes hold adjacent cells, so one
// instruction's addresses rarely collide), and one thread flushes the patch
// into the padded global grid with a single TMA tensor reduction
// (cp.reduce.async.bulk.tensor.2d ... .add, f32).  Two patch buffers
// alternate so the flush of one overlaps the accumulation of the next.  The
// halo of the padded grid is folded back onto the interior afterwards
// (k_halo_fold), so no kernel wraps indices.
//
// DIRECT variant (both precisions): one thread per sorted point, global
// atomics into the padded grid.
#include <cuda.h>
#include <cuda_runtime.h>

#include "nfft2d_device.cuh"
#include "nfft2d_internal.h"
#include "nfft2d_kargs.cuh"

namespace nfft2d {
namespace {

constexpr int kThreads = 256;

template <int K>
__global__ void __launch_bounds__(kThreads) k_spread_tiled(const __grid_constant__ CUtensorMap tmap,
                                                           const Rec32 *__restrict__ recs,
                                                           const int4 *__restrict__ chunks,
                                                           const float2 *__restrict__ f, const KArgs a) {
    extern __shared__ unsigned char smem_raw[];
    constexpr int W = 2 * K + 1;
    const Geom g = a.g;
    const int pstride = patch_stride_elems(g);
    // TMA shared-memory operands: 128-byte aligned (the launch adds 128 bytes of slack)
    float2 *bufs = reinterpret_cast<float2 *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    const int n = a.n_chunks;
    const int nvec = (g.PR * g.PC) / 2;  // float4 stores per patch (PC is even)

    int it = 0;
    for (int c = blockIdx.x; c < n; c += gridDim.x, ++it) {
        const int b = it & 1;
        float2 *patch = bufs + b * pstride;
        // the reduction issued two work items ago read from this buffer
        if (threadIdx.x == 0 && it >= 2) bulk_wait_read_le1();
        __syncthreads();
        float4 *pv = reinterpret_cast<float4 *>(patch);
        for (int k = threadIdx.x; k < nvec; k += kThreads) pv[k] = make_float4(0.f, 0.f, 0.f, 0.f);
        __syncthreads();

        const int4 ch = __ldg(&chunks[c]);
        const int tr = ch.x / g.tiles2, tc = ch.x - tr * g.tiles2;
        const int r0 = tr * g.T, c0 = tc * g.T;
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
            const float2 v = __ldg(&f[raw.w]);
            float w1[W], w2[W];
            weights_f32<K>(t1, w1, a.alpha, a.cn, a.kp);
            weights_f32<K>(t2, w2, a.alpha, a.cn, a.kp);
            float *base = reinterpret_cast<float *>(patch + lr * g.PC + lc + (g.Ke - K));
#pragma unroll
            for (int r = 0; r < W; ++r) {
                const float vx = v.x * w1[r], vy = v.y * w1[r];
                float *row = base + 2 * r * g.PC;
#pragma unroll
                for (int q = 0; q < W; ++q) {
                    atomicAdd(row + 2 * q, vx * w2[q]);
                    atomicAdd(row + 2 * q + 1, vy * w2[q]);
                }
            }
        }
        fence_proxy_async_smem();  // generic-proxy writes -> visible to the TMA engine
        __syncthreads();
        if (threadIdx.x == 0) {
            const int x = 2 * (g.H + c0 - g.Ke);
            const int y = g.H + r0 - K;
            tma_reduce_add_2d(&tmap, patch, x, y);
            bulk_commit();
        }
    }
    if (threadIdx.x == 0) bulk_wait_all();
}

template <int K, typename Real, typename RecT>
__global__ void __launch_bounds__(kThreads) k_spread_direct(Real *__restrict__ grid, const RecT *__restrict__ recs,
                                                            const Real *__restrict__ f, const KArgs a) {
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
    const Real vx = f[2 * static_cast<size_t>(r.orig)], vy = f[2 * static_cast<size_t>(r.orig) + 1];
    Real w1[W], w2[W];
    if constexpr (sizeof(Real) == 4) {
        weights_f32<K>(r.t1, w1, a.alpha, a.cn, a.kp);
        weights_f32<K>(r.t2, w2, a.alpha, a.cn, a.kp);
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
    if (p->precision == NFFT2D_F32 && p->spread_variant == NFFT2D_VARIANT_TILED) {
        if (p->n_chunks == 0) return cudaSuccess;
        const int smem = 2 * patch_stride_elems(p->g) * static_cast<int>(sizeof(float2)) + 128;
        auto kernel = k_spread_tiled<K>;
        if (smem > 48 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
            if (e != cudaSuccess) return e;
        }
        int blocks = grid_blocks(p, reinterpret_cast<const void *>(kernel), kThreads, smem);
        if (blocks > p->n_chunks) blocks = static_cast<int>(p->n_chunks);
        kernel<<<blocks, kThreads, smem, p->stream>>>(p->tmap, static_cast<const Rec32 *>(p->recs), p->chunks,
                                                      static_cast<const float2 *>(f), a);
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
