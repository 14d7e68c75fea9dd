// nfft2d_tile_ops.cuh -- the per-point work of the tiled kernels, shared by the
// single-transform kernels (nfft2d_gather.cu, nfft2d_spread.cu) and the
// batched ones (nfft2d_batch.cu).
#pragma once

#include <cuda_runtime.h>

#include <type_traits>
#include <utility>

#include "nfft2d_device.cuh"
#include "nfft2d_internal.h"

namespace nfft2d {

// ---------------------------------------------------------------------------
// gather: one point from a shared-memory tile patch
// ---------------------------------------------------------------------------

// f = sum_{r,q} w1[r] w2[q] patch[lr + r][lc + (Ke - K) + q]; row partial sums
// with FMA, the sum over rows compensated (TwoSum) when COMP.
template <int K, bool COMP>
__device__ __forceinline__ float2 gather_point(const float2 *__restrict__ patch, int PC, int Ke, int lr, int lc,
                                               float t1, float t2, const WinPoly &wp) {
    constexpr int W = 2 * K + 1;
    float w1[W], w2[W];
    weights_poly<K>(t1, w1, wp);
    weights_poly<K>(t2, w2, wp);
    const float2 *base = patch + lr * PC + lc + (Ke - K);
    float sx = 0.f, sy = 0.f, ex = 0.f, ey = 0.f;
#pragma unroll
    for (int r = 0; r < W; ++r) {
        const float2 *row = base + r * PC;
        float rx = 0.f, ry = 0.f;
#pragma unroll
        for (int q = 0; q < W; ++q) {
            const float2 v = row[q];
            rx = fmaf(w2[q], v.x, rx);
            ry = fmaf(w2[q], v.y, ry);
        }
        if (COMP) {
            float e;
            two_sum(sx, __fmul_rn(w1[r], rx), sx, e);
            ex = __fadd_rn(ex, e);
            two_sum(sy, __fmul_rn(w1[r], ry), sy, e);
            ey = __fadd_rn(ey, e);
        } else {
            sx = fmaf(w1[r], rx, sx);
            sy = fmaf(w1[r], ry, sy);
        }
    }
    return make_float2(sx + ex, sy + ey);
}

// ---------------------------------------------------------------------------
// gather: one point straight from the padded grid (L1/L2), FP32
// ---------------------------------------------------------------------------

// 16-byte loads, two taps each: a row's 2K+1 taps start at an even or odd
// complex column; the 2K+2 columns from the 16-byte boundary at or below it
// are read and the column weights shifted by one for odd starts (the extra
// column gets weight 0; it lies inside the padded grid, or in the zeroed
// slack after it).  Grid rows start on 16-byte boundaries (even pitch).
//
// COMP: the weighted row partials are summed with TwoSum and the rounding
// errors carried in a second accumulator (as the tiled gather does), else
// with plain FMAs.
template <int K, bool COMP>
__device__ __forceinline__ float2 gather_direct_f32(const float2 *__restrict__ grid, int H, int C, int mu1, int mu2,
                                                    float t1, float t2, const WinPoly &wp) {
    constexpr int W = 2 * K + 1;
    constexpr int V = K + 1;  // float4 loads per row
    float w1[W], w2[W];
    weights_poly<K>(t1, w1, wp);
    weights_poly<K>(t2, w2, wp);
    const int col0 = mu2 + H - K;
    const int odd = col0 & 1;
    float ws[2 * V];
#pragma unroll
    for (int q = 0; q < 2 * V; ++q) {
        const float lo = q < W ? w2[q] : 0.f;
        const float hi = (q >= 1 && q - 1 < W) ? w2[q - 1] : 0.f;
        ws[q] = odd ? hi : lo;
    }
    const float4 *rb = reinterpret_cast<const float4 *>(grid + static_cast<size_t>(mu1 + H - K) * C + (col0 - odd));
    const int pitch4 = C >> 1;
    // (re, im) of a cell times a real weight: one packed FP32x2 FMA, rounded
    // as two fmaf (2-3 % faster than scalar FMAs on GB300 at K = 2..8).
    float2 wsp[2 * V];
#pragma unroll
    for (int q = 0; q < 2 * V; ++q) wsp[q] = make_float2(ws[q], ws[q]);
    float2 s = make_float2(0.f, 0.f), e = make_float2(0.f, 0.f);
#pragma unroll
    for (int rr = 0; rr < W; ++rr) {
        const float4 *row = rb + rr * pitch4;
        float2 r = make_float2(0.f, 0.f);
#pragma unroll
        for (int q = 0; q < V; ++q) {
            const float4 v = __ldg(row + q);
            r = __ffma2_rn(make_float2(v.x, v.y), wsp[2 * q], r);
            r = __ffma2_rn(make_float2(v.z, v.w), wsp[2 * q + 1], r);
        }
        if constexpr (COMP) {
            float ex, ey;
            two_sum(s.x, __fmul_rn(w1[rr], r.x), s.x, ex);
            two_sum(s.y, __fmul_rn(w1[rr], r.y), s.y, ey);
            e.x = __fadd_rn(e.x, ex);
            e.y = __fadd_rn(e.y, ey);
        } else {
            s = __ffma2_rn(r, make_float2(w1[rr], w1[rr]), s);
        }
    }
    if constexpr (COMP) return make_float2(s.x + e.x, s.y + e.y);
    return s;
}

// ---------------------------------------------------------------------------
// spread: a warp accumulates a 16 x 16 tile's (16+2K) x 32 patch in registers
// ---------------------------------------------------------------------------
constexpr int kRegTile = 16;  // tile edge the register-resident spread requires

// Per-point scratch (floats): lr, lc, v.x, v.y; the row weights w1 padded to
// a multiple of 4 floats (2K+1 used); then the column products v * w2 as
// float2, same padding.  The stride between points is kept off multiples of
// 8 floats: the prepass has every lane write its own point, and a stride with
// a larger power-of-two factor maps more lanes onto one bank (at K = 8 the
// unpadded 64 put all 32 lanes on one bank).
template <int K>
constexpr int wpad() {
    return ((2 * K + 1 + 3) / 4) * 4;
}
template <int K>
constexpr int point_scratch() {
    return (4 + 3 * wpad<K>()) % 8 == 0 ? 4 + 3 * wpad<K>() + 4 : 4 + 3 * wpad<K>();
}

// acc[L + a] += (ax, ay) * w1[a] for the 2K+1 rows of a point whose first
// patch row is L (compile-time, so acc stays in registers).
template <int K, int PR, int L>
__device__ __forceinline__ void add_rows(float2 (&acc)[PR], const float (&w1)[wpad<K>()], float ax, float ay) {
#pragma unroll
    for (int a = 0; a <= 2 * K; ++a) {
        acc[L + a].x = fmaf(ax, w1[a], acc[L + a].x);
        acc[L + a].y = fmaf(ay, w1[a], acc[L + a].y);
    }
}

// Dispatch on the point's first patch row with a jump table (the row offset
// is warp-uniform, so every lane takes the same case).
template <int K, int PR>
__device__ __forceinline__ void add_rows_switch(int lr, float2 (&acc)[PR], const float (&w1)[wpad<K>()], float ax,
                                                float ay) {
    static_assert(kRegTile == 16, "one case per row of a 16-row tile");
#define NFFT2D_ROW_CASE(L)                   \
    case L:                                  \
        add_rows<K, PR, L>(acc, w1, ax, ay); \
        break;
    switch (lr) {
        NFFT2D_ROW_CASE(0) NFFT2D_ROW_CASE(1) NFFT2D_ROW_CASE(2) NFFT2D_ROW_CASE(3)
        NFFT2D_ROW_CASE(4) NFFT2D_ROW_CASE(5) NFFT2D_ROW_CASE(6) NFFT2D_ROW_CASE(7)
        NFFT2D_ROW_CASE(8) NFFT2D_ROW_CASE(9) NFFT2D_ROW_CASE(10) NFFT2D_ROW_CASE(11)
        NFFT2D_ROW_CASE(12) NFFT2D_ROW_CASE(13) NFFT2D_ROW_CASE(14) NFFT2D_ROW_CASE(15)
        default: break;
    }
#undef NFFT2D_ROW_CASE
}

// f(integral_constant<int, L>) for L = 0, 1, ..., in order.
template <typename F, int... Ls>
__device__ __forceinline__ void for_each_row(F &&f, std::integer_sequence<int, Ls...>) {
    (f(std::integral_constant<int, Ls>{}), ...);
}

// Add the contributions of points [first, first + cnt) of one tile (origin
// r0, c0) to the warp's register patch acc (lane = patch column).  scr is the
// warp's scratch of 32 * point_scratch<K>() floats.  A record outside the tile
// latches kErrBounds and contributes nothing.
template <int K>
__device__ __forceinline__ void spread_points(const Rec32 *__restrict__ recs, int first, int cnt, int r0, int c0,
                                              const float2 *__restrict__ f, float *scr,
                                              float2 (&acc)[kRegTile + 2 * K], const WinPoly &wp, int *status) {
    constexpr int W = 2 * K + 1;
    constexpr int PR = kRegTile + 2 * K;
    constexpr int KE = K + (K & 1);
    constexpr int SP = point_scratch<K>(), WP = wpad<K>();
    const int lane = threadIdx.x & 31;
    for (int base0 = 0; base0 < cnt; base0 += 32) {
        const int nb = min(32, cnt - base0);
        // 1) each lane prepares one point: offsets, value, 2(2K+1) weights
        if (lane < nb) {
            const int4 raw = __ldg(reinterpret_cast<const int4 *>(recs) + first + base0 + lane);
            const int mu1 = static_cast<int>(static_cast<unsigned>(raw.z) >> 16), mu2 = raw.z & 0xFFFF;
            int lr = mu1 - r0, lc = mu2 - c0;
            float2 v = __ldg(&f[raw.w]);
            if (static_cast<unsigned>(lr) >= static_cast<unsigned>(kRegTile) ||
                static_cast<unsigned>(lc) >= static_cast<unsigned>(kRegTile)) {
                latch_error(status, kErrBounds);
                lr = lc = 0;
                v = make_float2(0.f, 0.f);  // contributes nothing
            }
            float w1[W], w2[W];
            weights_poly<K>(__int_as_float(raw.x), w1, wp);
            weights_poly<K>(__int_as_float(raw.y), w2, wp);
            float *sp = scr + lane * SP;
            reinterpret_cast<float4 *>(sp)[0] = make_float4(__int_as_float(lr), __int_as_float(lc), v.x, v.y);
#pragma unroll
            for (int k = 0; k < WP; ++k) sp[4 + k] = k < W ? w1[k] : 0.f;
#pragma unroll
            for (int k = 0; k < WP; ++k)
                reinterpret_cast<float2 *>(sp + 4 + WP)[k] =
                    k < W ? make_float2(v.x * w2[k], v.y * w2[k]) : make_float2(0.f, 0.f);
        }
        __syncwarp();
        // 2) the warp walks the points; lane = patch column.  Operands of
        //    point j: the 2K+1 row weights (broadcast) and this lane's column
        //    product v * w2 (zero outside the point's columns).
        auto load = [&](int j, float (&w1)[WP], float &ax, float &ay) {
            const float *sp = scr + j * SP;
            const int lc = __float_as_int(sp[1]);
#pragma unroll
            for (int q = 0; q < WP / 4; ++q) {
                const float4 t = reinterpret_cast<const float4 *>(sp + 4)[q];
                w1[4 * q] = t.x;
                w1[4 * q + 1] = t.y;
                w1[4 * q + 2] = t.z;
                w1[4 * q + 3] = t.w;
            }
            const int b = lane - lc - (KE - K);  // this lane's tap column
            const float2 vw = (static_cast<unsigned>(b) < static_cast<unsigned>(W))
                                  ? reinterpret_cast<const float2 *>(sp + 4 + WP)[b] : make_float2(0.f, 0.f);
            ax = vw.x;
            ay = vw.y;
        };
        int j = 0;
        // The binning sorts a tile's points by row, so the walk visits the
        // row offsets in increasing order: phase L adds its run of points to
        // acc[L .. L+2K] with compile-time register indices and no indirect
        // branch.  A point out of order -- only after a latched bounds error
        // -- is left to the dispatch loop below.  From K = 6 up each run is
        // counted by one ballot; for narrower windows comparing each next
        // point's row measured faster (2-3x at K <= 5 on GB300).
        if constexpr (K < 6) {
            int lr_j = nb > 0 ? __float_as_int(scr[0]) : kRegTile;
            for_each_row(
                [&](auto Lc) {
                    constexpr int L = decltype(Lc)::value;
                    // two points per iteration: 2-3 us faster per 2^20 points at
                    // K = 2..5 (unrolling the ballot walk of K >= 6 was slower)
#pragma unroll 2
                    while (lr_j == L) {
                        float w1[WP], ax, ay;
                        load(j, w1, ax, ay);
                        ++j;
                        lr_j = j < nb ? __float_as_int(scr[j * SP]) : kRegTile;
                        add_rows<K, PR, L>(acc, w1, ax, ay);
                    }
                },
                std::make_integer_sequence<int, kRegTile>{});
        } else {
            const int my_lr = lane < nb ? __float_as_int(scr[lane * SP]) : kRegTile;
            const int prev = __shfl_up_sync(0xffffffffu, my_lr, 1);
            const bool sorted = __all_sync(0xffffffffu, lane == 0 || prev <= my_lr);
            if (sorted) {
                for_each_row(
                    [&](auto Lc) {
                        constexpr int L = decltype(Lc)::value;
                        const int e = j + __popc(__ballot_sync(0xffffffffu, my_lr == L));
                        for (; j < e; ++j) {
                            float w1[WP], ax, ay;
                            load(j, w1, ax, ay);
                            add_rows<K, PR, L>(acc, w1, ax, ay);
                        }
                    },
                    std::make_integer_sequence<int, kRegTile>{});
            }
        }
        for (; j < nb; ++j) {
            float w1[WP], ax, ay;
            load(j, w1, ax, ay);
            add_rows_switch<K, PR>(__float_as_int(scr[j * SP]), acc, w1, ax, ay);
        }
        __syncwarp();  // scratch is rewritten by the next batch
    }
}

// cp.async.bulk.wait_group.read 0: the thread's last bulk reduction has
// finished reading its shared-memory source.
__device__ __forceinline__ void bulk_wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }

// Flush a warp's register patch: lanes -> shared patch (PR x 32) -> one TMA
// tensor reduction into the grid at the tile (r0, c0).  `pending` tells
// whether the warp's previous flush may still be reading the patch.
template <int K>
__device__ __forceinline__ void flush_patch(const CUtensorMap *map, float2 *patch, const float2 (&acc)[kRegTile + 2 * K],
                                            int H, int r0, int c0, bool pending) {
    constexpr int PR = kRegTile + 2 * K;
    constexpr int KE = K + (K & 1);
    const int lane = threadIdx.x & 31;
    if (lane == 0 && pending) bulk_wait_read_all();
    __syncwarp();
#pragma unroll
    for (int r = 0; r < PR; ++r) patch[r * 32 + lane] = acc[r];
    fence_proxy_async_smem();  // generic-proxy writes -> visible to the TMA engine
    __syncwarp();
    if (lane == 0) {
        tma_reduce_add_2d(map, patch, 2 * (H + c0 - KE), H + r0 - K);
        bulk_commit();
    }
}

}  // namespace nfft2d
