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
// spread: lane groups accumulate a tile strip's patch in registers
// ---------------------------------------------------------------------------
// A work item holds points of one 16 x 16 tile, ordered strip by strip (SW
// columns each, spread_strip_width) and by row within a strip.  The warp
// splits into 32/G groups of G lanes; lane l of every group owns patch column
// l of the current strip, i.e. grid column c0 + s*SW - K + l, for the 16+2K
// patch rows (acc[r], one float2 per row).  A point at strip column q touches
// patch columns q .. q+2K, all inside the group, so 2K+1 of G lanes do useful
// work (13 of 16 at K = 6) where a lane-per-tile-column layout keeps 13 of 32.
// The groups take different points of the same row run at once (the static
// register indices need a warp-uniform row); when the strip is flushed each
// group's patch goes lanes -> its own shared patch -> one TMA tensor
// reduction (f32 add) into the grid (the TMA engine adds the groups'
// patches; no shuffles).
constexpr int kRegTile = 16;  // tile edge the register-resident spread requires

template <int K>
struct SpreadGeo {
    static constexpr int W = 2 * K + 1;
    static constexpr int G = spread_group_lanes(K);     // lanes per group
    static constexpr int NG = 32 / G;                   // groups per warp
    static constexpr int SW = spread_strip_width(K);    // strip width (columns)
    static constexpr int NS = kRegTile / SW;            // strips per tile
    static constexpr int PR = kRegTile + 2 * K;         // patch rows
    static constexpr int ODD = K & 1;                   // odd K: box starts one column early
    static constexpr int BOXC = G + 2 * ODD;            // shared patch / TMA box columns (complex)
    static constexpr int NBUF = NG;                     // flush buffers per warp: one per group
    static constexpr int W1 = ((W + 3) / 4) * 4;        // floats of the row weights (padded)
    // Column products v * w2 in the per-point scratch, either
    //  - lane-aligned (ALIGNED): one float2 per group lane, zero outside the
    //    point's 2K+1 columns, so a lane loads its operand at a fixed offset
    //    with no test; a zero row after the batch's 32 points serves a group
    //    without a point in a step.  Costs a zero fill and scattered stores
    //    in the prepass: it pays at K = 5..7 (13 x 13 taps: 72.9 -> 68.2 us
    //    per 2^20 polar points) but not at K = 4 or 8 (config-3 steps 3 %
    //    and 7 % slower: fewer taps per store, or 32-lane rows);
    //  - or packed (the 2K+1 products), each lane indexing them by its
    //    offset from the point's first column and testing the range.
    static constexpr bool ALIGNED = G == 16 && W >= 11;
    static constexpr int WV = ALIGNED ? 2 * G : ((2 * W + 3) / 4) * 4;
    // per-point scratch (floats): {lr, strip column, strip, -}, the row
    // weights, the column products.  The stride is 4 mod 8: the prepass's
    // 16-byte stores of 8 consecutive lanes hit 8 distinct bank quads, and
    // the groups' loads of consecutive points hit distinct banks.  (A
    // shared-memory load costs about one wavefront per float it delivers
    // whatever its width, so the row weights are stored once and broadcast.)
    static constexpr int SP0 = 4 + W1 + WV;
    static constexpr int SP = SP0 % 8 == 0 ? SP0 + 4 : SP0;
    static constexpr int ROWS = ALIGNED ? 33 : 32;      // scratch rows per warp (+ the zero row)
    static constexpr int PATCH = ((PR * BOXC + 15) / 16) * 16;  // float2 per buffer, 128-byte multiple
    static_assert(SW + 2 * K <= G, "strip windows must fit the group");
    static_assert(kRegTile % SW == 0, "strips tile the tile");
};

// Shared memory of one spreading warp: NBUF patch buffers + the point scratch.
template <int K>
__host__ __device__ constexpr int spread_warp_smem_bytes() {
    using S = SpreadGeo<K>;
    return S::NBUF * S::PATCH * 8 + S::ROWS * S::SP * 4;
}

// acc[L + a] += (ax, ay) * w1[a] for the 2K+1 rows of a point whose first
// patch row is L (compile-time, so acc stays in registers).
template <int K, int PR, int L>
__device__ __forceinline__ void add_rows2(float2 (&acc)[PR], const float (&w1)[2 * K + 1], float2 v) {
#pragma unroll
    for (int a = 0; a <= 2 * K; ++a) {
        acc[L + a].x = fmaf(v.x, w1[a], acc[L + a].x);
        acc[L + a].y = fmaf(v.y, w1[a], acc[L + a].y);
    }
}

// f(integral_constant<int, L>) for L = 0, 1, ..., in order.
template <typename F, int... Ls>
__device__ __forceinline__ void for_each_row(F &&f, std::integer_sequence<int, Ls...>) {
    (f(std::integral_constant<int, Ls>{}), ...);
}

// cp.async.bulk.wait_group.read N: at most N of the thread's bulk groups are
// still reading their shared-memory source.
__device__ __forceinline__ void bulk_wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }

// Per-warp flush state of the strip spread.
struct StripFlush {
    const CUtensorMap *map;  // the grid's strip-patch tensor map
    float2 *bufs;            // NBUF patch buffers of this warp
    int H;                   // grid halo
    int issued;              // flushes issued so far by this warp
};

// Zero the warp's patch buffers once (odd K: the columns outside the lanes
// stay zero for the life of the kernel) and the zero row of its scratch scr.
template <int K>
__device__ __forceinline__ void strip_flush_init(StripFlush &fs, float *scr) {
    using S = SpreadGeo<K>;
    const int lane = threadIdx.x & 31;
    for (int i = lane; i < S::NBUF * S::PATCH; i += 32) fs.bufs[i] = make_float2(0.f, 0.f);
    if constexpr (S::ALIGNED)
        for (int i = lane; i < S::SP; i += 32) scr[32 * S::SP + i] = 0.f;
    __syncwarp();
}

// Write each group's patch to its own shared buffer and reduce them into the
// grid with one TMA tensor reduction per group at strip s of the tile with
// origin (r0, c0).  Lane 0 issues every reduction, so its bulk-group wait
// covers the buffers' previous readers.
template <int K>
__device__ __forceinline__ void strip_flush(StripFlush &fs, float2 (&acc)[SpreadGeo<K>::PR], int r0, int c0, int s) {
    using S = SpreadGeo<K>;
    const int lane = threadIdx.x & 31;
    // the reductions issued by the previous flush have finished reading
    if (lane == 0 && fs.issued > 0) bulk_wait_read_all();
    __syncwarp();
    float2 *buf = fs.bufs + (lane / S::G) * S::PATCH;
#pragma unroll
    for (int r = 0; r < S::PR; ++r) buf[r * S::BOXC + S::ODD + (lane % S::G)] = acc[r];
    fence_proxy_async_smem();  // generic-proxy writes -> visible to the TMA engine
    __syncwarp();
    if (lane == 0) {
        const int x = 2 * (fs.H + c0 + s * S::SW - K - S::ODD), y = fs.H + r0 - K;
#pragma unroll
        for (int g = 0; g < S::NG; ++g) tma_reduce_add_2d(fs.map, fs.bufs + g * S::PATCH, x, y);
        bulk_commit();
    }
    ++fs.issued;
}

// Spread points [first, first + cnt) of one tile (origin r0, c0) into the
// grid, strip by strip, flushing each strip's register patch.  f is indexed
// by the record's caller index, or (binned_io) by the record's position.
// scr is the warp's scratch of SpreadGeo<K>::ROWS * SP floats.  A record
// outside the tile latches kErrBounds and contributes nothing.
template <int K>
__device__ __forceinline__ void spread_item(const Rec32 *__restrict__ recs, int first, int cnt, int r0, int c0,
                                            const float2 *__restrict__ f, int binned_io, float *scr, StripFlush &fs,
                                            const WinPoly &wp, int *status) {
    using S = SpreadGeo<K>;
    constexpr int W = S::W, PR = S::PR, SP = S::SP, W1 = S::W1;
    const int lane = threadIdx.x & 31;
    const int grp = lane / S::G, gl = lane % S::G;
    float2 acc[PR];
#pragma unroll
    for (int r = 0; r < PR; ++r) acc[r] = make_float2(0.f, 0.f);
    int cur = -1;  // strip held in acc
    // each batch's records are loaded one batch ahead (the next batch's load
    // overlaps this batch's walk)
    int4 raw_next = make_int4(0, 0, 0, 0);
    if (lane < cnt) raw_next = __ldg(reinterpret_cast<const int4 *>(recs) + first + lane);
    for (int base0 = 0; base0 < cnt; base0 += 32) {
        const int nb = min(32, cnt - base0);
        const int4 raw = raw_next;
        // 1) each lane prepares one point: offsets, value, 2(2K+1) weights
        int my_key = 0x7fffffff;  // (strip << 4) | row, sorted ascending along the batch
        if (lane < nb) {
            const int mu1 = static_cast<int>(static_cast<unsigned>(raw.z) >> 16), mu2 = raw.z & 0xFFFF;
            int lr = mu1 - r0, lc = mu2 - c0;
            float2 v = __ldg(&f[binned_io ? first + base0 + lane : raw.w]);
            if (static_cast<unsigned>(lr) >= static_cast<unsigned>(kRegTile) ||
                static_cast<unsigned>(lc) >= static_cast<unsigned>(kRegTile)) {
                latch_error(status, kErrBounds);
                lr = lc = 0;
                v = make_float2(0.f, 0.f);  // contributes nothing
            }
            const int st = lc / S::SW;
            my_key = (st << 4) | lr;
            float w1[W], w2[W];
            weights_poly<K>(__int_as_float(raw.x), w1, wp);
            weights_poly<K>(__int_as_float(raw.y), w2, wp);
            float *sp = scr + lane * SP;
            const int q = lc - st * S::SW;  // first patch column of the point within the strip
            reinterpret_cast<int4 *>(sp)[0] = make_int4(lr, q, st, 0);
            float4 *wq = reinterpret_cast<float4 *>(sp + 4);
#pragma unroll
            for (int k = 0; k < W1 / 4; ++k)
                wq[k] = make_float4(w1[4 * k], 4 * k + 1 < W ? w1[4 * k + 1] : 0.f,
                                    4 * k + 2 < W ? w1[4 * k + 2] : 0.f, 4 * k + 3 < W ? w1[4 * k + 3] : 0.f);
            float4 *vq = reinterpret_cast<float4 *>(sp + 4 + W1);
            if constexpr (S::ALIGNED) {
                // the group lanes' column products: zeros, then the 2K+1
                // products at lanes q .. q+2K (q + 2K < G)
#pragma unroll
                for (int k = 0; k < S::WV / 4; ++k) vq[k] = make_float4(0.f, 0.f, 0.f, 0.f);
                float2 *vl = reinterpret_cast<float2 *>(sp + 4 + W1) + q;
#pragma unroll
                for (int b = 0; b < W; ++b) vl[b] = make_float2(v.x * w2[b], v.y * w2[b]);
            } else {
#pragma unroll
                for (int k = 0; k < S::WV / 4; ++k) {
                    const float a = 2 * k < W ? w2[2 * k] : 0.f;
                    const float b = 2 * k + 1 < W ? w2[2 * k + 1] : 0.f;
                    vq[k] = make_float4(v.x * a, v.y * a, v.x * b, v.y * b);
                }
            }
        }
        if (base0 + 32 + lane < cnt) raw_next = __ldg(reinterpret_cast<const int4 *>(recs) + first + base0 + 32 + lane);
        __syncwarp();
        // 2) operands of point k + grp of the run starting at j0 for this
        //    lane: the row weights (broadcast within the group) and this
        //    lane's column product (zero outside the point's columns, or
        //    when the group has no point this step)
        auto load = [&](int j0, int k, int n, float (&w1)[W], float2 &vw) {
            const bool ok = k + grp < n;
            const int p = ok ? j0 + k + grp : (S::ALIGNED ? 32 : j0);
            const float *sp = scr + p * SP;
            const float4 *wq = reinterpret_cast<const float4 *>(sp + 4);
#pragma unroll
            for (int k = 0; k < W / 4; ++k) {
                const float4 t = wq[k];
                w1[4 * k] = t.x;
                w1[4 * k + 1] = t.y;
                w1[4 * k + 2] = t.z;
                w1[4 * k + 3] = t.w;
            }
#pragma unroll
            for (int a = (W / 4) * 4; a < W; ++a) w1[a] = sp[4 + a];
            if constexpr (S::ALIGNED) {
                vw = reinterpret_cast<const float2 *>(sp + 4 + W1)[gl];
            } else {
                const int b = gl - reinterpret_cast<const int *>(sp)[1];
                vw = (ok && static_cast<unsigned>(b) < static_cast<unsigned>(W))
                         ? reinterpret_cast<const float2 *>(sp + 4 + W1)[b] : make_float2(0.f, 0.f);
            }
        };
        // The binning keeps a work item's keys ascending; a batch out of
        // order can only follow a record that failed the bounds check above
        // (already latched): it is skipped rather than given a slow path of
        // its own (16 more copies of the row update would not fit the
        // instruction cache alongside the walk).
        const int prev = __shfl_up_sync(0xffffffffu, my_key, 1);
        const bool sorted = __all_sync(0xffffffffu, lane == 0 || lane >= nb || prev <= my_key);
        if (!sorted && lane == 0) latch_error(status, kErrBounds);
        int j = sorted ? 0 : nb;
        while (j < nb) {
            const int st = __shfl_sync(0xffffffffu, my_key, j) >> 4;
            if (st != cur) {
                if (cur >= 0) {
                    strip_flush<K>(fs, acc, r0, c0, cur);
#pragma unroll
                    for (int r = 0; r < PR; ++r) acc[r] = make_float2(0.f, 0.f);
                }
                cur = st;
            }
            // the strip's points, row run by row run: run L adds to
            // acc[L .. L+2K] with compile-time register indices, NG
            // points of the run per step; rows without points are
            // skipped by one mask test
            const unsigned rows =
                __reduce_or_sync(0xffffffffu, (my_key >> 4) == st ? (1u << (my_key & 15)) : 0u);
            for_each_row(
                [&](auto Lc) {
                    constexpr int L = decltype(Lc)::value;
                    if (!(rows & (1u << L))) return;
                    const int n = __popc(__ballot_sync(0xffffffffu, my_key == ((st << 4) | L)));
#pragma unroll 1
                    for (int k = 0; k < n; k += S::NG) {
                        float w1[W];
                        float2 vw;
                        load(j, k, n, w1, vw);
                        add_rows2<K, PR, L>(acc, w1, vw);
                    }
                    j += n;
                },
                std::make_integer_sequence<int, kRegTile>{});
        }
        __syncwarp();  // scratch is rewritten by the next batch
    }
    if (cur >= 0) strip_flush<K>(fs, acc, r0, c0, cur);
}

}  // namespace nfft2d
