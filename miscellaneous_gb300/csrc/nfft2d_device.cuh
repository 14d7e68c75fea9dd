// nfft2d_device.cuh -- device helpers: TMA / mbarrier / bulk-group inline PTX
// (sm_90+ forms, compiled for sm_103a) and the window pair in FP32 and FP64.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "nfft2d_internal.h"

namespace nfft2d {

// Spin bound for every device-side wait.  mbarrier.try_wait suspends for a
// hardware-defined time per call, so this bounds the wait to well under a
// second; on expiry the kernel latches kErrTimeout and returns.
constexpr uint32_t kSpinLimit = 1u << 22;

// ---------------------------------------------------------------------------
// shared-memory / async-proxy primitives
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Make mbarrier initialisation and prior generic-proxy shared-memory
// accesses visible to the async proxy (TMA).
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// One arrival on an mbarrier (no transaction bytes).
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, uint32_t limit = kSpinLimit) {
    for (uint32_t i = 0; i < limit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// 2D tiled TMA load global -> shared, completion signalled on an mbarrier.
// x is the innermost coordinate in elements of the tensor map (must make
// x * elemsize a multiple of 16 bytes), y the row.
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// 2D tiled TMA reduction shared -> global: global[box] += shared[box] (f32 add).
__device__ __forceinline__ void tma_reduce_add_2d(const CUtensorMap *map, const void *src, int x, int y) {
    asm volatile(
        "cp.reduce.async.bulk.tensor.2d.global.shared::cta.add.tile.bulk_group"
        " [%0, {%1, %2}], [%3];" ::"l"(reinterpret_cast<uint64_t>(map)),
        "r"(x), "r"(y), "r"(smem_u32(src))
        : "memory");
}

__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// Wait until at most one bulk group is still reading its shared-memory source.
__device__ __forceinline__ void bulk_wait_read_le1() {
    asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
}
// Wait until every committed bulk group has completed (writes performed).
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

__device__ __forceinline__ void latch_error(int *status, int bit) { atomicOr(status + 1, bit); }

// ---------------------------------------------------------------------------
// Window pair.  The reference window (NFFT1_2D.m:34-36, NFFT2_2D.cu:112-122)
//     phi_hat(u) = (1/pi) sinh(alpha s)/s,  s = sqrt(K^2 - u^2)
// (sin form for |u| > K) is used here normalised to 1 at u = 0:
//     w(u) = cn sinh(alpha s)/s,  cn = K / sinh(alpha K);
// the factor sinh(alpha K)/(pi K) moves into the deapodisation table.
// A tap of a point with offset t in [-1/2, 1/2] at grid offset m sits at
// u = t - m; K^2 - u^2 is formed as ((K+m) - t) * ((K-m) + t), a product of
// two well-conditioned factors, so its relative error stays near 1 ulp.
// ---------------------------------------------------------------------------

// Interior tap (|m| < K, so s >= sqrt(K - 1/4)): with cosh/sinh ~ e^{alpha s}/2
//     w = kp * exp(alpha (s - K)) / s,  s - K = -u^2 / (s + K),
// evaluated through the well-conditioned difference -u^2/(s+K); for K <= 3
// the dropped factor (1 - e^{-2 alpha s}) is restored.
template <int K>
__device__ __forceinline__ float win_interior_f32(float t, int m, float alpha, float kp) {
    const float pa = static_cast<float>(K + m) - t;
    const float pb = static_cast<float>(K - m) + t;
    const float P = pa * pb;
    const float r = rsqrtf(P);
    const float s = P * r;
    const float u = t - static_cast<float>(m);
    const float x = __fdividef(-alpha * (u * u), s + static_cast<float>(K));
    float w = kp * __expf(x) * r;
    if (K <= 3) w *= 1.0f - __expf(-2.0f * alpha * s);
    return w;
}

// Edge tap (m = -K or m = K): full formula, both branches.
template <int K>
__device__ __forceinline__ float win_edge_f32(float t, int m, float alpha, float cn) {
    const float pa = static_cast<float>(K + m) - t;
    const float pb = static_cast<float>(K - m) + t;
    const float P = pa * pb;
    const float s = sqrtf(fabsf(P));
    const float as = alpha * s;
    if (s == 0.0f) return cn * alpha;
    const float v = (P > 0.0f) ? sinhf(as) : __sinf(as);  // |as| < 13 here
    return cn * v / s;
}

template <int K>
__device__ __forceinline__ void weights_f32(float t, float (&w)[2 * K + 1], float alpha, float cn, float kp) {
#pragma unroll
    for (int a = 0; a <= 2 * K; ++a) {
        const int m = a - K;
        if (a == 0 || a == 2 * K)
            w[a] = win_edge_f32<K>(t, m, alpha, cn);
        else
            w[a] = win_interior_f32<K>(t, m, alpha, kp);
    }
}

// All 2K+1 taps from the plan's polynomials: Horner steps on FP32 FMAs whose
// coefficients are read from kernel parameter space (uniform across the warp).
// Taps (2j, 2j+1) share one packed FP32x2 FMA (__ffma2_rn) per Horner step;
// the odd last tap runs alone.
template <int K>
__device__ __forceinline__ void weights_poly(float t, float (&w)[2 * K + 1], const WinPoly &P) {
    constexpr int D = poly_degree(K);
    const float2 tt = make_float2(t, t);
    float2 acc[K];
    float last = P.c[D][2 * K];
#pragma unroll
    for (int j = 0; j < K; ++j) acc[j] = *reinterpret_cast<const float2 *>(&P.c[D][2 * j]);
#pragma unroll
    for (int d = D - 1; d >= 0; --d) {
#pragma unroll
        for (int j = 0; j < K; ++j) acc[j] = __ffma2_rn(acc[j], tt, *reinterpret_cast<const float2 *>(&P.c[d][2 * j]));
        last = fmaf(last, t, P.c[d][2 * K]);
    }
#pragma unroll
    for (int j = 0; j < K; ++j) {
        w[2 * j] = acc[j].x;
        w[2 * j + 1] = acc[j].y;
    }
    w[2 * K] = last;
}

// The taps and their derivatives d/dt from the same polynomials: Horner for
// value and slope together (slope = slope * t + value before each value
// step), two taps per packed FMA.  The slope of the fit differs from the
// closed form by less than 1e-7 of the window's peak slope.
template <int K>
__device__ __forceinline__ void weights_poly_d(float t, float (&w)[2 * K + 1], float (&dw)[2 * K + 1],
                                               const WinPoly &P) {
    constexpr int D = poly_degree(K);
    const float2 tt = make_float2(t, t);
    float2 acc[K], dacc[K];
    float last = P.c[D][2 * K], dlast = 0.f;
#pragma unroll
    for (int j = 0; j < K; ++j) {
        acc[j] = *reinterpret_cast<const float2 *>(&P.c[D][2 * j]);
        dacc[j] = make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int d = D - 1; d >= 0; --d) {
#pragma unroll
        for (int j = 0; j < K; ++j) {
            dacc[j] = __ffma2_rn(dacc[j], tt, acc[j]);
            acc[j] = __ffma2_rn(acc[j], tt, *reinterpret_cast<const float2 *>(&P.c[d][2 * j]));
        }
        dlast = fmaf(dlast, t, last);
        last = fmaf(last, t, P.c[d][2 * K]);
    }
#pragma unroll
    for (int j = 0; j < K; ++j) {
        w[2 * j] = acc[j].x;
        w[2 * j + 1] = acc[j].y;
        dw[2 * j] = dacc[j].x;
        dw[2 * j + 1] = dacc[j].y;
    }
    w[2 * K] = last;
    dw[2 * K] = dlast;
}

// Derivative dw/dt of the same taps (d/dt of w(t - m)), closed form.
//   interior: dw/du = w * (alpha s coth(alpha s) - 1) * (-u) / s^2
//   edge:     dw/du = cn * g'(P) * (-2u),  g(P) = sinh(alpha sqrt(P))/sqrt(P),
//             g' by its series near P = 0, closed forms elsewhere.
template <int K>
__device__ __forceinline__ void dweights_f32(float t, const float (&w)[2 * K + 1], float (&dw)[2 * K + 1],
                                             float alpha, float cn) {
#pragma unroll
    for (int a = 0; a <= 2 * K; ++a) {
        const int m = a - K;
        const float pa = static_cast<float>(K + m) - t;
        const float pb = static_cast<float>(K - m) + t;
        const float P = pa * pb;
        const float u = t - static_cast<float>(m);
        if (a != 0 && a != 2 * K) {
            const float s = sqrtf(P);
            const float as = alpha * s;
            float coth = 1.0f;
            if (K <= 3) {
                const float e = __expf(-2.0f * as);
                coth = (1.0f + e) / (1.0f - e);
            }
            dw[a] = w[a] * (as * coth - 1.0f) * (-u) / P;
        } else {
            const float a2 = alpha * alpha;
            float gp;
            if (fabsf(a2 * P) < 0.5f) {
                // alpha^3/6 + alpha^5 P/60 + alpha^7 P^2/1680 + alpha^9 P^3/90720
                gp = alpha * a2 * (1.0f / 6.0f + a2 * P * (1.0f / 60.0f + a2 * P * (1.0f / 1680.0f + a2 * P * (1.0f / 90720.0f))));
            } else if (P > 0.0f) {
                const float s = sqrtf(P), as = alpha * s;
                gp = (as * coshf(as) - sinhf(as)) / (2.0f * s * P);
            } else {
                const float s = sqrtf(-P), as = alpha * s;
                gp = -(as * cosf(as) - sinf(as)) / (2.0f * s * (-P));
            }
            dw[a] = cn * gp * (-2.0f * u);
        }
    }
}

// FP64 versions: the reference formula directly (FP64 plans are the
// precision / compatibility path; GB300 FP64 throughput is low, so the FP32
// plans never use these in their hot loops).
template <int K>
__device__ __forceinline__ void weights_f64(double t, double (&w)[2 * K + 1], double alpha, double cn) {
#pragma unroll
    for (int a = 0; a <= 2 * K; ++a) {
        const int m = a - K;
        const double pa = static_cast<double>(K + m) - t;
        const double pb = static_cast<double>(K - m) + t;
        const double P = pa * pb;
        const double s = sqrt(fabs(P));
        if (s == 0.0) {
            w[a] = cn * alpha;
        } else {
            const double v = (P > 0.0) ? sinh(alpha * s) : sin(alpha * s);
            w[a] = cn * v / s;
        }
    }
}

template <int K>
__device__ __forceinline__ void dweights_f64(double t, double (&dw)[2 * K + 1], double alpha, double cn) {
#pragma unroll
    for (int a = 0; a <= 2 * K; ++a) {
        const int m = a - K;
        const double pa = static_cast<double>(K + m) - t;
        const double pb = static_cast<double>(K - m) + t;
        const double P = pa * pb;
        const double u = t - static_cast<double>(m);
        const double a2 = alpha * alpha;
        double gp;
        if (fabs(a2 * P) < 1.0) {
            double term = alpha * a2 / 6.0, acc = 0.0;
#pragma unroll 1
            for (int n = 1; n < 24; ++n) {
                acc += n * term;
                term *= a2 * P / ((2.0 * n + 2.0) * (2.0 * n + 3.0));
            }
            gp = acc;
        } else if (P > 0.0) {
            const double s = sqrt(P), as = alpha * s;
            gp = (as * cosh(as) - sinh(as)) / (2.0 * s * P);
        } else {
            const double s = sqrt(-P), as = alpha * s;
            gp = -(as * cos(as) - sin(as)) / (2.0 * s * (-P));
        }
        dw[a] = cn * gp * (-2.0 * u);
    }
}

// Error-free transformation (Knuth TwoSum): s + e == a + b exactly.  The
// _rn intrinsics keep the compiler from contracting or reassociating.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    const float bp = __fsub_rn(s, a);
    const float ap = __fsub_rn(s, bp);
    e = __fadd_rn(__fsub_rn(a, ap), __fsub_rn(b, bp));
}

}  // namespace nfft2d
