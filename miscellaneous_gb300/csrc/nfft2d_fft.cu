// nfft2d_fft.cu -- the oversampled FFT of FP32 plans on power-of-two grids,
// written here and fused with the stages around it.
//
// The reference runs the oversampled FFT as a separate library call between
// a deapodize/zero-pad pass and the interpolation (NFFT1_2D.m:48-55) and
// between the spreading and the crop (NFFT2_2D.cu:380-402).  Here each
// direction is two passes over the padded grid, and each pass does the
// neighbouring elementwise stage on the data it holds in shared memory:
//
//   type 2:  k_fft_cols_pad   deapodize + zero-pad + FFT of the N2 band
//                             columns (the other columns are zero and stay
//                             untouched: no pass reads them)
//            k_fft_rows_fill  FFT of every row, reading only its band
//                             columns, writing the row and its periodic halo
//                             (the halo-fill kernel's job)
//   type 1:  k_fft_rows_fold  fold of the spread's halo images onto each row
//                             (the halo-fold kernel's job) + row FFT, writing
//                             back only the band columns
//            k_fft_cols_crop  FFT of the band columns, writing only the N1
//                             band rows, deapodized, to F (the crop)
//
// so a direction moves the grid 1.5 times instead of four separate kernels
// plus the library's two passes.  The index maps are the ones of k_pad /
// k_crop: grid index m holds frequency m (m < n/2) or m - n.
//
// Each CTA transforms P sequences of length n held in shared memory with an
// in-place Stockham autosort FFT: radix-16 butterflies in registers (one per
// thread per stage; one radix-2/4/8 first stage when log2 n is not a
// multiple of 4), so n = 1024 takes three shared-memory round trips.  The
// twiddles come from a per-plan table exp(-2 pi i m / n) computed in FP64 on
// the host.  Column passes keep the P sequences interleaved (element i of
// sequence q at i * P + q, so a warp's global accesses cover P adjacent
// columns of consecutive rows), row passes keep them contiguous; shared
// memory indices carry one pad element per 16.
//
// The plan uses these passes by default below 2048 x 2048 oversampled cells
// (nfft2d_plan.cu, use_fused).  From there up a row of 2048 or 4096 points
// needs 128 or 256 threads at ~115 registers, two CTAs per SM, and cuFFT's
// pruned passes are faster (4096^2: 292 vs 421 us for both directions).
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "nfft2d_internal.h"

namespace nfft2d {
namespace {

constexpr int kFftMaxElems = 4096;  // complex elements per CTA (P * n): 256 threads
constexpr int kFftMinElems = 1024;  // at least 64 threads per CTA
// The kernels declare two CTAs of the largest shape per SM (at most 128
// registers a thread): the fold pass otherwise took 145 and its 512 CTAs of
// 128 threads no longer fitted in one wave on GB300 (14 vs 18 us).

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// s * i * a for s = +-1
__device__ __forceinline__ float2 mul_si(float2 a, float s) { return make_float2(-s * a.y, s * a.x); }

// Shared-memory index with one pad element per 16: the Stockham stores of
// the first stages (each thread writing up to 16 consecutive elements) and
// the interleaved column layout would otherwise hit one bank group.
__device__ __forceinline__ int pad16(int i) { return i + (i >> 4); }
__host__ __device__ inline int padded_elems(int n) { return n + (n >> 4); }

// Element (q, i) of the P sequences: interleaved (column passes) or
// contiguous (row passes).
template <bool INTERLEAVED>
__device__ __forceinline__ int at(int q, int i, int logP, int logN) {
    return pad16(INTERLEAVED ? (i << logP) + q : (q << logN) + i);
}

// In-place 4-point DFT z_q = sum_r a_r w^(rq), w = exp(s 2 pi i / 4).
__device__ __forceinline__ void dft4(float2 &a0, float2 &a1, float2 &a2, float2 &a3, float s) {
    const float2 t0 = cadd(a0, a2), t1 = csub(a0, a2), t2 = cadd(a1, a3), t3 = mul_si(csub(a1, a3), s);
    a0 = cadd(t0, t2);
    a2 = csub(t0, t2);
    a1 = cadd(t1, t3);
    a3 = csub(t1, t3);
}

// cos and sin of pi/8 and pi/4
constexpr float kC8 = 0.92387953251128675613f, kS8 = 0.38268343236508977173f, kR2 = 0.70710678118654752440f;

// 16-point DFT in registers as 4 x 4: y[r1 + 4 r2] -> z[q2 + 4 q1] left at
// y[q1 + 4 q2] (a 4 x 4 transpose of the natural order).
__device__ __forceinline__ void dft16(float2 (&y)[16], float s) {
#pragma unroll
    for (int r1 = 0; r1 < 4; ++r1) dft4(y[r1], y[r1 + 4], y[r1 + 8], y[r1 + 12], s);
    // y[r1 + 4 q2] *= w16^(r1 q2)
    const float2 w1 = make_float2(kC8, s * kS8), w2 = make_float2(kR2, s * kR2), w3 = make_float2(kS8, s * kC8);
    const float2 w6 = make_float2(-kR2, s * kR2), w9 = make_float2(-kC8, -s * kS8);
    y[5] = cmul(y[5], w1);
    y[9] = cmul(y[9], w2);
    y[13] = cmul(y[13], w3);
    y[6] = cmul(y[6], w2);
    y[10] = mul_si(y[10], s);
    y[14] = cmul(y[14], w6);
    y[7] = cmul(y[7], w3);
    y[11] = cmul(y[11], w6);
    y[15] = cmul(y[15], w9);
#pragma unroll
    for (int q2 = 0; q2 < 4; ++q2) dft4(y[4 * q2], y[4 * q2 + 1], y[4 * q2 + 2], y[4 * q2 + 3], s);
}

// 8-point DFT in registers as 2 x 4: y[r1 + 2 r2] -> z[q2 + 4 q1] left at
// y[q1 + 2 q2].
__device__ __forceinline__ void dft8(float2 *y, float s) {
    dft4(y[0], y[2], y[4], y[6], s);
    dft4(y[1], y[3], y[5], y[7], s);
    y[3] = cmul(y[3], make_float2(kR2, s * kR2));
    y[5] = mul_si(y[5], s);
    y[7] = cmul(y[7], make_float2(-kR2, s * kR2));
#pragma unroll
    for (int q2 = 0; q2 < 4; ++q2) {
        const float2 a = y[2 * q2], b = y[2 * q2 + 1];
        y[2 * q2] = cadd(a, b);
        y[2 * q2 + 1] = csub(a, b);
    }
}

// First stage of a length whose log2 is not a multiple of 4: radix R (2, 4
// or 8) at L = 1 (no twiddles), 16/R butterflies per thread.
template <int R, bool INTERLEAVED>
__device__ __forceinline__ void first_stage(float2 *buf, int logN, int logP, float s) {
    constexpr int NB = 16 / R;
    constexpr int LOGR = R == 2 ? 1 : (R == 4 ? 2 : 3);
    const int logB = logN - LOGR;  // N/R butterflies per sequence
    const int T = blockDim.x, t = threadIdx.x;
    float2 y[16];
    int qs[NB], bs[NB];
#pragma unroll
    for (int m = 0; m < NB; ++m) {
        const int bi = t + m * T;
        qs[m] = INTERLEAVED ? (bi & ((1 << logP) - 1)) : (bi >> logB);
        bs[m] = INTERLEAVED ? (bi >> logP) : (bi & ((1 << logB) - 1));
#pragma unroll
        for (int r = 0; r < R; ++r) y[m * R + r] = buf[at<INTERLEAVED>(qs[m], bs[m] + (r << logB), logP, logN)];
    }
    __syncthreads();
#pragma unroll
    for (int m = 0; m < NB; ++m) {
        float2 *z = y + m * R;
        const int q = qs[m], b = bs[m];
        if constexpr (R == 2) {
            buf[at<INTERLEAVED>(q, 2 * b, logP, logN)] = cadd(z[0], z[1]);
            buf[at<INTERLEAVED>(q, 2 * b + 1, logP, logN)] = csub(z[0], z[1]);
        } else if constexpr (R == 4) {
            dft4(z[0], z[1], z[2], z[3], s);
#pragma unroll
            for (int k = 0; k < 4; ++k) buf[at<INTERLEAVED>(q, 4 * b + k, logP, logN)] = z[k];
        } else {
            dft8(z, s);  // z[q2 + 4 q1] sits at z[q1 + 2 q2]
#pragma unroll
            for (int q1 = 0; q1 < 2; ++q1)
#pragma unroll
                for (int q2 = 0; q2 < 4; ++q2)
                    buf[at<INTERLEAVED>(q, 8 * b + q2 + 4 * q1, logP, logN)] = z[q1 + 2 * q2];
        }
    }
    __syncthreads();
}

// The table twiddles of a thread's radix-16 butterflies (at most three
// radix-16 stages for N <= 4096): exp(s 2 pi i j r / 16L) for r = 1, 2, 4, 8.
// Loaded at kernel start so their latency hides behind the grid loads.
struct Twiddles {
    float2 w[3][4];
};

template <bool INTERLEAVED>
__device__ __forceinline__ void prefetch_twiddles(Twiddles &T, int logN, int logP, float s,
                                                  const float2 *__restrict__ tw) {
    const int t = threadIdx.x, logQ = logN - 4;
    const int b = INTERLEAVED ? (t >> logP) : (t & ((1 << logQ) - 1));
#pragma unroll
    for (int st = 0; st < 3; ++st) {
        const int logL = (logN & 3) + 4 * st;
        if (logL >= logN) break;
        const int j = b & ((1 << logL) - 1);
        const int m = j << (logN - logL - 4);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            float2 w = __ldg(tw + (m << e));
            if (s > 0) w.y = -w.y;  // the table holds exp(-2 pi i m / N)
            T.w[st][e] = w;
        }
    }
}

// In-place Stockham FFT of P sequences of length N = 2^logN in (padded)
// shared memory, X_k = sum_m x_m exp(s 2 pi i m k / N).  blockDim.x must be
// P N / 16: every thread holds 16 elements per stage -- one radix-16
// butterfly, or 16/R butterflies of the first stage (radix R = 2^(logN mod
// 4), no twiddles), loaded before a barrier and stored after it.
template <bool INTERLEAVED>
__device__ void fft_inplace(float2 *buf, int logN, int logP, float s, const Twiddles &tws) {
    const int t = threadIdx.x;
    const int rem = logN & 3;
    if (rem == 1) first_stage<2, INTERLEAVED>(buf, logN, logP, s);
    if (rem == 2) first_stage<4, INTERLEAVED>(buf, logN, logP, s);
    if (rem == 3) first_stage<8, INTERLEAVED>(buf, logN, logP, s);
    int logL = rem;
    float2 y[16];
    const int logQ = logN - 4;  // N/16 butterflies per sequence
#pragma unroll
    for (int st = 0; st < 3; ++st, logL += 4) {
        if (logL >= logN) break;
        const int L = 1 << logL;
        const int q = INTERLEAVED ? (t & ((1 << logP) - 1)) : (t >> logQ);
        const int b = INTERLEAVED ? (t >> logP) : (t & ((1 << logQ) - 1));
        const int j = b & (L - 1), k = b >> logL;
#pragma unroll
        for (int r = 0; r < 16; ++r) y[r] = buf[at<INTERLEAVED>(q, b + (r << logQ), logP, logN)];
        __syncthreads();
        if (j) {
            // w^r = exp(s 2 pi i j r / 16L): powers 1, 2, 4, 8 from the table,
            // the rest as products of at most three of them
            float2 w[16];
            w[1] = tws.w[st][0];
            w[2] = tws.w[st][1];
            w[4] = tws.w[st][2];
            w[8] = tws.w[st][3];
            w[3] = cmul(w[1], w[2]);
            w[5] = cmul(w[4], w[1]);
            w[6] = cmul(w[4], w[2]);
            w[7] = cmul(w[4], w[3]);
#pragma unroll
            for (int r = 1; r < 8; ++r) w[8 + r] = cmul(w[8], w[r]);
#pragma unroll
            for (int r = 1; r < 16; ++r) y[r] = cmul(y[r], w[r]);
        }
        dft16(y, s);
        const int o = (k << (logL + 4)) + j;
#pragma unroll
        for (int q1 = 0; q1 < 4; ++q1)
#pragma unroll
            for (int q2 = 0; q2 < 4; ++q2)
                buf[at<INTERLEAVED>(q, o + ((q2 + 4 * q1) << logL), logP, logN)] = y[q1 + 4 * q2];
        __syncthreads();
    }
}

// Band column bc in [0, N2) -> grid column c and coefficient column j
// (c < n2/2 holds k2 = c, j = k2 + N2/2; the upper band holds k2 = c - n2).
__device__ __forceinline__ int band_col(int bc, int N2, int n2) { return bc < N2 / 2 ? bc : n2 - N2 + bc; }
__device__ __forceinline__ int band_coef(int bc, int N2) { return bc < N2 / 2 ? bc + N2 / 2 : bc - N2 / 2; }

struct FftArgs {
    int N1, N2, n1, n2, H, C, R, Cl;
    int logn1, logn2;
    int logP;  // sequences per CTA
    float s;   // exponent sign
};

// Type 2, pass 1: P band columns per CTA.
__global__ void __launch_bounds__(kFftMaxElems / 16, 2) k_fft_cols_pad(const float2 *__restrict__ F, float2 *__restrict__ grid,
                                                              const float *__restrict__ d1,
                                                              const float *__restrict__ d2,
                                                              const float2 *__restrict__ tw, const FftArgs a) {
    extern __shared__ float2 fsm[];
    Twiddles tws;
    prefetch_twiddles<true>(tws, a.logn1, a.logP, a.s, tw);
    const int P = 1 << a.logP, n1 = a.n1;
    const int bc0 = blockIdx.x << a.logP;
    // every thread owns 16 elements (blockDim = P n / 16): all loads first
    float2 v[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) {
        const int e = threadIdx.x + u * blockDim.x;
        const int q = e & (P - 1), r = e >> a.logP, bc = bc0 + q;
        v[u] = make_float2(0.f, 0.f);
        const int k1 = r < n1 / 2 ? r : r - n1;
        if (bc < a.N2 && k1 >= -a.N1 / 2 && k1 < a.N1 / 2) {
            const int i = k1 + a.N1 / 2, j = band_coef(bc, a.N2);
            const float sc = __ldg(d1 + i) * __ldg(d2 + j);
            const float2 f = __ldg(F + static_cast<size_t>(i) * a.N2 + j);
            v[u] = make_float2(f.x * sc, f.y * sc);
        }
    }
#pragma unroll
    for (int u = 0; u < 16; ++u) fsm[pad16(threadIdx.x + u * blockDim.x)] = v[u];
    __syncthreads();
    fft_inplace<true>(fsm, a.logn1, a.logP, a.s, tws);
    const int q = threadIdx.x & (P - 1), bc = bc0 + q;  // blockDim is a multiple of P
    if (bc >= a.N2) return;
    float2 *col = grid + static_cast<size_t>(a.H) * a.C + a.H + band_col(bc, a.N2, a.n2);
#pragma unroll 4
    for (int e = threadIdx.x; e < (n1 << a.logP); e += blockDim.x)
        col[static_cast<size_t>(e >> a.logP) * a.C] = fsm[pad16(e)];
}

// Type 2, pass 2: P rows per CTA; only band columns are read (the rest of
// the column-transformed grid is zero), the whole row and its halo images
// are written: side halo columns for every row, and for the first and last
// H rows the full padded row (every allocated column) in the halo rows.
__global__ void __launch_bounds__(kFftMaxElems / 16, 2) k_fft_rows_fill(float2 *__restrict__ grid,
                                                               const float2 *__restrict__ tw, const FftArgs a) {
    extern __shared__ float2 fsm[];
    Twiddles tws;
    prefetch_twiddles<false>(tws, a.logn2, a.logP, a.s, tw);
    const int n2 = a.n2;
    const int r0 = blockIdx.x << a.logP;
    {
        float2 v[16];
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            const int e = threadIdx.x + u * blockDim.x;
            const int q = e >> a.logn2, c = e & (n2 - 1);
            const int k2 = c < n2 / 2 ? c : c - n2;
            const bool band = k2 >= -a.N2 / 2 && k2 < a.N2 / 2;
            v[u] = band ? grid[static_cast<size_t>(r0 + q + a.H) * a.C + a.H + c] : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < 16; ++u) fsm[pad16(threadIdx.x + u * blockDim.x)] = v[u];
    }
    __syncthreads();
    fft_inplace<false>(fsm, a.logn2, a.logP, a.s, tws);
    const int P = 1 << a.logP;
    for (int q = 0; q < P; ++q) {
        const int r = r0 + q;
        float2 *dst = grid + static_cast<size_t>(r + a.H) * a.C;
        const int base = q << a.logn2;
        for (int col = threadIdx.x; col < a.Cl; col += blockDim.x) {
            int c = col - a.H;
            c += c < 0 ? n2 : (c >= n2 ? -n2 : 0);
            dst[col] = fsm[pad16(base + c)];
        }
        // halo rows: row r's images at padded rows r + H + n1 (r < H) and r + H - n1 (r >= n1 - H)
        int img = -1;
        if (r < a.H) img = r + a.H + a.n1;
        if (r >= a.n1 - a.H) img = r + a.H - a.n1;
        if (img >= 0) {
            float2 *hdst = grid + static_cast<size_t>(img) * a.C;
            for (int col = threadIdx.x; col < a.C; col += blockDim.x) {
                int c = (col - a.H) % n2;
                c += c < 0 ? n2 : 0;
                hdst[col] = fsm[pad16(base + c)];
            }
        }
    }
}

// Type 1, pass 1: P rows per CTA; each interior cell gathers its periodic
// images inside the logical padded grid (R x Cl), the row is transformed and
// only its band columns are written back (in place: a CTA reads other rows'
// images only in halo rows and columns, which no CTA writes).
__global__ void __launch_bounds__(kFftMaxElems / 16, 2) k_fft_rows_fold(float2 *__restrict__ grid,
                                                               const float2 *__restrict__ tw, const FftArgs a) {
    extern __shared__ float2 fsm[];
    Twiddles tws;
    const int n2 = a.n2, n1 = a.n1;
    const int r0 = blockIdx.x << a.logP;
    // images inside the logical padded grid R x Cl = (n1 + 2H) x (n2 + 2H):
    // columns c < H and c >= n2 - H have one side image, rows r < H and
    // r >= n1 - H one row image (with its side image at the corners); only
    // CTAs holding edge rows look at row images
    float2 vs[16];
    const int H = a.H;
#pragma unroll
    for (int u = 0; u < 16; ++u) {
        const int e = threadIdx.x + u * blockDim.x;
        const int q = e >> a.logn2, c = e & (n2 - 1);
        const float2 *src = grid + static_cast<size_t>(r0 + q + H) * a.C + H + c;
        float2 v = *src;
        const int dc = c < H ? n2 : (c >= n2 - H ? -n2 : 0);
        if (dc) v = cadd(v, src[dc]);
        vs[u] = v;
    }
    if (r0 < H || r0 + (1 << a.logP) > n1 - H) {
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            const int e = threadIdx.x + u * blockDim.x;
            const int r = r0 + (e >> a.logn2), c = e & (n2 - 1);
            const int dr = r < H ? n1 : (r >= n1 - H ? -n1 : 0);
            if (!dr) continue;
            const float2 *src = grid + static_cast<size_t>(r + H + dr) * a.C + H + c;
            float2 v = cadd(vs[u], *src);
            const int dc = c < H ? n2 : (c >= n2 - H ? -n2 : 0);
            if (dc) v = cadd(v, src[dc]);
            vs[u] = v;
        }
    }
#pragma unroll
    for (int u = 0; u < 16; ++u) fsm[pad16(threadIdx.x + u * blockDim.x)] = vs[u];
    prefetch_twiddles<false>(tws, a.logn2, a.logP, a.s, tw);
    __syncthreads();
    fft_inplace<false>(fsm, a.logn2, a.logP, a.s, tws);
    for (int e = threadIdx.x; e < (a.N2 << a.logP); e += blockDim.x) {
        const int q = e / a.N2, bc = e - q * a.N2;
        const int c = band_col(bc, a.N2, n2);
        grid[static_cast<size_t>(r0 + q + a.H) * a.C + a.H + c] = fsm[pad16((q << a.logn2) + c)];
    }
}

// Type 1, pass 2: P band columns per CTA, transformed, cropped to the N1 band
// rows and deapodized into F (N1 x N2, row-major).
__global__ void __launch_bounds__(kFftMaxElems / 16, 2) k_fft_cols_crop(const float2 *__restrict__ grid, float2 *__restrict__ F,
                                                               const float *__restrict__ d1,
                                                               const float *__restrict__ d2,
                                                               const float2 *__restrict__ tw, const FftArgs a) {
    extern __shared__ float2 fsm[];
    Twiddles tws;
    prefetch_twiddles<true>(tws, a.logn1, a.logP, a.s, tw);
    const int P = 1 << a.logP, n1 = a.n1;
    const int bc0 = blockIdx.x << a.logP;
    {
        float2 v[16];
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            const int e = threadIdx.x + u * blockDim.x;
            const int q = e & (P - 1), r = e >> a.logP, bc = bc0 + q;
            v[u] = bc < a.N2 ? grid[static_cast<size_t>(r + a.H) * a.C + a.H + band_col(bc, a.N2, a.n2)]
                             : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < 16; ++u) fsm[pad16(threadIdx.x + u * blockDim.x)] = v[u];
    }
    __syncthreads();
    fft_inplace<true>(fsm, a.logn1, a.logP, a.s, tws);
    // blockDim is a multiple of P, so a thread keeps one column q
    const int q = threadIdx.x & (P - 1), bc = bc0 + q;
    if (bc >= a.N2) return;
    const int j = band_coef(bc, a.N2);
    const float s2 = __ldg(d2 + j);
#pragma unroll 4
    for (int e = threadIdx.x; e < (a.N1 << a.logP); e += blockDim.x) {
        const int i = e >> a.logP;
        const int k1 = i - a.N1 / 2, r = k1 < 0 ? k1 + n1 : k1;
        const float sc = __ldg(d1 + i) * s2;
        const float2 g = fsm[pad16((r << a.logP) + q)];
        F[static_cast<size_t>(i) * a.N2 + j] = make_float2(g.x * sc, g.y * sc);
    }
}

int ilog2(int n) {
    int l = 0;
    while ((1 << l) < n) ++l;
    return l;
}

// sequences per CTA: up to kFftMaxElems elements, fewer while that leaves
// under min_ctas CTAs, but not under kFftMinElems (or one sequence).  The
// thread count (16 elements each) does not depend on it: the column passes
// keep more columns per CTA (one 32-byte sector per row at P = 4) and accept
// fewer, larger CTAs.
int seqs_log(int logn, int seqs, int min_ctas) {
    int logP = ilog2(kFftMaxElems) - logn;
    if (logP < 0) logP = 0;
    while (logP > 0 && (seqs >> logP) < min_ctas && (1 << (logn + logP - 1)) >= kFftMinElems) --logP;
    return logP;
}

FftArgs fft_args(const nfft2d_plan_s *p, int sign) {
    const Geom &g = p->g;
    FftArgs a{};
    a.N1 = p->N1;
    a.N2 = p->N2;
    a.n1 = g.n1;
    a.n2 = g.n2;
    a.H = g.H;
    a.C = g.C;
    a.R = g.R;
    a.Cl = g.Cl;
    a.logn1 = ilog2(g.n1);
    a.logn2 = ilog2(g.n2);
    a.s = sign < 0 ? -1.f : 1.f;
    return a;
}

// Dynamic shared memory above the 48 KB default needs an opt-in per kernel.
template <typename KernelT>
cudaError_t allow_smem(KernelT kernel, int smem) {
    if (smem > 48 * 1024) return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    return cudaSuccess;
}

}  // namespace

bool fused_fft_eligible(int precision, int n1, int n2) {
    auto pow2 = [](int n) { return n >= 64 && n <= kFftMaxElems && (n & (n - 1)) == 0; };
    return precision == NFFT2D_F32 && pow2(n1) && pow2(n2);
}

int setup_fused_fft(nfft2d_plan_s *p) {
    if (p->tw1 || p->tw2) cudaStreamSynchronize(p->stream);  // no transform on the old tables in flight
    plan_free(p->tw1);
    plan_free(p->tw2);
    p->tw1 = p->tw2 = nullptr;
    p->fused_ok = false;
    if (!fused_fft_eligible(p->precision, p->g.n1, p->g.n2)) return NFFT2D_OK;
    for (int d = 0; d < 2; ++d) {
        const int n = d == 0 ? p->g.n1 : p->g.n2;
        std::vector<float2> h(n);
        for (int m = 0; m < n; ++m) {
            const double ang = -2.0 * 3.141592653589793238462643383279502884 * m / n;
            h[m] = make_float2(static_cast<float>(std::cos(ang)), static_cast<float>(std::sin(ang)));
        }
        float2 **dst = d == 0 ? &p->tw1 : &p->tw2;
        if (plan_malloc(reinterpret_cast<void **>(dst), sizeof(float2) * n) != cudaSuccess) return NFFT2D_ERR_OOM;
        if (cudaMemcpyAsync(*dst, h.data(), sizeof(float2) * n, cudaMemcpyHostToDevice, p->stream) != cudaSuccess ||
            cudaStreamSynchronize(p->stream) != cudaSuccess)
            return NFFT2D_ERR_CUDA;
    }
    p->fused_ok = true;
    return NFFT2D_OK;
}

cudaError_t fused_type2_cols(const nfft2d_plan_s *p, int sign, const void *F) {
    FftArgs a = fft_args(p, sign);
    a.logP = seqs_log(a.logn1, p->N2, p->num_sms / 2);
    const int blocks = (p->N2 + (1 << a.logP) - 1) >> a.logP;
    const int threads = (a.n1 << a.logP) / 16;
    const int smem = padded_elems(a.n1 << a.logP) * static_cast<int>(sizeof(float2));
    cudaError_t e = allow_smem(k_fft_cols_pad, smem);
    if (e != cudaSuccess) return e;
    k_fft_cols_pad<<<blocks, threads, smem, p->stream>>>(
        static_cast<const float2 *>(F), static_cast<float2 *>(p->grid), static_cast<const float *>(p->deap1),
        static_cast<const float *>(p->deap2), p->tw1, a);
    return cudaGetLastError();
}

cudaError_t fused_type2_rows(const nfft2d_plan_s *p, int sign) {
    FftArgs a = fft_args(p, sign);
    a.logP = seqs_log(a.logn2, a.n1, 2 * p->num_sms);
    const int blocks = a.n1 >> a.logP;
    const int threads = (a.n2 << a.logP) / 16;
    const int smem = padded_elems(a.n2 << a.logP) * static_cast<int>(sizeof(float2));
    cudaError_t e = allow_smem(k_fft_rows_fill, smem);
    if (e != cudaSuccess) return e;
    k_fft_rows_fill<<<blocks, threads, smem, p->stream>>>(static_cast<float2 *>(p->grid), p->tw2, a);
    return cudaGetLastError();
}

cudaError_t fused_type1_rows(const nfft2d_plan_s *p, int sign) {
    FftArgs a = fft_args(p, sign);
    a.logP = seqs_log(a.logn2, a.n1, 2 * p->num_sms);
    const int blocks = a.n1 >> a.logP;
    const int threads = (a.n2 << a.logP) / 16;
    const int smem = padded_elems(a.n2 << a.logP) * static_cast<int>(sizeof(float2));
    cudaError_t e = allow_smem(k_fft_rows_fold, smem);
    if (e != cudaSuccess) return e;
    k_fft_rows_fold<<<blocks, threads, smem, p->stream>>>(static_cast<float2 *>(p->grid), p->tw2, a);
    return cudaGetLastError();
}

cudaError_t fused_type1_cols(const nfft2d_plan_s *p, int sign, void *F) {
    FftArgs a = fft_args(p, sign);
    a.logP = seqs_log(a.logn1, p->N2, p->num_sms / 2);
    const int blocks = (p->N2 + (1 << a.logP) - 1) >> a.logP;
    const int threads = (a.n1 << a.logP) / 16;
    const int smem = padded_elems(a.n1 << a.logP) * static_cast<int>(sizeof(float2));
    cudaError_t e = allow_smem(k_fft_cols_crop, smem);
    if (e != cudaSuccess) return e;
    k_fft_cols_crop<<<blocks, threads, smem, p->stream>>>(
        static_cast<const float2 *>(p->grid), static_cast<float2 *>(F), static_cast<const float *>(p->deap1),
        static_cast<const float *>(p->deap2), p->tw1, a);
    return cudaGetLastError();
}

}  // namespace nfft2d
