// nfft2d_type3.cu -- type-3 2D NUFFT (nonuniform points to nonuniform
// frequencies) by Gaussian gridding, the reference's other native NUFFT:
//     F_k = sum_j f_j exp(-i (s_k x_j + t_k y_j))
// following NUFFT_2D_CPU (NFFT/NFFT3/C/NFFT3_2D_C.cpp:199-312): extents and
// centres of both point sets, R = 2.2 and the Gaussian half-width msp for
// the requested accuracy (:234-238), a rescaling that maps the points onto
// [-pi/2, pi/2] around their centre (:243-264), then
//   1) Gaussian spreading of the phase-shifted values onto an Mry x Mrx grid
//      with the pre-compensation exp(b (Dy^2 n_j^2 + Dx^2 n_i^2)) (:38-85);
//   2) a forward 2D FFT (cuFFT here, MKL there, :283-292);
//   3) Gaussian gathering at the scaled frequencies with the
//      post-compensation and the phase of the centres (:156-194).
// The reference's circular shift by half the grid with the (-1)^(i+j)
// checkerboard (:135-151) is folded into the gather's indexing: no pass.
//
// Kernels: the Gaussian weight of a footprint tap factors into a row and a
// column weight, so a point or frequency needs 2(2 msp + 1) exponentials
// (FP64, from FP64 coordinates), not (2 msp + 1)^2.  The spread bins the
// points by 16 x 16 grid tile and accumulates each tile's points in a
// shared-memory patch (warps own disjoint patch rows: no atomics) that one
// global atomic add per cell puts into the grid; the gather runs one warp
// per output frequency over the footprint with coalesced row reads and a
// warp-shuffle reduction.  The grid, the products and the sums use the
// data precision.
#include <cuda_runtime.h>
#include <cufft.h>

#include <cfloat>
#include <cmath>
#include <cstring>

#include "nfft2d_internal.h"

namespace {

constexpr double kPi = 3.141592653589793238463;  // the reference's PI (NFFT3_2D_C.cpp:24)
constexpr int kWarpsPerBlock = 8;

__device__ __forceinline__ unsigned long long ord_key(double v) {
    const unsigned long long u = static_cast<unsigned long long>(__double_as_longlong(v));
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
double ord_value(unsigned long long k) {
    const unsigned long long u = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    double v;
    std::memcpy(&v, &u, sizeof v);
    return v;
}

// min / max of two arrays of n values: mm[0..3] = keys of min a, max a, min b, max b
__global__ void k_minmax2(const double *__restrict__ a, const double *__restrict__ b, long long n,
                          unsigned long long *mm) {
    double amin = DBL_MAX, amax = -DBL_MAX, bmin = DBL_MAX, bmax = -DBL_MAX;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        amin = fmin(amin, a[i]);
        amax = fmax(amax, a[i]);
        bmin = fmin(bmin, b[i]);
        bmax = fmax(bmax, b[i]);
    }
    for (int o = 16; o > 0; o >>= 1) {
        amin = fmin(amin, __shfl_xor_sync(0xffffffffu, amin, o));
        amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, o));
        bmin = fmin(bmin, __shfl_xor_sync(0xffffffffu, bmin, o));
        bmax = fmax(bmax, __shfl_xor_sync(0xffffffffu, bmax, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(mm + 0, ord_key(amin));
        atomicMax(mm + 1, ord_key(amax));
        atomicMin(mm + 2, ord_key(bmin));
        atomicMax(mm + 3, ord_key(bmax));
    }
}

struct Params {
    double xb, yb, sb, tb;   // centres after the rescaling
    double kx, ky;           // rescaling X1 / (pi/2), Y1 / (pi/2)
    double Dx, Dy;           // grid steps 2 pi / Mr
    double b, t1, fact;      // Gaussian constants, fact = (1 / (4 pi b))^2
    int Mrx, Mry, ms;        // grid and footprint half-width
};

__device__ __forceinline__ int wrap(long long i, int n) {
    long long r = i % n;
    return static_cast<int>(r < 0 ? r + n : r);
}

// ---------------------------------------------------------------------------
// Spreading (NFFT3_2D_C.cpp:38-85), binned.  Tap (r, c) of a point has the
// weight exp(ex(c) + ey(r)) with ex depending on the column only and ey on
// the row only (:61-74), so a point needs 2(2ms+1) exponentials, not
// (2ms+1)^2, and the products wr(r) wc(c) are formed in the data precision.
// Points are binned by the TS x TS grid tile of their footprint's first
// cell; a CTA accumulates one work item (at most kT3Item points of one
// tile) into a shared-memory patch of (TS + W - 1)^2 cells -- warp w owns
// the patch rows r = w (mod 8), so no two threads ever touch one cell and no
// shared atomics are needed -- and adds the patch into the grid with one
// global atomic add per cell and component.
// ---------------------------------------------------------------------------
constexpr int kT3Tile = 16;    // TS
constexpr int kT3Item = 1024;  // points per work item
constexpr int kT3Warps = 8;    // warps of a spreading CTA

struct T3Rec {
    double xt, yt;  // (x - xb) / Dx, (y - yb) / Dy (:53-54)
    double re, im;  // the value with the centre phase removed and the constant factor (:48-51)
    int i0, j0;     // first footprint column and row, unwrapped (floor(M/2 + t) - ms)
};

// The pre-compensation factors exp(b D^2 ds^2) of every grid offset ds a
// footprint can reach (FP64, stored as FP32 for the FP32 spread):
// tab[ds + off], ds in [-off, n - off).
__global__ void k_t3_table(float *__restrict__ tab, int n, int off, double bD2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double d = static_cast<double>(i - off);
    tab[i] = static_cast<float>(exp(bD2 * d * d));
}

// Per point: the record fields and its tile; the rank within the tile from
// the tile's counter.
template <typename C2>
__global__ void k_t3_prep(const double *__restrict__ x, const double *__restrict__ y, const C2 *__restrict__ f,
                          long long n, Params P, int tiles_x, T3Rec *__restrict__ tmp, int2 *__restrict__ tile_rank,
                          unsigned *__restrict__ counts) {
    const long long p = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
    if (p >= n) return;
    const double xs = x[p] / P.kx, ys = y[p] / P.ky;  // :245-246
    const double arg = P.sb * xs + P.tb * ys;
    double sa, ca;
    sincos(arg, &sa, &ca);
    const double fr = static_cast<double>(f[p].x), fi = static_cast<double>(f[p].y);
    T3Rec r;
    r.re = (fr * ca + fi * sa) * P.fact;
    r.im = (fi * ca - fr * sa) * P.fact;
    r.xt = (xs - P.xb) / P.Dx;
    r.yt = (ys - P.yb) / P.Dy;
    r.i0 = static_cast<int>(floor(P.Mrx / 2 + r.xt)) - P.ms;
    r.j0 = static_cast<int>(floor(P.Mry / 2 + r.yt)) - P.ms;
    const int tile = (wrap(r.j0, P.Mry) / kT3Tile) * tiles_x + wrap(r.i0, P.Mrx) / kT3Tile;
    tmp[p] = r;
    tile_rank[p] = make_int2(tile, static_cast<int>(atomicAdd(counts + tile, 1u)));
}

// One CTA: exclusive scan of the tile counts into starts, and of the work
// items per tile; counts[ntiles] receives the number of work items.
__global__ void __launch_bounds__(1024) k_t3_scan(unsigned *__restrict__ counts, int ntiles,
                                                  unsigned *__restrict__ starts, unsigned *__restrict__ item_starts) {
    __shared__ unsigned s_pts[32], s_items[32];
    __shared__ unsigned carry_pts, carry_items;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) carry_pts = carry_items = 0;
    __syncthreads();
    for (int base = 0; base < ntiles; base += 1024) {
        const int i = base + tid;
        const unsigned c = i < ntiles ? counts[i] : 0u;
        const unsigned it = (c + kT3Item - 1) / kT3Item;
        unsigned a = c, b = it;  // inclusive warp scans
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned ua = __shfl_up_sync(0xffffffffu, a, o), ub = __shfl_up_sync(0xffffffffu, b, o);
            if (lane >= o) {
                a += ua;
                b += ub;
            }
        }
        if (lane == 31) {
            s_pts[warp] = a;
            s_items[warp] = b;
        }
        __syncthreads();
        if (warp == 0) {
            unsigned wa = s_pts[lane], wb = s_items[lane];
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned ua = __shfl_up_sync(0xffffffffu, wa, o), ub = __shfl_up_sync(0xffffffffu, wb, o);
                if (lane >= o) {
                    wa += ua;
                    wb += ub;
                }
            }
            s_pts[lane] = wa;
            s_items[lane] = wb;
        }
        __syncthreads();
        const unsigned before_pts = carry_pts + (warp ? s_pts[warp - 1] : 0u) + a - c;
        const unsigned before_items = carry_items + (warp ? s_items[warp - 1] : 0u) + b - it;
        if (i < ntiles) {
            starts[i] = before_pts;
            item_starts[i] = before_items;
        }
        __syncthreads();
        if (tid == 0) {
            carry_pts += s_pts[31];
            carry_items += s_items[31];
        }
        __syncthreads();
    }
    if (tid == 0) counts[ntiles] = carry_items;
}

// Records to their tile's range; the tile's work items {tile, first, count}.
__global__ void k_t3_scatter(const T3Rec *__restrict__ tmp, const int2 *__restrict__ tile_rank, long long n,
                             const unsigned *__restrict__ starts, T3Rec *__restrict__ recs) {
    const long long p = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
    if (p >= n) return;
    const int2 tr = tile_rank[p];
    recs[starts[tr.x] + static_cast<unsigned>(tr.y)] = tmp[p];
}

__global__ void k_t3_items(const unsigned *__restrict__ counts, const unsigned *__restrict__ starts,
                           const unsigned *__restrict__ item_starts, int ntiles, int4 *__restrict__ items) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntiles) return;
    const unsigned c = counts[t];
    for (unsigned k = 0; k * kT3Item < c; ++k)
        items[item_starts[t] + k] = make_int4(t, static_cast<int>(starts[t] + k * kT3Item),
                                              static_cast<int>(min(static_cast<unsigned>(kT3Item), c - k * kT3Item)),
                                              0);
}

// Dynamic shared memory of a spreading CTA: the patch, then B points'
// row and column weights, values, patch origins and fractional offsets.
__host__ __device__ inline size_t t3_spread_smem(int W, int B, size_t real_bytes) {
    const size_t PP = static_cast<size_t>(kT3Tile + W - 1);
    return PP * PP * 2 * real_bytes + static_cast<size_t>(B) * (2 * W + 2) * real_bytes +
           static_cast<size_t>(B) * (sizeof(int2) + sizeof(float2)) + 16;
}

template <typename Real>
__global__ void __launch_bounds__(kT3Warps * 32)
    k_t3_spread(const T3Rec *__restrict__ recs, const int4 *__restrict__ items, const unsigned *__restrict__ n_items,
                Params P, int tiles_x, int B, const float *__restrict__ prex, int tabo_x, const float *__restrict__ prey,
                int tabo_y, Real *__restrict__ grid) {
    extern __shared__ __align__(16) unsigned char t3_smem[];
    const int it = blockIdx.x;
    if (it >= static_cast<int>(*n_items)) return;
    const int4 item = items[it];
    const int W = 2 * P.ms + 1, PP = kT3Tile + W - 1;
    Real *patch = reinterpret_cast<Real *>(t3_smem);  // PP x PP complex, row-major
    Real *wgt = patch + 2 * PP * PP;                  // per point: W row weights, then W column weights
    Real *pval = wgt + 2 * B * W;                     // per point: the value
    int2 *pinfo = reinterpret_cast<int2 *>(pval + 2 * B);  // per point: patch row, column of its first cell
    float2 *pfrac = reinterpret_cast<float2 *>(pinfo + B);  // per point: fractional x, y offsets
    const float t1f = static_cast<float>(P.t1);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int i = tid; i < 2 * PP * PP; i += blockDim.x) patch[i] = Real(0);
    const int tr0 = (item.x / tiles_x) * kT3Tile, tc0 = (item.x % tiles_x) * kT3Tile;  // tile origin (wrapped)
    for (int b0 = 0; b0 < item.z; b0 += B) {
        const int nb = min(B, item.z - b0);
        __syncthreads();  // the previous batch's weights are consumed (and the patch zeroed)
        // per point: its patch origin and value; weights: point q, k < W rows
        // then W columns (:61-74), FP64 exponentials
        for (int q = tid; q < nb; q += blockDim.x) {
            const T3Rec &r = recs[item.y + b0 + q];
            pinfo[q] = make_int2(wrap(r.j0, P.Mry) - tr0, wrap(r.i0, P.Mrx) - tc0);
            pval[2 * q] = static_cast<Real>(r.re);
            pval[2 * q + 1] = static_cast<Real>(r.im);
            // fractional offsets within the first cell: the Gaussian's argument
            // yt - dsj = fy + ms - k (exact integer part, FP64 difference once)
            pfrac[q] = make_float2(static_cast<float>(r.xt - floor(r.xt)), static_cast<float>(r.yt - floor(r.yt)));
        }
        __syncthreads();
        for (int e = tid; e < nb * 2 * W; e += blockDim.x) {
            const int q = e / (2 * W), k = e - q * 2 * W;
            const T3Rec &r = recs[item.y + b0 + q];
            const bool row = k < W;
            const int kk = row ? k : k - W;
            const int ds = row ? r.j0 + kk - P.Mry / 2 : r.i0 + kk - P.Mrx / 2;  // dsj or dsi (:61-74)
            if constexpr (sizeof(Real) == sizeof(double)) {
                const double d = static_cast<double>(ds);
                const double t = row ? r.yt : r.xt;
                const double D = row ? P.Dy : P.Dx;
                wgt[q * 2 * W + k] = exp(P.b * D * D * d * d - P.t1 * (t - d) * (t - d));
            } else {
                // FP32 data: exp(b D^2 ds^2) from the table (FP64-computed),
                // the Gaussian exp(-t1 (frac + ms - k)^2) in FP32 on an exact
                // argument
                const float fr = row ? pfrac[q].y : pfrac[q].x;
                const float g = fr + static_cast<float>(P.ms - kk);
                const int ti = row ? min(max(ds + tabo_y, 0), 2 * tabo_y)
                                   : min(max(ds + tabo_x, 0), 2 * tabo_x);  // inside the table by construction
                const float pre = row ? prey[ti] : prex[ti];
                wgt[q * 2 * W + k] = pre * expf(-t1f * g * g);
            }
        }
        __syncthreads();
        for (int q = 0; q < nb; ++q) {
            // footprint origin in the patch: the tile offset of the first cell
            const int2 o = pinfo[q];
            const int lr = o.x, lc = o.y;
            const Real *wr = wgt + q * 2 * W, *wc = wr + W;
            const Real vr = pval[2 * q], vi = pval[2 * q + 1];
            // this lane's columns c = lane + 32 m of the footprint: v * wc(c)
            for (int c0 = 0; c0 < W; c0 += 32) {
                const int c = c0 + lane;
                if (c >= W) continue;
                const Real ax = vr * wc[c], ay = vi * wc[c];
                Real *col = patch + 2 * (lc + c);
#pragma unroll 4
                for (int k = (warp - lr % kT3Warps + kT3Warps) % kT3Warps; k < W; k += kT3Warps) {
                    Real *cell = col + 2 * (lr + k) * PP;  // patch row lr + k = warp (mod 8)
                    const Real w = wr[k];
                    cell[0] += ax * w;
                    cell[1] += ay * w;
                }
            }
        }
    }
    __syncthreads();
    for (int i = tid; i < PP * PP; i += blockDim.x) {
        const Real ax = patch[2 * i], ay = patch[2 * i + 1];
        if (ax == Real(0) && ay == Real(0)) continue;
        const int pr = i / PP, pc = i - pr * PP;
        Real *g = grid + 2 * (static_cast<size_t>(wrap(tr0 + pr, P.Mry)) * P.Mrx + wrap(tc0 + pc, P.Mrx));
        atomicAdd(g, ax);
        atomicAdd(g + 1, ay);
    }
}

// ---------------------------------------------------------------------------
// Gathering (:156-194).  The Gaussian weight of tap (r, c) is
// exp(-t1 (difs - npj)^2) exp(-t1 (dift - npi)^2) and the shift's (-1)^(i+j)
// (:147-148) is (-1)^i (-1)^j, so both factor per column and per row.  A
// warp owns 32 output frequencies: each lane sets up one of them (FP64:
// scaling, cell, fractional offsets, the post-compensation and the centres'
// phase), then the warp sums the footprints one frequency after the other --
// lane l owns footprint columns l and l + 32 and runs down the rows -- and
// the lane that owns the frequency finishes it.  FP32 data take the
// Gaussian factors in FP32 on exact arguments (fractional offset + integer).
// ---------------------------------------------------------------------------
template <typename C2, typename Real>
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
    k_t3_gather(const double *__restrict__ s, const double *__restrict__ t, long long n, Params P,
                const C2 *__restrict__ grid, C2 *__restrict__ F) {
    const long long k0 = (blockIdx.x * static_cast<long long>(kWarpsPerBlock) + (threadIdx.x >> 5)) * 32;
    const int lane = threadIdx.x & 31;
    if (k0 >= n) return;
    const long long k = k0 + lane;
    const bool mine = k < n;
    // this lane's frequency (:163-172, :189)
    double ss = 0.0, ts = 0.0;
    if (mine) {
        ss = s[k] * P.kx;  // :247-248
        ts = t[k] * P.ky;
    }
    const double us = P.Mrx / 2 + (ss - P.sb), ut = P.Mry / 2 + (ts - P.tb);  // Ds = Dt = 1
    const double fs = floor(us), ft = floor(ut);
    const Real difs = static_cast<Real>(us - fs), dift = static_cast<Real>(ut - ft);
    const int ifirst = wrap(static_cast<long long>(fs) - P.ms + P.Mrx / 2, P.Mrx);
    const int jfirst = wrap(static_cast<long long>(ft) - P.ms + P.Mry / 2, P.Mry);
    const int W = 2 * P.ms + 1;
    const Real t1 = static_cast<Real>(P.t1);
    Real res0 = Real(0), res1 = Real(0);
    const int nk = static_cast<int>(min(32LL, n - k0));
    for (int o = 0; o < nk; ++o) {
        const Real ds = __shfl_sync(0xffffffffu, difs, o), dt = __shfl_sync(0xffffffffu, dift, o);
        const int i0 = __shfl_sync(0xffffffffu, ifirst, o), j0 = __shfl_sync(0xffffffffu, jfirst, o);
        // row weights of rows lane + 32 m (the grid has even sides: the
        // wrapped row's parity is that of j0 + r)
        Real wrow[3];
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            const int r = lane + 32 * m;
            const Real g = dt - static_cast<Real>(r - P.ms);
            const Real e = r < W ? exp(-t1 * g * g) : Real(0);
            wrow[m] = ((j0 + r) & 1) ? -e : e;
        }
        Real acc0 = Real(0), acc1 = Real(0);
        for (int c0 = 0; c0 < W; c0 += 32) {
            const int c = c0 + lane;
            const bool on = c < W;
            const int cc = on ? c : 0;
            const int i = i0 + cc >= P.Mrx ? i0 + cc - P.Mrx : i0 + cc;
            const Real g = ds - static_cast<Real>(cc - P.ms);
            const Real es = exp(-t1 * g * g);
            // lanes past the footprint read a valid cell and weigh it by 0
            const Real wcol = on ? (((i0 + cc) & 1) ? -es : es) : Real(0);
            const C2 *col = grid + i;
            Real s0 = Real(0), s1 = Real(0);
            int j = j0;
#pragma unroll
            for (int m = 0; m < 3; ++m) {  // footprint rows 32 m .. 32 m + 31
                const int rn = min(32, W - 32 * m);
#pragma unroll 8
                for (int rr = 0; rr < rn; ++rr) {
                    const Real wr = __shfl_sync(0xffffffffu, wrow[m], rr);
                    const C2 v = col[static_cast<size_t>(j) * P.Mrx];
                    s0 += static_cast<Real>(v.x) * wr;
                    s1 += static_cast<Real>(v.y) * wr;
                    j = j + 1 == P.Mry ? 0 : j + 1;
                }
            }
            acc0 += s0 * wcol;
            acc1 += s1 * wcol;
        }
        for (int x = 16; x > 0; x >>= 1) {
            acc0 += __shfl_xor_sync(0xffffffffu, acc0, x);
            acc1 += __shfl_xor_sync(0xffffffffu, acc1, x);
        }
        if (lane == o) {
            res0 = acc0;
            res1 = acc1;
        }
    }
    if (mine) {
        double tmp1 = P.Dy * (ts - P.tb);
        tmp1 = tmp1 * tmp1;
        double tmp2 = P.Dx * (ss - P.sb);
        tmp2 = tmp2 * tmp2;
        const double comp = exp(P.b * (tmp1 + tmp2));                 // :170-172
        const double arg = (ss - P.sb) * P.xb + (ts - P.tb) * P.yb;   // :189
        double sa, ca;
        sincos(arg, &sa, &ca);
        const double a0 = static_cast<double>(res0), a1 = static_cast<double>(res1);
        C2 out;
        out.x = static_cast<decltype(out.x)>((a0 * ca + a1 * sa) * comp);
        out.y = static_cast<decltype(out.x)>((a1 * ca - a0 * sa) * comp);
        F[k] = out;
    }
}

int cuda_status(cudaError_t e) {
    if (e == cudaSuccess) return NFFT2D_OK;
    return e == cudaErrorMemoryAllocation ? NFFT2D_ERR_OOM : NFFT2D_ERR_CUDA;
}

#define T3_CUDA(expr)                                   \
    do {                                                \
        const int st_ = cuda_status(expr);              \
        if (st_ != NFFT2D_OK) return st_;               \
    } while (0)

int minmax(const double *a, const double *b, long long n, unsigned long long *d_mm, cudaStream_t st, double out[4]) {
    const unsigned long long init[4] = {~0ull, 0ull, ~0ull, 0ull};
    T3_CUDA(cudaMemcpyAsync(d_mm, init, sizeof init, cudaMemcpyHostToDevice, st));
    const int blocks = static_cast<int>(std::max<long long>(1, std::min<long long>((n + 255) / 256, 1024)));
    k_minmax2<<<blocks, 256, 0, st>>>(a, b, n, d_mm);
    T3_CUDA(cudaGetLastError());
    unsigned long long h[4];
    T3_CUDA(cudaMemcpyAsync(h, d_mm, sizeof h, cudaMemcpyDeviceToHost, st));
    T3_CUDA(cudaStreamSynchronize(st));
    for (int i = 0; i < 4; ++i) out[i] = ord_value(h[i]);
    return NFFT2D_OK;
}

struct Scratch {
    cudaStream_t st;
    void *mm = nullptr, *grid = nullptr;
    cufftHandle plan = 0;
    bool plan_ok = false;
    ~Scratch() {
        if (plan_ok) {
            cudaStreamSynchronize(st);  // no FFT in flight when the handle goes back to the pool
            nfft2d::pooled_plan_release(plan);
        }
        if (grid) cudaFreeAsync(grid, st);
        if (mm) cudaFreeAsync(mm, st);
    }
};

}  // namespace

extern "C" int nfft2d_nufft3_2d(const double *x, const double *y, const double *s, const double *t, const void *f,
                                void *F, double eps, long long len_in, long long len_out, int precision,
                                void *stream) {
    if (!x || !y || !s || !t || !f || !F || len_in < 1 || len_out < 1) return NFFT2D_ERR_INVALID_ARG;
    if (!(eps > 0 && eps < 1)) return NFFT2D_ERR_INVALID_ARG;
    if (precision != NFFT2D_F32 && precision != NFFT2D_F64) return NFFT2D_ERR_INVALID_ARG;
    if (len_in > (1LL << 40) || len_out > (1LL << 40)) return NFFT2D_ERR_INVALID_ARG;
    const cudaStream_t st = static_cast<cudaStream_t>(stream);
    Scratch S{st};
    T3_CUDA(cudaMallocAsync(&S.mm, 4 * sizeof(unsigned long long), st));
    double exy[4], est[4];
    int rc = minmax(x, y, len_in, static_cast<unsigned long long *>(S.mm), st, exy);
    if (rc != NFFT2D_OK) return rc;
    rc = minmax(s, t, len_out, static_cast<unsigned long long *>(S.mm), st, est);
    if (rc != NFFT2D_OK) return rc;
    for (double v : exy)
        if (!std::isfinite(v)) return NFFT2D_ERR_NONFINITE;
    for (double v : est)
        if (!std::isfinite(v)) return NFFT2D_ERR_NONFINITE;
    // :214-232 (the reductions start from -+FLT_MAX, which finite data within
    // range never leaves)
    double Max_x = exy[1], min_x = exy[0], Max_y = exy[3], min_y = exy[2];
    double Max_s = est[1], min_s = est[0], Max_t = est[3], min_t = est[2];
    double xb = (Max_x + min_x) / 2, X1 = std::fabs(Max_x - xb);
    double yb = (Max_y + min_y) / 2, Y1 = std::fabs(Max_y - yb);
    double sb = (Max_s + min_s) / 2, Sx = std::fabs(Max_s - sb);
    double tb = (Max_t + min_t) / 2, Ty = std::fabs(Max_t - tb);
    if (!(X1 > 0) || !(Y1 > 0)) return NFFT2D_ERR_INVALID_ARG;  // all points on one line: no scale
    const double R = 2.2;
    double msp = 2 + 2 * (R * R) * (-std::log(eps / 76)) / (kPi * (R * R - 2));  // :235
    const double mrx = 2 * std::ceil((X1 * Sx / kPi) * R * R + R * msp);         // :237-238
    const double mry = 2 * std::ceil((Y1 * Ty / kPi) * R * R + R * msp);
    if (!(mrx <= 65536) || !(mry <= 65536) || mrx * mry > 1.5e9) return NFFT2D_ERR_UNSUPPORTED;
    Params P{};
    P.Mrx = static_cast<int>(mrx);
    P.Mry = static_cast<int>(mry);
    P.Dx = 2 * kPi / P.Mrx;
    P.Dy = 2 * kPi / P.Mry;
    P.kx = X1 / (kPi / 2);
    P.ky = Y1 / (kPi / 2);
    Max_x = Max_x / P.kx;
    min_x = min_x / P.kx;
    P.xb = (Max_x + min_x) / 2;
    Max_s = Max_s * P.kx;
    min_s = min_s * P.kx;
    P.sb = (Max_s + min_s) / 2;
    Max_y = Max_y / P.ky;
    min_y = min_y / P.ky;
    P.yb = (Max_y + min_y) / 2;
    Max_t = Max_t * P.ky;
    min_t = min_t * P.ky;
    P.tb = (Max_t + min_t) / 2;
    P.b = (msp - 2) / (4 * kPi);
    P.t1 = 1 / (4 * P.b);
    msp = std::floor(msp - 2);
    P.ms = static_cast<int>(msp);
    const double f0 = 1. / (4. * kPi * P.b);
    P.fact = f0 * f0;

    const bool dbl = precision == NFFT2D_F64;
    const int W = 2 * P.ms + 1;
    if (W > 96) return NFFT2D_ERR_UNSUPPORTED;  // the gather's lanes hold at most 96 row weights
    const size_t rb = dbl ? sizeof(double) : sizeof(float);
    int B = 32;  // points per weight batch of the spread
    while (B > 4 && t3_spread_smem(W, B, rb) > 227 * 1024) B /= 2;
    const size_t smem = t3_spread_smem(W, B, rb);
    if (smem > 227 * 1024) return NFFT2D_ERR_UNSUPPORTED;
    const size_t cells = static_cast<size_t>(P.Mrx) * P.Mry;
    const size_t csz = 2 * rb;
    const int tiles_x = (P.Mrx + kT3Tile - 1) / kT3Tile, tiles_y = (P.Mry + kT3Tile - 1) / kT3Tile;
    const long long ntiles = static_cast<long long>(tiles_x) * tiles_y;
    const long long max_items = ntiles + len_in / kT3Item + 1;
    if (len_in > 0x7fffffffLL || max_items > 0x7fffffffLL) return NFFT2D_ERR_UNSUPPORTED;
    // work buffers: grid, records (unsorted, sorted), tile/rank, counts, starts, item starts, items
    const size_t off_tmp = (cells * csz + 255) / 256 * 256;
    const size_t off_recs = off_tmp + (static_cast<size_t>(len_in) * sizeof(T3Rec) + 255) / 256 * 256;
    const size_t off_tr = off_recs + (static_cast<size_t>(len_in) * sizeof(T3Rec) + 255) / 256 * 256;
    const size_t off_cnt = off_tr + (static_cast<size_t>(len_in) * sizeof(int2) + 255) / 256 * 256;
    const size_t off_st = off_cnt + (static_cast<size_t>(ntiles + 1) * sizeof(unsigned) + 255) / 256 * 256;
    const size_t off_ist = off_st + (static_cast<size_t>(ntiles) * sizeof(unsigned) + 255) / 256 * 256;
    const size_t off_items = off_ist + (static_cast<size_t>(ntiles) * sizeof(unsigned) + 255) / 256 * 256;
    // pre-compensation tables over ds in [-off, off]: |ds| <= M/4 + ms + 1 for
    // points inside the extents, off = M/2 + ms + 2 leaves margin
    const int tabo_x = P.Mrx / 2 + P.ms + 2, tabo_y = P.Mry / 2 + P.ms + 2;
    const size_t off_tx = off_items + (static_cast<size_t>(max_items) * sizeof(int4) + 255) / 256 * 256;
    const size_t off_ty = off_tx + (static_cast<size_t>(2 * tabo_x + 1) * sizeof(float) + 255) / 256 * 256;
    const size_t total = off_ty + static_cast<size_t>(2 * tabo_y + 1) * sizeof(float);
    T3_CUDA(cudaMallocAsync(&S.grid, total, st));
    unsigned char *base = static_cast<unsigned char *>(S.grid);
    T3Rec *tmp = reinterpret_cast<T3Rec *>(base + off_tmp), *recs = reinterpret_cast<T3Rec *>(base + off_recs);
    int2 *tr = reinterpret_cast<int2 *>(base + off_tr);
    unsigned *counts = reinterpret_cast<unsigned *>(base + off_cnt), *starts = reinterpret_cast<unsigned *>(base + off_st);
    unsigned *istarts = reinterpret_cast<unsigned *>(base + off_ist);
    int4 *items = reinterpret_cast<int4 *>(base + off_items);
    float *prex = reinterpret_cast<float *>(base + off_tx), *prey = reinterpret_cast<float *>(base + off_ty);
    k_t3_table<<<(2 * tabo_x + 1 + 255) / 256, 256, 0, st>>>(prex, 2 * tabo_x + 1, tabo_x, P.b * P.Dx * P.Dx);
    k_t3_table<<<(2 * tabo_y + 1 + 255) / 256, 256, 0, st>>>(prey, 2 * tabo_y + 1, tabo_y, P.b * P.Dy * P.Dy);
    T3_CUDA(cudaGetLastError());
    T3_CUDA(cudaMemsetAsync(S.grid, 0, cells * csz, st));
    T3_CUDA(cudaMemsetAsync(counts, 0, static_cast<size_t>(ntiles + 1) * sizeof(unsigned), st));
    const unsigned pb = static_cast<unsigned>((len_in + 255) / 256);
    if (dbl)
        k_t3_prep<double2><<<pb, 256, 0, st>>>(x, y, static_cast<const double2 *>(f), len_in, P, tiles_x, tmp, tr,
                                              counts);
    else
        k_t3_prep<float2><<<pb, 256, 0, st>>>(x, y, static_cast<const float2 *>(f), len_in, P, tiles_x, tmp, tr,
                                             counts);
    T3_CUDA(cudaGetLastError());
    k_t3_scan<<<1, 1024, 0, st>>>(counts, static_cast<int>(ntiles), starts, istarts);
    T3_CUDA(cudaGetLastError());
    k_t3_scatter<<<pb, 256, 0, st>>>(tmp, tr, len_in, starts, recs);
    T3_CUDA(cudaGetLastError());
    k_t3_items<<<static_cast<unsigned>((ntiles + 255) / 256), 256, 0, st>>>(counts, starts, istarts,
                                                                           static_cast<int>(ntiles), items);
    T3_CUDA(cudaGetLastError());
    // one CTA per possible work item; those beyond the device-side count return
    if (dbl) {
        T3_CUDA(cudaFuncSetAttribute(k_t3_spread<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     static_cast<int>(smem)));
        k_t3_spread<double><<<static_cast<unsigned>(max_items), kT3Warps * 32, smem, st>>>(
            recs, items, counts + ntiles, P, tiles_x, B, prex, tabo_x, prey, tabo_y, static_cast<double *>(S.grid));
    } else {
        T3_CUDA(cudaFuncSetAttribute(k_t3_spread<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     static_cast<int>(smem)));
        k_t3_spread<float><<<static_cast<unsigned>(max_items), kT3Warps * 32, smem, st>>>(
            recs, items, counts + ntiles, P, tiles_x, B, prex, tabo_x, prey, tabo_y, static_cast<float *>(S.grid));
    }
    T3_CUDA(cudaGetLastError());
    // :283-292 -- rows are Mry, the fast (column) dimension Mrx
    if (nfft2d::pooled_plan_2d(&S.plan, P.Mry, P.Mrx, dbl ? CUFFT_Z2Z : CUFFT_C2C) != CUFFT_SUCCESS)
        return NFFT2D_ERR_CUFFT;
    S.plan_ok = true;
    if (cufftSetStream(S.plan, st) != CUFFT_SUCCESS) return NFFT2D_ERR_CUFFT;
    const cufftResult fr =
        dbl ? cufftExecZ2Z(S.plan, static_cast<cufftDoubleComplex *>(S.grid), static_cast<cufftDoubleComplex *>(S.grid),
                           CUFFT_FORWARD)
            : cufftExecC2C(S.plan, static_cast<cufftComplex *>(S.grid), static_cast<cufftComplex *>(S.grid),
                           CUFFT_FORWARD);
    if (fr != CUFFT_SUCCESS) return NFFT2D_ERR_CUFFT;
    const long long warps_out = (len_out + 31) / 32;  // 32 frequencies per warp
    const unsigned blk_out = static_cast<unsigned>((warps_out + kWarpsPerBlock - 1) / kWarpsPerBlock);
    if (dbl)
        k_t3_gather<double2, double><<<blk_out, kWarpsPerBlock * 32, 0, st>>>(
            s, t, len_out, P, static_cast<const double2 *>(S.grid), static_cast<double2 *>(F));
    else
        k_t3_gather<float2, float><<<blk_out, kWarpsPerBlock * 32, 0, st>>>(
            s, t, len_out, P, static_cast<const float2 *>(S.grid), static_cast<float2 *>(F));
    T3_CUDA(cudaGetLastError());
    return cuda_status(cudaStreamSynchronize(st));
}
