// nfft2d_knab.cu -- Knab-window band-limited regridding on the GPU, the SAR
// code's caller of the forward NFFT (BP_FBP_FFBP/knabNFFT2D.m:1-79 with
// NFFT_Based_Selvas_Approach_for_Signal_Interp_2D.m:4-28, KnabWindow.m:11-47,
// ConvWindow.m:5-11 and IntervalIntersection.m:4-22).
//
// A raster sampled on a rectilinear grid -- rows at cos_in[i] (spacing T2),
// columns at rho_in[j] (spacing T1) -- is interpolated to arbitrary output
// points as the band-limited trigonometric polynomial
//
//   out(p) = sum_{|k1| <= kgm, |k2| <= kgn} Gm[k1] Gn[k2] E[k1 mod Nrows][k2 mod Ncols]
//            exp(+2 pi i (k1 (c_p - cos_in[0]) / (Nrows T2) + k2 (r_p - rho_in[0]) / (Ncols T1)))
//
// where E is the raster's 2D DFT (sign -1) and Gm, Gn are Knab windows (1/N
// in the signal band, a prolate-like roll-off outside it).  The reference
// repeats and windows the spectrum, zero-pads it to (a Ncols) x (b Nrows) and
// evaluates it with conj(NFFT1_2D(conj(.))), a type-2 NFFT with sign +1 on
// that grid, at x = (r - rho_in[0]) / (T1 / a), (c - cos_in[0]) / (T2 / b);
// a and b are oversampling factors detected from the output points.
//
// Here the periodic repetition, the window, the zero padding and the NFFT's
// own deapodization are one kernel (k_knab_pad) that reads the raster
// spectrum and writes the oversampled grid directly; the plan's FFT, halo
// fill and gather follow.  The (N a)(M b) factor of Interp_2D.m:11 and the
// 1/(a b N M) of :28 cancel and are not applied.
//
// Axes: the internal plan's rows (N1 = b Nrows) pair with cos alpha and its
// columns (N2 = a Ncols) with rho, so k_knab_pad reads spectrum rows along
// consecutive addresses.  The reference's NFFT1_2D is fixed at c = 2, K = 6
// (NFFT1_2D.m:9-10); so is the plan here.
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "nfft2d_internal.h"

using namespace nfft2d;

namespace {

constexpr double kPi = 3.141592653589793238462643383279502884;
constexpr int kKnabP = 18;       // 2P+1 samples in the sampling series (knabNFFT2D.m:63)
constexpr double kSigma = 2.0;   // NFFT1_2D.m:9
constexpr int kKernelK = 6;      // NFFT1_2D.m:10
constexpr int kMinmaxBlocks = 256;

int cuda_status(cudaError_t e) {
    if (e == cudaSuccess) return NFFT2D_OK;
    return e == cudaErrorMemoryAllocation ? NFFT2D_ERR_OOM : NFFT2D_ERR_CUDA;
}

#define KNAB_TRY_CUDA(expr)                             \
    do {                                                \
        cudaError_t e_ = (expr);                        \
        if (e_ != cudaSuccess) return cuda_status(e_);  \
    } while (0)

// ---------------------------------------------------------------------------
// host FP64: the Knab window
// ---------------------------------------------------------------------------

// 16-point Gauss-Legendre nodes and weights on [-1, 1], by Newton's method on
// the Legendre recurrence (Golub & Welsch give the same nodes).
struct GaussLegendre16 {
    double x[16], w[16];
    GaussLegendre16() {
        const int n = 16;
        for (int i = 0; i < n; ++i) {
            double z = std::cos(kPi * (i + 0.75) / (n + 0.5));
            double dp = 1.0;
            for (int it = 0; it < 100; ++it) {
                double p0 = 1.0, p1 = z;
                for (int k = 2; k <= n; ++k) {
                    const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
                    p0 = p1;
                    p1 = p2;
                }
                dp = n * (z * p1 - p0) / (z * z - 1.0);
                const double dz = p1 / dp;
                z -= dz;
                if (std::fabs(dz) < 1e-16) break;
            }
            x[i] = z;
            w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
        }
    }
};

// ConvWindow(f, B1, TT) (ConvWindow.m:11) integrated over theta in [t0, t1]
// after f = (B1/2) sin(theta): the square-root edge of the window becomes the
// smooth integrand (B1/2) cos(theta) I0(beta cos(theta)) / D, beta = pi B1 TT / 2,
// D = B1 sinh(beta) / beta (B1 sinc(i B1 TT/2) in MATLAB's sinc).  Composite
// 16-point Gauss-Legendre on sub-panels of at most 0.05 rad.
double window_integral_theta(double t0, double t1, double B1, double TT, const GaussLegendre16 &gl) {
    if (!(t1 > t0)) return 0.0;
    const double beta = kPi * B1 * TT / 2.0;
    const double D = B1 * (beta == 0.0 ? 1.0 : std::sinh(beta) / beta);
    const int nsub = std::max(1, static_cast<int>(std::ceil((t1 - t0) / 0.05)));
    const double h = (t1 - t0) / nsub;
    double sum = 0.0;
    for (int s = 0; s < nsub; ++s) {
        const double a = t0 + s * h, mid = a + 0.5 * h;
        double ps = 0.0;
        for (int i = 0; i < 16; ++i) {
            const double th = mid + 0.5 * h * gl.x[i];
            const double ct = std::cos(th);
            ps += gl.w[i] * ct * bessel_i0_host(beta * ct);
        }
        sum += 0.5 * h * ps;
    }
    return sum * (B1 / 2.0) / D;
}

// KnabWindow.m:11-47.  Returns kg (G has 2 kg + 1 entries, frequencies
// -kg..kg), or -1 for parameters outside 0 < B < 1/T, T > 0, N >= 1.  The
// operation order of df, kg and f(k) follows :16-22, since kg is the floor of
// a quotient.  Transition entries: IntervalIntersection([-B1/2, B1/2],
// f + [-B0/2, B0/2]) is [-B1/2, f + B0/2] for every f <= 0 with f + B0/2 <
// B1/2 (because B0 >= B1), so G(k) is a cumulative integral of the window
// from its left edge, accumulated panel by panel in theta.
// Windows already computed in this process, by their exact parameters: an
// FFBP image builds two windows per regridding (~0.1-0.3 ms each, 4000
// Bessel evaluations), and every image of the same geometry asks for the
// same ones.  Up to 1024 windows are kept, the oldest replaced first.
struct WindowEntry {
    double T, B;
    int P;
    long N;
    long kg;
    std::vector<double> G;
};
std::mutex g_win_mu;
std::vector<WindowEntry> g_win_cache;
size_t g_win_next = 0;

long knab_window_compute(double T, double B, int P, long N, std::vector<double> *G);

long knab_window(double T, double B, int P, long N, std::vector<double> *G) {
    if (!G) return knab_window_compute(T, B, P, N, nullptr);
    {
        std::lock_guard<std::mutex> lock(g_win_mu);
        for (const auto &e : g_win_cache)
            if (e.T == T && e.B == B && e.P == P && e.N == N) {
                *G = e.G;
                return e.kg;
            }
    }
    const long kg = knab_window_compute(T, B, P, N, G);
    if (kg >= 0) {
        std::lock_guard<std::mutex> lock(g_win_mu);
        WindowEntry e{T, B, P, N, kg, *G};
        if (g_win_cache.size() < 1024) {
            g_win_cache.push_back(std::move(e));
        } else {
            g_win_cache[g_win_next] = std::move(e);
            g_win_next = (g_win_next + 1) % g_win_cache.size();
        }
    }
    return kg;
}

long knab_window_compute(double T, double B, int P, long N, std::vector<double> *G) {
    if (!(T > 0) || !(B > 0) || !(B < 1.0 / T) || N < 1 || P < 1 || !std::isfinite(T) || !std::isfinite(B))
        return -1;
    const double df = 1.0 / (static_cast<double>(N) * T);            // :16
    const long kg = static_cast<long>(std::floor((1.0 / T - B / 2.0) / df));  // :19
    if (kg < 0) return -1;
    if (!G) return kg;
    const double B0 = 1.0 / T;                                       // :24
    const double B1 = B0 - B;                                        // :25
    const double TT = 2.0 * P * T;                                   // :34
    const long n = 2 * kg + 1;
    std::vector<double> g(static_cast<size_t>(n), 0.0);              // :29
    long last = -1;
    for (long k = 0; k <= kg; ++k) {
        const double f = -df * static_cast<double>(kg) + df * static_cast<double>(k);  // :22
        if (B1 / 2.0 <= f + B0 / 2.0)                                // :26
            g[k] = 1.0;                                              // :32
        else
            last = k;
    }
    static const GaussLegendre16 gl;
    double acc = 0.0, th_prev = -kPi / 2.0;
    for (long k = 0; k <= last; ++k) {                               // :36
        const double f = -df * static_cast<double>(kg) + df * static_cast<double>(k);
        const double hi = f + B0 / 2.0;
        if (hi < -B1 / 2.0) continue;                                // no overlap (IntervalIntersection.m:6)
        const double th = std::asin(std::max(-1.0, std::min(1.0, 2.0 * hi / B1)));
        acc += window_integral_theta(th_prev, th, B1, TT, gl);       // :40
        th_prev = th;
        g[k] = acc;
    }
    G->assign(static_cast<size_t>(n), 0.0);
    for (long i = 0; i < n; ++i) (*G)[i] = g[i] + g[n - 1 - i];      // :45
    (*G)[kg] -= 1.0;                                                 // :46
    for (long i = 0; i < n; ++i) (*G)[i] /= static_cast<double>(N);  // :47
    return kg;
}

// mean(diff(v)) (knabNFFT2D.m:6-7), summed in index order.
double mean_diff(const double *v, int n) {
    double s = 0.0;
    for (int i = 0; i + 1 < n; ++i) s += v[i + 1] - v[i];
    return s / static_cast<double>(n - 1);
}

// ---------------------------------------------------------------------------
// device kernels
// ---------------------------------------------------------------------------

// Windowed, periodically repeated, deapodized raster spectrum on the
// oversampled grid interior.  One grid row r per blockIdx.y: FFT index r
// holds frequency k1 = r (r < n1/2) or r - n1 (the ifftshift of
// NFFT1_2D.m:55 on the centered block of Interp_2D.m:14-25); coefficients
// with |k1| > kgm or |k2| > kgn are the zero padding.
template <typename Cx, typename Rl>
__global__ void k_knab_pad(const Cx *__restrict__ spec, int Nrows, int Ncols, const Rl *__restrict__ wrow, int kgm,
                           const Rl *__restrict__ wcol, int kgn, Cx *__restrict__ grid, int n1, int n2, int H,
                           int C) {
    const int r = blockIdx.y;
    const int k1 = (r < n1 / 2) ? r : r - n1;
    const bool row_in = k1 >= -kgm && k1 <= kgm;
    const Rl s1 = row_in ? wrow[k1 + kgm] : Rl(0);
    int i = k1 % Nrows;
    if (i < 0) i += Nrows;
    const Cx *src = spec + static_cast<size_t>(i) * Ncols;
    Cx *dst = grid + static_cast<size_t>(r + H) * C + H;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n2; c += gridDim.x * blockDim.x) {
        const int k2 = (c < n2 / 2) ? c : c - n2;
        Cx v;
        v.x = Rl(0);
        v.y = Rl(0);
        if (row_in && k2 >= -kgn && k2 <= kgn) {
            int j = k2 % Ncols;
            if (j < 0) j += Ncols;
            const Rl s = s1 * wcol[k2 + kgn];
            const Cx e = src[j];
            v.x = e.x * s;
            v.y = e.y * s;
        }
        dst[c] = v;
    }
}

// Per-block min / max of two coordinate arrays: partial[4 b + {0, 1, 2, 3}] =
// min x1, max x1, min x2, max x2.  A NaN or infinite coordinate sets
// *nonfinite and is left out of the extent.
template <typename CT>
__global__ void k_knab_minmax(const CT *__restrict__ x1, const CT *__restrict__ x2, long long M,
                              double *__restrict__ partial, int *__restrict__ nonfinite) {
    double v[4] = {INFINITY, -INFINITY, INFINITY, -INFINITY};
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < M;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const double a = static_cast<double>(x1[i]), b = static_cast<double>(x2[i]);
        if (!isfinite(a) || !isfinite(b)) {
            *nonfinite = 1;
            continue;
        }
        v[0] = fmin(v[0], a);
        v[1] = fmax(v[1], a);
        v[2] = fmin(v[2], b);
        v[3] = fmax(v[3], b);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v[0] = fmin(v[0], __shfl_xor_sync(0xffffffffu, v[0], o));
        v[1] = fmax(v[1], __shfl_xor_sync(0xffffffffu, v[1], o));
        v[2] = fmin(v[2], __shfl_xor_sync(0xffffffffu, v[2], o));
        v[3] = fmax(v[3], __shfl_xor_sync(0xffffffffu, v[3], o));
    }
    __shared__ double sm[32][4];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    if (lane == 0)
        for (int q = 0; q < 4; ++q) sm[warp][q] = v[q];
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < nw; ++w) {
            v[0] = fmin(v[0], sm[w][0]);
            v[1] = fmax(v[1], sm[w][1]);
            v[2] = fmin(v[2], sm[w][2]);
            v[3] = fmax(v[3], sm[w][3]);
        }
        for (int q = 0; q < 4; ++q) partial[4 * blockIdx.x + q] = v[q];
    }
}

// Extrapolation masks (knabNFFT2D.m:75-76): column j is outside when
// rho_out[0][j] lies outside the input range, row i when cos_out[i][0] does.
template <typename CT>
__global__ void k_knab_masks(const CT *__restrict__ rho_out, const CT *__restrict__ cos_out, int len1, int len2,
                             double rmin, double rmax, double cmin, double cmax, unsigned char *__restrict__ row_mask,
                             unsigned char *__restrict__ col_mask, int *__restrict__ count) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < len1 + len2; t += gridDim.x * blockDim.x) {
        bool m;
        if (t < len2) {
            const double v = static_cast<double>(rho_out[t]);
            m = v < rmin || v > rmax;
            col_mask[t] = m ? 1 : 0;
        } else {
            const int i = t - len2;
            const double v = static_cast<double>(cos_out[static_cast<size_t>(i) * len2]);
            m = v < cmin || v > cmax;
            row_mask[i] = m ? 1 : 0;
        }
        if (m) atomicAdd(count, 1);
    }
}

// result(:, xout) = result(yout, :) = ExtrapVal (knabNFFT2D.m:77-78).
template <typename Cx, typename Rl>
__global__ void k_knab_extrap(Cx *__restrict__ out, const unsigned char *__restrict__ row_mask,
                              const unsigned char *__restrict__ col_mask, int len1, int len2, Rl ev_re, Rl ev_im) {
    const long long n = static_cast<long long>(len1) * len2;
    for (long long q = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; q < n;
         q += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int i = static_cast<int>(q / len2), j = static_cast<int>(q - static_cast<long long>(i) * len2);
        if (row_mask[i] | col_mask[j]) {
            Cx v;
            v.x = ev_re;
            v.y = ev_im;
            out[q] = v;
        }
    }
}

}  // namespace

struct nfft2d_knab_s {
    int Nrows = 0, Ncols = 0, precision = NFFT2D_F32;
    double T1 = 0, T2 = 0, B1 = 0, B2 = 0;
    double rho0 = 0, cos0 = 0;                   // rho_in[0], cos_in[0] (knabNFFT2D.m:23-24)
    double rmin = 0, rmax = 0, cmin = 0, cmax = 0;  // input axis ranges (:75-76)
    long kgn = 0, kgm = 0;                       // window half-lengths along rho, cos alpha
    std::vector<double> Gn, Gm;                  // Knab windows (FP64, host)
    cudaStream_t stream = nullptr;
    int num_sms = 1;
    cufftHandle raster_fft = 0;
    bool fft_ok = false;
    void *spec = nullptr;                        // Nrows x Ncols raster spectrum
    double *d_partial = nullptr;                 // min / max partials
    int *d_count = nullptr;                      // [0] masked rows + columns, [1] non-finite seen
    // bound by set_points
    nfft2d_plan_s *plan = nullptr;               // (b Nrows) x (a Ncols), sigma 2, K 6
    int a = 0, b = 0;
    void *wrow = nullptr, *wcol = nullptr;       // Gm * deap1, Gn * deap2 in the plan precision
    size_t wrow_cap = 0, wcol_cap = 0;
    unsigned char *row_mask = nullptr, *col_mask = nullptr;
    int row_cap = 0, col_cap = 0;
    int len1 = 0, len2 = 0;
    int n_masked = 0;
    bool points_valid = false;
};

namespace {

void knab_free(nfft2d_knab_s *k) {
    if (!k) return;
    // nothing of the regridder in flight: its FFT handle and buffers go back
    // to the library's caches
    cudaStreamSynchronize(k->stream);
    if (k->plan) release_plan(k->plan);
    if (k->fft_ok) pooled_plan_release(k->raster_fft);
    plan_free(k->spec);
    plan_free(k->d_partial);
    plan_free(k->d_count);
    plan_free(k->wrow);
    plan_free(k->wcol);
    plan_free(k->row_mask);
    plan_free(k->col_mask);
    delete k;
}

size_t real_bytes(int precision) { return precision == NFFT2D_F64 ? sizeof(double) : sizeof(float); }
size_t cplx_bytes(int precision) { return 2 * real_bytes(precision); }

// A device buffer of at least `need` bytes; a smaller one goes back to the
// cache once the stream's work on it is done.
int ensure_bytes(void **ptr, size_t *cap, size_t need, cudaStream_t st) {
    if (*cap >= need && *ptr) return NFFT2D_OK;
    if (*ptr) {
        cudaStreamSynchronize(st);
        plan_free(*ptr);
    }
    *ptr = nullptr;
    *cap = 0;
    KNAB_TRY_CUDA(plan_malloc(ptr, need));
    *cap = need;
    return NFFT2D_OK;
}

cudaError_t launch_knab_pad(const nfft2d_plan_s *p, const void *ctx) {
    const nfft2d_knab_s *k = static_cast<const nfft2d_knab_s *>(ctx);
    const Geom &g = p->g;
    const dim3 grid(std::max(1, std::min((g.n2 + 255) / 256, 64)), g.n1, 1);
    if (k->precision == NFFT2D_F64)
        k_knab_pad<double2, double><<<grid, 256, 0, p->stream>>>(
            static_cast<const double2 *>(k->spec), k->Nrows, k->Ncols, static_cast<const double *>(k->wrow),
            static_cast<int>(k->kgm), static_cast<const double *>(k->wcol), static_cast<int>(k->kgn),
            static_cast<double2 *>(p->grid), g.n1, g.n2, g.H, g.C);
    else
        k_knab_pad<float2, float><<<grid, 256, 0, p->stream>>>(
            static_cast<const float2 *>(k->spec), k->Nrows, k->Ncols, static_cast<const float *>(k->wrow),
            static_cast<int>(k->kgm), static_cast<const float *>(k->wcol), static_cast<int>(k->kgn),
            static_cast<float2 *>(p->grid), g.n1, g.n2, g.H, g.C);
    return cudaGetLastError();
}

// Upload Gm * deap1 and Gn * deap2 for the current plan.
int upload_weights(nfft2d_knab_s *k) {
    const nfft2d_plan_s *p = k->plan;
    const int N1 = p->N1, N2 = p->N2;
    std::vector<double> d1(N1), d2(N2);
    deapod_table_host(N1, p->g.n1, p->K, p->w.alpha, d1.data());
    deapod_table_host(N2, p->g.n2, p->K, p->w.alpha, d2.data());
    const long nr = 2 * k->kgm + 1, nc = 2 * k->kgn + 1;
    std::vector<double> wr(nr), wc(nc);
    for (long j = 0; j < nr; ++j) wr[j] = k->Gm[j] * d1[(j - k->kgm) + N1 / 2];
    for (long j = 0; j < nc; ++j) wc[j] = k->Gn[j] * d2[(j - k->kgn) + N2 / 2];
    const size_t rb = real_bytes(k->precision);
    int st = ensure_bytes(&k->wrow, &k->wrow_cap, rb * nr, k->stream);
    if (st != NFFT2D_OK) return st;
    if ((st = ensure_bytes(&k->wcol, &k->wcol_cap, rb * nc, k->stream)) != NFFT2D_OK) return st;
    if (k->precision == NFFT2D_F64) {
        KNAB_TRY_CUDA(cudaMemcpy(k->wrow, wr.data(), rb * nr, cudaMemcpyHostToDevice));
        KNAB_TRY_CUDA(cudaMemcpy(k->wcol, wc.data(), rb * nc, cudaMemcpyHostToDevice));
    } else {
        std::vector<float> fr(wr.begin(), wr.end()), fc(wc.begin(), wc.end());
        KNAB_TRY_CUDA(cudaMemcpy(k->wrow, fr.data(), rb * nr, cudaMemcpyHostToDevice));
        KNAB_TRY_CUDA(cudaMemcpy(k->wcol, fc.data(), rb * nc, cudaMemcpyHostToDevice));
    }
    return NFFT2D_OK;
}

template <typename CT>
int minmax_and_masks(nfft2d_knab_s *k, long long M, const CT *rho_out, const CT *cos_out, double mm[4]) {
    int blocks = std::max(1, std::min(kMinmaxBlocks, static_cast<int>((M + 255) / 256)));
    KNAB_TRY_CUDA(cudaMemsetAsync(k->d_count, 0, 2 * sizeof(int), k->stream));
    k_knab_minmax<CT><<<blocks, 256, 0, k->stream>>>(rho_out, cos_out, M, k->d_partial, k->d_count + 1);
    KNAB_TRY_CUDA(cudaGetLastError());
    const int nm = k->len1 + k->len2;
    k_knab_masks<CT><<<std::max(1, std::min(4 * k->num_sms, (nm + 255) / 256)), 256, 0, k->stream>>>(
        rho_out, cos_out, k->len1, k->len2, k->rmin, k->rmax, k->cmin, k->cmax, k->row_mask, k->col_mask,
        k->d_count);
    KNAB_TRY_CUDA(cudaGetLastError());
    std::vector<double> part(4 * static_cast<size_t>(blocks));
    KNAB_TRY_CUDA(cudaMemcpyAsync(part.data(), k->d_partial, sizeof(double) * part.size(), cudaMemcpyDeviceToHost,
                                  k->stream));
    int counts[2] = {0, 0};
    KNAB_TRY_CUDA(cudaMemcpyAsync(counts, k->d_count, 2 * sizeof(int), cudaMemcpyDeviceToHost, k->stream));
    KNAB_TRY_CUDA(cudaStreamSynchronize(k->stream));
    k->n_masked = counts[0];
    if (counts[1]) return NFFT2D_ERR_NONFINITE;
    mm[0] = INFINITY;
    mm[1] = -INFINITY;
    mm[2] = INFINITY;
    mm[3] = -INFINITY;
    for (int bl = 0; bl < blocks; ++bl) {
        mm[0] = std::fmin(mm[0], part[4 * bl + 0]);
        mm[1] = std::fmax(mm[1], part[4 * bl + 1]);
        mm[2] = std::fmin(mm[2], part[4 * bl + 2]);
        mm[3] = std::fmax(mm[3], part[4 * bl + 3]);
    }
    return NFFT2D_OK;
}

}  // namespace

extern "C" {

int nfft2d_knab_window(double T, double B, int P, int N, double *G, int G_len, int *kg) {
    if (!kg) return NFFT2D_ERR_INVALID_ARG;
    const long k = knab_window(T, B, P, N, nullptr);
    if (k < 0) return NFFT2D_ERR_INVALID_ARG;
    *kg = static_cast<int>(k);
    if (!G) return NFFT2D_OK;
    if (G_len < 2 * k + 1) return NFFT2D_ERR_INVALID_ARG;
    std::vector<double> w;
    knab_window(T, B, P, N, &w);
    std::memcpy(G, w.data(), sizeof(double) * w.size());
    return NFFT2D_OK;
}

int nfft2d_knab_create(nfft2d_knab *out, int Nrows, int Ncols, const double *rho_in, const double *cos_in, double B1,
                       double B2, int precision, void *stream) {
    if (!out) return NFFT2D_ERR_INVALID_ARG;
    *out = nullptr;
    if (Nrows < 2 || Ncols < 2 || !rho_in || !cos_in) return NFFT2D_ERR_INVALID_ARG;  // knabNFFT2D.m:15-20
    if (precision != NFFT2D_F32 && precision != NFFT2D_F64) return NFFT2D_ERR_INVALID_ARG;
    for (int j = 0; j < Ncols; ++j)
        if (!std::isfinite(rho_in[j])) return NFFT2D_ERR_NONFINITE;
    for (int i = 0; i < Nrows; ++i)
        if (!std::isfinite(cos_in[i])) return NFFT2D_ERR_NONFINITE;
    nfft2d_knab_s *k = new (std::nothrow) nfft2d_knab_s();
    if (!k) return NFFT2D_ERR_OOM;
    auto fail = [&](int s) {
        knab_free(k);
        return s;
    };
    k->Nrows = Nrows;
    k->Ncols = Ncols;
    k->precision = precision;
    k->stream = static_cast<cudaStream_t>(stream);
    k->B1 = B1;
    k->B2 = B2;
    k->T1 = mean_diff(rho_in, Ncols);  // :6
    k->T2 = mean_diff(cos_in, Nrows);  // :7
    k->rho0 = rho_in[0];
    k->cos0 = cos_in[0];
    k->rmin = *std::min_element(rho_in, rho_in + Ncols);
    k->rmax = *std::max_element(rho_in, rho_in + Ncols);
    k->cmin = *std::min_element(cos_in, cos_in + Nrows);
    k->cmax = *std::max_element(cos_in, cos_in + Nrows);
    // windows: Gn along rho with N = Ncols, Gm along cos alpha with N = Nrows (:64-65)
    k->kgn = knab_window(k->T1, B1, kKnabP, Ncols, &k->Gn);
    k->kgm = knab_window(k->T2, B2, kKnabP, Nrows, &k->Gm);
    if (k->kgn < 0 || k->kgm < 0) return fail(NFFT2D_ERR_INVALID_ARG);
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return fail(NFFT2D_ERR_CUDA);
    if (cudaDeviceGetAttribute(&k->num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return fail(NFFT2D_ERR_CUDA);
    const cufftType t = precision == NFFT2D_F64 ? CUFFT_Z2Z : CUFFT_C2C;
    if (pooled_plan_2d(&k->raster_fft, Nrows, Ncols, t) != CUFFT_SUCCESS) return fail(NFFT2D_ERR_CUFFT);
    k->fft_ok = true;
    if (cufftSetStream(k->raster_fft, k->stream) != CUFFT_SUCCESS) return fail(NFFT2D_ERR_CUFFT);
    if (plan_malloc(&k->spec, cplx_bytes(precision) * static_cast<size_t>(Nrows) * Ncols) != cudaSuccess)
        return fail(NFFT2D_ERR_OOM);
    if (plan_malloc(reinterpret_cast<void **>(&k->d_partial), sizeof(double) * 4 * kMinmaxBlocks) != cudaSuccess)
        return fail(NFFT2D_ERR_OOM);
    if (plan_malloc(reinterpret_cast<void **>(&k->d_count), 2 * sizeof(int)) != cudaSuccess) return fail(NFFT2D_ERR_OOM);
    *out = k;
    return NFFT2D_OK;
}

int nfft2d_knab_destroy(nfft2d_knab k) {
    if (!k) return NFFT2D_ERR_INVALID_ARG;
    cudaStreamSynchronize(k->stream);
    knab_free(k);
    return NFFT2D_OK;
}

int nfft2d_knab_set_points(nfft2d_knab k, int len1, int len2, const void *rho_out, const void *cos_out,
                           int coord_dtype) {
    if (!k) return NFFT2D_ERR_INVALID_ARG;
    k->points_valid = false;
    if (len1 < 1 || len2 < 1 || !rho_out || !cos_out) return NFFT2D_ERR_INVALID_ARG;
    if (coord_dtype != NFFT2D_COORD_F32 && coord_dtype != NFFT2D_COORD_F64) return NFFT2D_ERR_INVALID_ARG;
    const long long M = static_cast<long long>(len1) * len2;
    if (M > 0x7fffffffLL) return NFFT2D_ERR_INVALID_ARG;
    k->len1 = len1;
    k->len2 = len2;
    int st;
    {
        void *p = k->row_mask;
        size_t cap = static_cast<size_t>(k->row_cap);
        if ((st = ensure_bytes(&p, &cap, static_cast<size_t>(len1), k->stream)) != NFFT2D_OK) return st;
        k->row_mask = static_cast<unsigned char *>(p);
        k->row_cap = static_cast<int>(cap);
        p = k->col_mask;
        cap = static_cast<size_t>(k->col_cap);
        if ((st = ensure_bytes(&p, &cap, static_cast<size_t>(len2), k->stream)) != NFFT2D_OK) return st;
        k->col_mask = static_cast<unsigned char *>(p);
        k->col_cap = static_cast<int>(cap);
    }
    // extent of the shifted output points (:23-35) and the extrapolation masks
    double mm[4];
    st = coord_dtype == NFFT2D_COORD_F64
             ? minmax_and_masks(k, M, static_cast<const double *>(rho_out), static_cast<const double *>(cos_out), mm)
             : minmax_and_masks(k, M, static_cast<const float *>(rho_out), static_cast<const float *>(cos_out), mm);
    if (st != NFFT2D_OK) return st;
    if (!std::isfinite(mm[0]) || !std::isfinite(mm[1]) || !std::isfinite(mm[2]) || !std::isfinite(mm[3]))
        return NFFT2D_ERR_NONFINITE;
    // rounding is monotone, so min(x - o) = fl(min(x) - o)
    const double mnr = mm[0] - k->rho0, mxr = mm[1] - k->rho0;
    const double mnc = mm[2] - k->cos0, mxc = mm[3] - k->cos0;
    double Nn = (mxr - mnr) / (k->T1 * (1.0 - 1.0 / len2));  // :34
    double Mm = (mxc - mnc) / (k->T2 * (1.0 - 1.0 / len1));  // :35
    if (Nn < 1 || std::isnan(Nn)) Nn = 1;                    // :37-42
    if (Mm < 1 || std::isnan(Mm)) Mm = 1;
    double ad = std::round(len2 / Nn), bd = std::round(len1 / Mm);  // :45-46 (MATLAB round: half away from 0)
    if (ad < 2) ad = 2;  // :48-60; the zero points appended there are cropped away at :72
    if (bd < 2) bd = 2;
    if (ad * k->Ncols > 23000.0 || bd * k->Nrows > 23000.0) return NFFT2D_ERR_UNSUPPORTED;
    const int a = static_cast<int>(ad), b = static_cast<int>(bd);
    const int N1 = b * k->Nrows, N2 = a * k->Ncols;
    // the reference's NFFT1_2D needs even sizes, and its zero padding
    // (Interp_2D.m:15,22) needs the windowed spectrum to fit the grid
    if ((N1 & 1) || (N2 & 1) || k->kgm > N1 / 2 - 1 || k->kgn > N2 / 2 - 1) return NFFT2D_ERR_INVALID_ARG;
    if (!k->plan || k->plan->N1 != N1 || k->plan->N2 != N2) {
        if (k->plan) {
            release_plan(k->plan);
            k->plan = nullptr;
        }
        // the regridder only gathers: row-major cell order (fewer distinct rows per warp)
        if ((st = create_plan(&k->plan, N1, N2, kSigma, kKernelK, k->precision, 0, k->stream, nullptr, false)) !=
            NFFT2D_OK)
            return st;
    }
    k->a = a;
    k->b = b;
    if ((st = upload_weights(k)) != NFFT2D_OK) return st;
    // grid-unit coordinates x1 = (c - cos_in[0]) b / T2, x2 = (r - rho_in[0]) a / T1 (Interp_2D.m:28)
    // the binning is enqueued (the extents above were the host round trip);
    // nfft2d_knab_synchronize reports its errors
    st = set_points_scaled(k->plan, M, cos_out, rho_out, coord_dtype, b / k->T2, a / k->T1, k->cos0, k->rho0, true);
    if (st != NFFT2D_OK) return st;
    k->points_valid = true;
    return NFFT2D_OK;
}

int nfft2d_knab_execute(nfft2d_knab k, double extrap_re, double extrap_im, const void *data, void *out) {
    if (!k || !data || !out) return NFFT2D_ERR_INVALID_ARG;
    if (!k->points_valid) return NFFT2D_ERR_NO_POINTS;
    cufftResult r;
    if (k->precision == NFFT2D_F64)
        r = cufftExecZ2Z(k->raster_fft, static_cast<cufftDoubleComplex *>(const_cast<void *>(data)),
                         static_cast<cufftDoubleComplex *>(k->spec), CUFFT_FORWARD);
    else
        r = cufftExecC2C(k->raster_fft, static_cast<cufftComplex *>(const_cast<void *>(data)),
                         static_cast<cufftComplex *>(k->spec), CUFFT_FORWARD);
    if (r != CUFFT_SUCCESS) return NFFT2D_ERR_CUFFT;
    int st = type2_with_pad(k->plan, +1, out, launch_knab_pad, k);
    if (st != NFFT2D_OK) return st;
    if (k->n_masked > 0) {
        const long long n = static_cast<long long>(k->len1) * k->len2;
        const int blocks = static_cast<int>(std::min<long long>((n + 255) / 256, 8LL * k->num_sms));
        if (k->precision == NFFT2D_F64)
            k_knab_extrap<double2, double><<<blocks, 256, 0, k->stream>>>(
                static_cast<double2 *>(out), k->row_mask, k->col_mask, k->len1, k->len2, extrap_re, extrap_im);
        else
            k_knab_extrap<float2, float><<<blocks, 256, 0, k->stream>>>(
                static_cast<float2 *>(out), k->row_mask, k->col_mask, k->len1, k->len2,
                static_cast<float>(extrap_re), static_cast<float>(extrap_im));
        KNAB_TRY_CUDA(cudaGetLastError());
    }
    return NFFT2D_OK;
}

int nfft2d_knab_get_info(nfft2d_knab k, nfft2d_knab_info *info) {
    if (!k || !info) return NFFT2D_ERR_INVALID_ARG;
    std::memset(info, 0, sizeof(*info));
    info->Nrows = k->Nrows;
    info->Ncols = k->Ncols;
    info->kgn = static_cast<int>(k->kgn);
    info->kgm = static_cast<int>(k->kgm);
    info->T1 = k->T1;
    info->T2 = k->T2;
    if (k->points_valid) {
        info->a = k->a;
        info->b = k->b;
        info->N1 = k->plan->N1;
        info->N2 = k->plan->N2;
        info->len1 = k->len1;
        info->len2 = k->len2;
        info->masked_lines = k->n_masked;
    }
    return NFFT2D_OK;
}

nfft2d_plan nfft2d_knab_plan(nfft2d_knab k) { return (k && k->points_valid) ? k->plan : nullptr; }

int nfft2d_knab_synchronize(nfft2d_knab k) {
    if (!k) return NFFT2D_ERR_INVALID_ARG;
    if (k->plan) return nfft2d_synchronize(k->plan);
    return cuda_status(cudaStreamSynchronize(k->stream));
}

int nfft2d_knab_nfft2d(double extrap_re, double extrap_im, const double *rho_in, int Ncols, const double *cos_in,
                       int Nrows, const void *data, const double *rho_out, const double *cos_out, int len1, int len2,
                       double B1, double B2, int precision, void *out, void *stream) {
    nfft2d_knab k = nullptr;
    int st = nfft2d_knab_create(&k, Nrows, Ncols, rho_in, cos_in, B1, B2, precision, stream);
    if (st != NFFT2D_OK) return st;
    st = nfft2d_knab_set_points(k, len1, len2, rho_out, cos_out, NFFT2D_COORD_F64);
    if (st == NFFT2D_OK) st = nfft2d_knab_execute(k, extrap_re, extrap_im, data, out);
    if (st == NFFT2D_OK) st = nfft2d_knab_synchronize(k);
    nfft2d_knab_destroy(k);
    return st;
}

}  // extern "C"
