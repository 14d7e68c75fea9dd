// nfft2d_ffbp.cu -- fast factorized back-projection (FFBP) over a straight
// track, the NFFT-interpolated branch of the reference's SAR code:
//   BP_FBP_FFBP/FFBP_POLAR_NFFT.m:1-158 (the recursion, its knabNFFT2D
//     regridding of each sub-aperture's polar raster onto the parent's
//     points, :24-71, :81-89, :96-123, :133-152),
//   BP_FBP_FFBP/BP_POLAR_NFFT.m:1-25 (the leaf back-projection of at most
//     three pulses, each through a 1D type-2 NFFT, NFFT1_1D.m).
//
// The host side (this file) walks the recursion; the device work is the
// library's: the Knab regridder (nfft2d_knab_*, its own FFTs, pad and NFFT
// gather) and one 2D plan for the leaves' 1D transforms (the pulse's nf
// samples in the k2 = 0 column of an nf x 8 coefficient grid, every point at
// x2 = 0: the 2D type-2 sum then equals the 1D one), plus the per-pixel
// kernels below (polar shift with its extents, phase ramps, leaf ranges).
//
// Each level's raster sizes and axes come from floor() of extents and from
// mean sample spacings that fix the Knab windows' lengths (a floor that sits
// on an exact tie when B T = 1/2, as here), so the coordinates are computed
// with unfused IEEE operations (__dmul_rn etc.) and cos(atan2(y, x)) as
// x / sqrt(x^2 + y^2): the same value within an ulp or two, and exactly what
// an IEEE restatement on the host computes.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "nfft2d_internal.h"

namespace {

constexpr double kPi = 3.141592653589793238462643383279502884;
constexpr int kLeafN2 = 8;  // columns of the leaves' coefficient grid (sigma*8 >= 2K+2 at K = 6)

// Order-preserving map of doubles onto unsigned 64-bit keys (atomic min/max).
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

// FFBP_POLAR_NFFT.m:39,44-46 (96-98): the parent's points in the polar frame of
// an antenna `dist` further along the track, and the extents (:49-52):
//   x = rho cos - dist, y = rho sqrt(1 - cos^2), rho' = sqrt(x^2 + y^2),
//   cos' = x / rho'  (cos(atan2(y, x)); 1 at the origin, as atan2(0, 0) = 0).
// mm[0..3] = keys of min rho', max rho', min cos', max cos'.
__global__ void k_polar_shift(const double *__restrict__ rho, const double *__restrict__ cs, long long n, double dist,
                              double *__restrict__ rho_o, double *__restrict__ cos_o, unsigned long long *mm) {
    double rmin = INFINITY, rmax = -INFINITY, cmin = INFINITY, cmax = -INFINITY;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const double r = rho[i], c = cs[i];
        const double s = __dsqrt_rn(__dsub_rn(1.0, __dmul_rn(c, c)));
        const double x = __dsub_rn(__dmul_rn(r, c), dist);
        const double y = __dmul_rn(r, s);
        const double rr = __dsqrt_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)));
        const double cc = rr > 0.0 ? __ddiv_rn(x, rr) : 1.0;
        rho_o[i] = rr;
        cos_o[i] = cc;
        rmin = fmin(rmin, rr);
        rmax = fmax(rmax, rr);
        cmin = fmin(cmin, cc);
        cmax = fmax(cmax, cc);
    }
    for (int o = 16; o > 0; o >>= 1) {
        rmin = fmin(rmin, __shfl_xor_sync(0xffffffffu, rmin, o));
        rmax = fmax(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
        cmin = fmin(cmin, __shfl_xor_sync(0xffffffffu, cmin, o));
        cmax = fmax(cmax, __shfl_xor_sync(0xffffffffu, cmax, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(mm + 0, ord_key(rmin));
        atomicMax(mm + 1, ord_key(rmax));
        atomicMin(mm + 2, ord_key(cmin));
        atomicMax(mm + 3, ord_key(cmax));
    }
}

// [RHO, COS] = meshgrid(rho_axis, cos_axis): rows follow cos, columns rho
// (FFBP_POLAR_NFFT.m:66, :118).
__global__ void k_meshgrid(const double *__restrict__ rax, const double *__restrict__ cax, int rows, int cols,
                           double *__restrict__ R, double *__restrict__ Cg) {
    const long long n = static_cast<long long>(rows) * cols;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int r = static_cast<int>(i / cols), c = static_cast<int>(i - static_cast<long long>(r) * cols);
        R[i] = rax[c];
        Cg[i] = cax[r];
    }
}

// phase = ((4 pi / c) rho) fc, the order of FFBP_POLAR_NFFT.m:73 and :89.
__device__ __forceinline__ double ramp(double rho, double k4c, double fc) { return __dmul_rn(__dmul_rn(k4c, rho), fc); }

template <typename C2>
__device__ __forceinline__ C2 cmul_phase(C2 v, double ph, double sgn) {
    double s, c;
    sincos(ph, &s, &c);
    s *= sgn;
    const double vx = static_cast<double>(v.x), vy = static_cast<double>(v.y);
    C2 o;
    o.x = static_cast<decltype(v.x)>(vx * c - vy * s);
    o.y = static_cast<decltype(v.x)>(vx * s + vy * c);
    return o;
}

// data .*= exp(-1j (4 pi / c RHO) fc)   (FFBP_POLAR_NFFT.m:73-79, 125-131)
template <typename C2>
__global__ void k_phase_mul(C2 *__restrict__ data, const double *__restrict__ rho, long long n, double k4c, double fc,
                            double sgn) {
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x)
        data[i] = cmul_phase(data[i], ramp(rho[i], k4c, fc), sgn);
}

// out (=|+=) rec .* exp(1j (4 pi / c RHO') fc)   (:89, :141, summed at :152)
template <typename C2>
__global__ void k_phase_acc(const C2 *__restrict__ rec, const double *__restrict__ rho, long long n, double k4c,
                            double fc, C2 *__restrict__ out, int first) {
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const C2 v = cmul_phase(rec[i], ramp(rho[i], k4c, fc), 1.0);
        if (first) {
            out[i] = v;
        } else {
            C2 o = out[i];
            o.x += v.x;
            o.y += v.y;
            out[i] = o;
        }
    }
}

// BP_POLAR_NFFT.m:14-15,19: delta_r = sqrt(pho^2 + xsi^2 - 2 pho xsi cos) - R0(n)
// and the NFFT1_1D abscissa x = (-2 BW / c) delta_r.
__global__ void k_leaf_prep(const double *__restrict__ pho, const double *__restrict__ cs, long long n, double xsi,
                            double xsi2, double r0, double scale, double *__restrict__ x1, double *__restrict__ dr) {
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const double p = pho[i];
        const double t = __dadd_rn(__dmul_rn(p, p), xsi2);
        const double u = __dmul_rn(__dmul_rn(__dmul_rn(2.0, p), xsi), cs[i]);
        const double d = __dsub_rn(__dsqrt_rn(__dsub_rn(t, u)), r0);
        dr[i] = d;
        x1[i] = __dmul_rn(scale, d);
    }
}

// The pulse's nf samples in column k2 = 0 (index kLeafN2 / 2) of an nf x 8 grid.
template <typename C2>
__global__ void k_leaf_embed(const C2 *__restrict__ ph, int nf, C2 *__restrict__ F) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nf * kLeafN2) return;
    const int k = i / kLeafN2, j = i - k * kLeafN2;
    C2 v;
    v.x = 0;
    v.y = 0;
    if (j == kLeafN2 / 2) v = ph[k];
    F[i] = v;
}

// im (=|+=) exp(1j 4 pi fc delta_r / c) .* f   (BP_POLAR_NFFT.m:17,19)
template <typename C2>
__global__ void k_leaf_acc(const C2 *__restrict__ f, const double *__restrict__ dr, long long n, double k4fc, double c,
                           C2 *__restrict__ im, int first) {
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const C2 v = cmul_phase(f[i], __ddiv_rn(__dmul_rn(k4fc, dr[i]), c), 1.0);
        if (first) {
            im[i] = v;
        } else {
            C2 o = im[i];
            o.x += v.x;
            o.y += v.y;
            im[i] = o;
        }
    }
}

int launch_blocks(long long n) { return static_cast<int>(std::max<long long>(1, std::min<long long>((n + 255) / 256, 4096))); }

int cuda_status(cudaError_t e) {
    if (e == cudaSuccess) return NFFT2D_OK;
    return e == cudaErrorMemoryAllocation ? NFFT2D_ERR_OOM : NFFT2D_ERR_CUDA;
}

#define FB_TRY(expr)                          \
    do {                                      \
        const int st_ = (expr);               \
        if (st_ != NFFT2D_OK) return st_;     \
    } while (0)
#define FB_CUDA(expr) FB_TRY(cuda_status(expr))

// Stream-ordered device buffers freed when the scope ends.
struct DevBufs {
    cudaStream_t st;
    std::vector<void *> ptrs;
    explicit DevBufs(cudaStream_t s) : st(s) {}
    ~DevBufs() {
        for (void *p : ptrs) cudaFreeAsync(p, st);
    }
    template <typename T>
    int get(T **out, size_t count) {
        void *p = nullptr;
        const cudaError_t e = cudaMallocAsync(&p, count * sizeof(T) + 16, st);
        if (e != cudaSuccess) return cuda_status(e);
        ptrs.push_back(p);
        *out = static_cast<T *>(p);
        return NFFT2D_OK;
    }
};

struct KnabGuard {
    nfft2d_knab k = nullptr;
    ~KnabGuard() {
        if (k) nfft2d_knab_destroy(k);
    }
};

// MATLAB linspace(d1, d2, n): d1 + i (d2 - d1)/(n - 1), the last sample d2.
std::vector<double> linspace(double d1, double d2, int n) {
    std::vector<double> v(static_cast<size_t>(n));
    const double step = (d2 - d1) / (n - 1);
    for (int i = 0; i < n - 1; ++i) v[static_cast<size_t>(i)] = d1 + static_cast<double>(i) * step;
    v[static_cast<size_t>(n - 1)] = d2;
    return v;
}

// mean(diff(v)): the differences summed in index order.
double mean_diff(const std::vector<double> &v) {
    double s = 0.0;
    for (size_t i = 0; i + 1 < v.size(); ++i) s += v[i + 1] - v[i];
    return s / static_cast<double>(v.size() - 1);
}

struct Ffbp {
    nfft2d_sar sar{};
    const double *X = nullptr, *Y = nullptr, *Z = nullptr, *R0 = nullptr;
    int nf = 0;
    const void *ph = nullptr;
    int prec = NFFT2D_F64;
    cudaStream_t st = nullptr;
    size_t csize = 16;          // bytes per complex sample
    nfft2d_plan leaf = nullptr;  // nf x 8 plan of the leaves' 1D transforms
    void *leaf_F = nullptr;
    nfft2d_ffbp_stats stats{};
    ~Ffbp() {
        if (leaf) nfft2d_plan_destroy(leaf);
        if (leaf_F) cudaFreeAsync(leaf_F, st);
    }
    // sqrt((X(i) - X(j))^2 + (Y(i) - Y(j))^2 + (Z(i) - Z(j))^2)
    double dist(int i, int j) const {
        const double dx = X[i] - X[j], dy = Y[i] - Y[j], dz = Z[i] - Z[j];
        return std::sqrt(dx * dx + dy * dy + dz * dz);
    }
};

// BP_POLAR_NFFT.m: pulses a..b back-projected onto the points (pho, cs).
int leaf(Ffbp &F, int a, int b, const double *pho, const double *cs, long long n, void *im) {
    if (!F.leaf) {
        FB_TRY(nfft2d_plan_create(&F.leaf, F.nf, kLeafN2, 2.0, 6, F.prec, F.st));
        FB_CUDA(cudaMallocAsync(&F.leaf_F, F.csize * F.nf * kLeafN2, F.st));
    }
    DevBufs mem(F.st);
    double *x1, *x2, *dr;
    void *f;
    FB_TRY(mem.get(&x1, n));
    FB_TRY(mem.get(&x2, n));
    FB_TRY(mem.get(&dr, n));
    FB_TRY(mem.get(reinterpret_cast<char **>(&f), n * F.csize));
    FB_CUDA(cudaMemsetAsync(x2, 0, sizeof(double) * n, F.st));
    const int nb = launch_blocks(n);
    ++F.stats.leaves;
    F.stats.leaf_points += n * (b - a + 1);
    const double scale = (-2.0 * F.sar.bw) / F.sar.c;
    const double k4fc = 4.0 * kPi * F.sar.fc;
    for (int p = a; p <= b; ++p) {
        const double xsi = F.dist(p, a);
        k_leaf_prep<<<nb, 256, 0, F.st>>>(pho, cs, n, xsi, xsi * xsi, F.R0[p], scale, x1, dr);
        const int eb = (F.nf * kLeafN2 + 255) / 256;
        if (F.prec == NFFT2D_F64)
            k_leaf_embed<double2><<<eb, 256, 0, F.st>>>(static_cast<const double2 *>(F.ph) + static_cast<size_t>(p) * F.nf,
                                                       F.nf, static_cast<double2 *>(F.leaf_F));
        else
            k_leaf_embed<float2><<<eb, 256, 0, F.st>>>(static_cast<const float2 *>(F.ph) + static_cast<size_t>(p) * F.nf,
                                                      F.nf, static_cast<float2 *>(F.leaf_F));
        FB_CUDA(cudaGetLastError());
        // no host round trip per pulse: the transform reads the work-item
        // count on the device; nfft2d_synchronize below reports errors
        FB_TRY(nfft2d_set_points_async(F.leaf, n, x1, x2, NFFT2D_COORD_F64, NFFT2D_UNITS_GRID));
        FB_TRY(nfft2d_type2(F.leaf, -1, F.leaf_F, f));  // NFFT1_1D.m:43: fft, negative exponent
        if (F.prec == NFFT2D_F64)
            k_leaf_acc<double2><<<nb, 256, 0, F.st>>>(static_cast<const double2 *>(f), dr, n, k4fc, F.sar.c,
                                                     static_cast<double2 *>(im), p == a);
        else
            k_leaf_acc<float2><<<nb, 256, 0, F.st>>>(static_cast<const float2 *>(f), dr, n, k4fc, F.sar.c,
                                                    static_cast<float2 *>(im), p == a);
        FB_CUDA(cudaGetLastError());
    }
    return nfft2d_synchronize(F.leaf);
}

// FFBP_POLAR_NFFT.m: the image of pulses a..b at the points (rho, cs), a
// len1 x len2 raster in the polar frame of antenna a.
int node(Ffbp &F, int a, int b, const double *rho, const double *cs, int len1, int len2, void *out, int level) {
    const long long n = static_cast<long long>(len1) * len2;
    if (level > F.stats.depth) F.stats.depth = level;
    if (b - a <= 2) return leaf(F, a, b, rho, cs, n, out);  // :27-36
    const int center = (a + b) / 2;                         // :24
    const double cl = F.sar.c;
    const double k4c = 4.0 * kPi / cl;
    const int nb = launch_blocks(n);
    for (int h = 0; h < 2; ++h) {
        const int sa = h ? center + 1 : a, sb = h ? b : center;
        const double dist = h ? F.dist(center + 1, a) : F.dist(a, a);  // :44, :96
        const double L = h ? F.dist(b, center) : F.dist(center, a);    // :54, :106
        DevBufs mem(F.st);
        double *rho_i, *cos_i;
        unsigned long long *mm;
        FB_TRY(mem.get(&rho_i, n));
        FB_TRY(mem.get(&cos_i, n));
        FB_TRY(mem.get(&mm, 4));
        const unsigned long long init[4] = {~0ull, 0ull, ~0ull, 0ull};
        FB_CUDA(cudaMemcpyAsync(mm, init, sizeof init, cudaMemcpyHostToDevice, F.st));
        k_polar_shift<<<nb, 256, 0, F.st>>>(rho, cs, n, dist, rho_i, cos_i, mm);
        FB_CUDA(cudaGetLastError());
        unsigned long long hm[4];
        FB_CUDA(cudaMemcpyAsync(hm, mm, sizeof hm, cudaMemcpyDeviceToHost, F.st));
        FB_CUDA(cudaStreamSynchronize(F.st));
        const double minrho = ord_value(hm[0]), maxrho = ord_value(hm[1]);
        const double mincos = ord_value(hm[2]), maxcos = ord_value(hm[3]);
        if (!std::isfinite(minrho) || !std::isfinite(maxrho) || !std::isfinite(mincos) || !std::isfinite(maxcos))
            return NFFT2D_ERR_NONFINITE;
        // :58-64 (110-116): sample counts and the padded sub-aperture axes
        const double Nrho = std::floor((maxrho - minrho) / (cl / (2.0 * F.sar.bw))) * 5.0;
        const double Ncos = std::floor((maxcos - mincos) / (cl / (2.0 * F.sar.f_max * L))) * 5.0 + 3.0;
        if (!(Nrho >= 2.0) || !(Ncos >= 2.0)) return NFFT2D_ERR_INVALID_ARG;
        if (Nrho + 60.0 > 46000.0 || Ncos + 60.0 > 46000.0) return NFFT2D_ERR_UNSUPPORTED;
        const int ncol = static_cast<int>(Nrho) + 60, nrow = static_cast<int>(Ncos) + 60;
        const double tr = 30.0 * (maxrho - minrho) / (Nrho - 1.0);
        const double tc = 30.0 * (maxcos - mincos) / (Ncos - 1.0);
        const std::vector<double> rho_in = linspace(minrho - tr, maxrho + tr, ncol);
        const std::vector<double> cos_in = linspace(mincos - tc, maxcos + tc, nrow);
        const long long ns = static_cast<long long>(nrow) * ncol;
        double *rax, *cax, *RHO, *COS;
        void *sub, *rec;
        FB_TRY(mem.get(&rax, ncol));
        FB_TRY(mem.get(&cax, nrow));
        FB_TRY(mem.get(&RHO, ns));
        FB_TRY(mem.get(&COS, ns));
        FB_TRY(mem.get(reinterpret_cast<char **>(&sub), ns * F.csize));
        FB_TRY(mem.get(reinterpret_cast<char **>(&rec), n * F.csize));
        FB_CUDA(cudaMemcpyAsync(rax, rho_in.data(), sizeof(double) * ncol, cudaMemcpyHostToDevice, F.st));
        FB_CUDA(cudaMemcpyAsync(cax, cos_in.data(), sizeof(double) * nrow, cudaMemcpyHostToDevice, F.st));
        k_meshgrid<<<launch_blocks(ns), 256, 0, F.st>>>(rax, cax, nrow, ncol, RHO, COS);
        FB_CUDA(cudaGetLastError());
        FB_TRY(node(F, sa, sb, RHO, COS, nrow, ncol, sub, level + 1));  // :71, :123
        ++F.stats.regrids;
        F.stats.regrid_points += n;
        F.stats.raster_cells += ns;
        // :73-79 -- back to baseband
        if (F.prec == NFFT2D_F64)
            k_phase_mul<double2><<<launch_blocks(ns), 256, 0, F.st>>>(static_cast<double2 *>(sub), RHO, ns, k4c,
                                                                    F.sar.fc, -1.0);
        else
            k_phase_mul<float2><<<launch_blocks(ns), 256, 0, F.st>>>(static_cast<float2 *>(sub), RHO, ns, k4c,
                                                                   F.sar.fc, -1.0);
        FB_CUDA(cudaGetLastError());
        // :81-89 -- Knab regridding onto this node's points, extrapolation NaN
        const double drho = mean_diff(rho_in), dcos = mean_diff(cos_in);
        KnabGuard kn;
        FB_TRY(nfft2d_knab_create(&kn.k, nrow, ncol, rho_in.data(), cos_in.data(), (1.0 / drho) * 0.5,
                                  (1.0 / dcos) * 0.5, F.prec, F.st));
        FB_TRY(nfft2d_knab_set_points(kn.k, len1, len2, rho_i, cos_i, NFFT2D_COORD_F64));
        FB_TRY(nfft2d_knab_execute(kn.k, NAN, 0.0, sub, rec));
        if (F.prec == NFFT2D_F64)
            k_phase_acc<double2><<<nb, 256, 0, F.st>>>(static_cast<const double2 *>(rec), rho_i, n, k4c, F.sar.fc,
                                                      static_cast<double2 *>(out), h == 0);
        else
            k_phase_acc<float2><<<nb, 256, 0, F.st>>>(static_cast<const float2 *>(rec), rho_i, n, k4c, F.sar.fc,
                                                     static_cast<float2 *>(out), h == 0);
        FB_CUDA(cudaGetLastError());
        FB_TRY(nfft2d_knab_synchronize(kn.k));
    }
    return NFFT2D_OK;
}

}  // namespace

extern "C" int nfft2d_ffbp_polar(const nfft2d_sar *sar, int np, const double *ant_x, const double *ant_y,
                                 const double *ant_z, const double *r0, int nf, const void *phdata, int a, int b,
                                 int len1, int len2, const double *rho_out, const double *cos_out, int precision,
                                 void *image, void *stream, nfft2d_ffbp_stats *stats) {
    if (!sar || !ant_x || !ant_y || !ant_z || !r0 || !phdata || !rho_out || !cos_out || !image)
        return NFFT2D_ERR_INVALID_ARG;
    if (np < 2 || nf < 2 || (nf & 1) || a < 0 || b >= np || a > b || len1 < 1 || len2 < 1)
        return NFFT2D_ERR_INVALID_ARG;
    if (precision != NFFT2D_F32 && precision != NFFT2D_F64) return NFFT2D_ERR_INVALID_ARG;
    if (!(sar->c > 0) || !(sar->bw > 0) || !(sar->f_max > 0) || !std::isfinite(sar->fc)) return NFFT2D_ERR_INVALID_ARG;
    Ffbp F;
    F.sar = *sar;
    F.X = ant_x;
    F.Y = ant_y;
    F.Z = ant_z;
    F.R0 = r0;
    F.nf = nf;
    F.ph = phdata;
    F.prec = precision;
    F.st = static_cast<cudaStream_t>(stream);
    F.csize = precision == NFFT2D_F64 ? sizeof(double2) : sizeof(float2);
    int st = node(F, a, b, rho_out, cos_out, len1, len2, image, 0);
    if (st == NFFT2D_OK) st = cuda_status(cudaStreamSynchronize(F.st));
    if (stats) *stats = F.stats;
    return st;
}
