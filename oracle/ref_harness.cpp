// ref_harness.cpp -- runs the reference's own GPU spreading as a parity
// oracle.  TEST INFRASTRUCTURE ONLY: tests and bench.py's reference arm load
// it; the library never does.
//
// The reference's device code (NFFT/NFFT2_2D.cu: Kernel_Bessel,
// Interpolation_NFFT2_2D_GPUKernel with its dynamic-parallelism child
// series_terms, Decimation_and_Scaling) is compiled unchanged, together with
// the stand-in headers in oracle/ref_shims, into one device-linked cubin
// (oracle/build_ref.py).  A cubin carries no host code, so this file restates
// the host side of NFFT2_2D_GPU (NFFT/NFFT2_2D.cu:329-411 float, :413-495
// double) over the CUDA driver API: the same constants, launch shapes and
// launch order, the same per-call allocations and DEBUG synchronisations,
// and the process-global cuFFT plan of :11,49-55.
//
// Two things the reference leaves to its caller are done here:
//  * cudaLimitDevRuntimePendingLaunchCount >= the number of interpolation
//    threads (the reference's own call sits under `#if __CUDA_ARCH__ >= 350`
//    in host code, NFFT2_2D.cu:371-373, so it is compiled out);
//  * x, y and data are read before the kernel's `i < M` guard
//    (NFFT2_2D.cu:167-176), so the caller must pass arrays of at least
//    iDivUp(M, 256) * 256 elements; ref_nfft2_2d_gpu refuses shorter ones.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cufft.h>

#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>

namespace {

constexpr int kCC = 2;                  // NFFT2_2D.cu:20
constexpr int kK = 6;                   // NFFT2_2D.cu:21
constexpr int kBlockInterp = 256;       // BLOCKSIZE_INTERPOLATION
constexpr int kBlockXY = 16;            // BLOCK_SIZE_x / BLOCK_SIZE_y
constexpr int kBlockBessel = 32;        // BLOCKSIZE_BESSEL
constexpr double kPi = 3.141592653589793238463;

CUmodule g_mod = nullptr;
CUfunction g_bessel[2], g_interp[2], g_shift[2], g_decim[2];  // [0] float, [1] double
cufftHandle g_plan = 0;
int g_plan_n1 = 0, g_plan_n2 = 0, g_plan_type = -1;
size_t g_pending_limit = 0;
char g_err[512] = "";

int fail(const char *what, int code) {
    std::snprintf(g_err, sizeof g_err, "%s (code %d)", what, code);
    return code == 0 ? -1 : (code > 0 ? -code : code);
}

int idiv_up(int a, int b) { return (a + b - 1) / b; }

bool find_fn(const char *const *names, const CUfunction *fns, unsigned n, const char *a, const char *b,
             CUfunction *out) {
    for (unsigned i = 0; i < n; ++i)
        if (std::strstr(names[i], a) && std::strstr(names[i], b)) {
            *out = fns[i];
            return true;
        }
    return false;
}

int set_const_int(const char *name, int v) {
    CUdeviceptr p;
    size_t bytes;
    if (cuModuleGetGlobal(&p, &bytes, g_mod, name) != CUDA_SUCCESS || bytes != sizeof(int))
        return fail(name, -20);
    return cuMemcpyHtoD(p, &v, sizeof v) == CUDA_SUCCESS ? 0 : fail(name, -21);
}

template <class T>
int set_const_real(const char *name, T v) {
    CUdeviceptr p;
    size_t bytes;
    if (cuModuleGetGlobal(&p, &bytes, g_mod, name) != CUDA_SUCCESS || bytes != sizeof(T))
        return fail(name, -20);
    return cuMemcpyHtoD(p, &v, sizeof v) == CUDA_SUCCESS ? 0 : fail(name, -21);
}

// NFFT2_2D.cu:333-346 (float) / :417-430 (double): the constants are written
// on every call, as the reference does.
int write_constants(int N1, int N2, bool dbl) {
    int rc = 0;
    rc |= set_const_int("constant1_GPU", (kCC - 1) * N1 / 2);
    rc |= set_const_int("constant2_GPU", (kCC + 1) * N1 / 2);
    rc |= set_const_int("constant3_GPU", (kCC - 1) * N2 / 2);
    rc |= set_const_int("constant4_GPU", (kCC + 1) * N2 / 2);
    rc |= set_const_int("constant5_GPU", (kCC - 1) * N1 / 2 - N1 / 2);
    rc |= set_const_int("constant6_GPU", (kCC - 1) * N2 / 2 - N2 / 2);
    rc |= set_const_int("constant7_GPU", static_cast<int>(2. * kPi / (kCC * N1)));
    rc |= set_const_int("constant8_GPU", static_cast<int>(2. * kPi / (kCC * N2)));
    rc |= set_const_int("constant9_GPU", 2 * kK + 1);
    rc |= set_const_int("constant10_GPU", kK * kK);
    const double alfa = (2. - 1. / kCC) * kPi - 0.01;
    if (dbl) {
        rc |= set_const_real<double>("constant11_GPU", 1. / kPi);
        rc |= set_const_real<double>("constant12_GPU", alfa / kPi);
    } else {
        const float alfa_f = static_cast<float>(alfa);
        rc |= set_const_real<float>("constant11_GPU_f", static_cast<float>(1. / kPi));
        rc |= set_const_real<float>("constant12_GPU_f", static_cast<float>(alfa_f / kPi));
    }
    rc |= set_const_int("constant13_GPU", kCC * N1);
    rc |= set_const_int("constant14_GPU", kCC * N2);
    return rc ? fail("constant upload", -22) : 0;
}

// Calculate_cuFFT_plan_{C2C,Z2Z}_NFFT2_2D (NFFT2_2D.cu:49-50), kept per
// size so one process can run several shapes.
int ensure_plan(int N1, int N2, bool dbl) {
    const int type = dbl ? CUFFT_Z2Z : CUFFT_C2C;
    if (g_plan && g_plan_n1 == N1 && g_plan_n2 == N2 && g_plan_type == type) return 0;
    if (g_plan) cufftDestroy(g_plan);
    g_plan = 0;
    const cufftResult r = cufftPlan2d(&g_plan, kCC * N1, kCC * N2, static_cast<cufftType>(type));
    if (r != CUFFT_SUCCESS) {
        g_plan = 0;
        return fail("cufftPlan2d", -30 - static_cast<int>(r));
    }
    g_plan_n1 = N1;
    g_plan_n2 = N2;
    g_plan_type = type;
    return 0;
}

#define RT(call, code)                                                           \
    do {                                                                         \
        cudaError_t e_ = (call);                                                 \
        if (e_ != cudaSuccess) return fail(cudaGetErrorString(e_), code);        \
    } while (0)
#define DRV(call, code)                                                          \
    do {                                                                         \
        if ((call) != CUDA_SUCCESS) return fail(#call, code);                    \
    } while (0)

template <class Real, class Cplx>
int run(Cplx *result, const Cplx *data, const Real *x, const Real *y, int N1, int N2, int M, long long M_alloc,
        float *interp_ms, float *total_ms) {
    const bool dbl = sizeof(Real) == 8;
    const int v = dbl ? 1 : 0;
    if (!g_mod) return fail("ref_load not called", -2);
    if (N1 <= 0 || N2 <= 0 || (N1 & 1) || (N2 & 1) || M <= 0) return fail("bad size", -3);
    const int grid_interp = idiv_up(M, kBlockInterp);
    // The interpolation kernel reads x[i], y[i], data[i] for every launched
    // thread before its i < M guard (NFFT2_2D.cu:167-176).
    if (M_alloc < static_cast<long long>(grid_interp) * kBlockInterp) return fail("inputs not padded to 256", -4);

    const auto t0 = std::chrono::steady_clock::now();
    if (int rc = ensure_plan(N1, N2, dbl)) return rc;
    if (int rc = write_constants(N1, N2, dbl)) return rc;

    Real *bx = nullptr, *by = nullptr;
    Cplx *grid = nullptr;
    RT(cudaMalloc(&bx, sizeof(Real) * N1), -5);
    RT(cudaMalloc(&by, sizeof(Real) * N2), -5);
    // Kernel_Bessel<T>(T*, int), NFFT2_2D.cu:352-363
    {
        int n = N1;
        void *args[] = {&bx, &n};
        DRV(cuLaunchKernel(g_bessel[v], idiv_up(N1, kBlockBessel), 1, 1, kBlockBessel, 1, 1, 0, 0, args, nullptr), -6);
        RT(cudaDeviceSynchronize(), -7);
        n = N2;
        void *args2[] = {&by, &n};
        DRV(cuLaunchKernel(g_bessel[v], idiv_up(N2, kBlockBessel), 1, 1, kBlockBessel, 1, 1, 0, 0, args2, nullptr), -6);
        RT(cudaDeviceSynchronize(), -7);
    }
    const size_t cells = static_cast<size_t>(kCC) * N1 * kCC * N2;
    RT(cudaMalloc(&grid, sizeof(Cplx) * cells), -5);
    RT(cudaMemset(grid, 0, sizeof(Cplx) * cells), -8);

    const size_t need = static_cast<size_t>(grid_interp) * kBlockInterp;
    if (need > g_pending_limit) {
        RT(cudaDeviceSetLimit(cudaLimitDevRuntimePendingLaunchCount, need), -9);
        g_pending_limit = need;
    }
    cudaEvent_t e0, e1;
    RT(cudaEventCreate(&e0), -10);
    RT(cudaEventCreate(&e1), -10);
    // Interpolation_NFFT2_2D_GPUKernel<<<iDivUp(M,256),256>>>(data, grid, x, y, N1, N2, M), :370-378
    {
        int n1 = N1, n2 = N2, m = M;
        void *args[] = {&data, &grid, &x, &y, &n1, &n2, &m};
        RT(cudaEventRecord(e0, 0), -10);
        DRV(cuLaunchKernel(g_interp[v], grid_interp, 1, 1, kBlockInterp, 1, 1, 0, 0, args, nullptr), -6);
        RT(cudaEventRecord(e1, 0), -10);
        RT(cudaDeviceSynchronize(), -7);
    }
    float ms = 0.f;
    RT(cudaEventElapsedTime(&ms, e0, e1), -10);
    if (interp_ms) *interp_ms = ms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);

    // fftshift_2D, cuFFT forward, fftshift_2D, :380-397
    const unsigned gs1 = (kCC * N1) / kBlockXY + ((kCC * N1) % kBlockXY == 0 ? 0 : 1);
    const unsigned gs2 = (kCC * N2) / kBlockXY + ((kCC * N2) % kBlockXY == 0 ? 0 : 1);
    {
        int n1 = kCC * N1, n2 = kCC * N2;
        void *args[] = {&grid, &n1, &n2};
        DRV(cuLaunchKernel(g_shift[v], gs1, gs2, 1, kBlockXY, kBlockXY, 1, 0, 0, args, nullptr), -6);
        RT(cudaDeviceSynchronize(), -7);
        cufftResult r;
        if (dbl)
            r = cufftExecZ2Z(g_plan, reinterpret_cast<cufftDoubleComplex *>(grid),
                             reinterpret_cast<cufftDoubleComplex *>(grid), CUFFT_FORWARD);
        else
            r = cufftExecC2C(g_plan, reinterpret_cast<cufftComplex *>(grid), reinterpret_cast<cufftComplex *>(grid),
                             CUFFT_FORWARD);
        if (r != CUFFT_SUCCESS) return fail("cufftExec", -30 - static_cast<int>(r));
        DRV(cuLaunchKernel(g_shift[v], gs1, gs2, 1, kBlockXY, kBlockXY, 1, 0, 0, args, nullptr), -6);
        RT(cudaDeviceSynchronize(), -7);
    }
    // Decimation_and_Scaling, :400-406 (grid x over c N2, y over c N1)
    {
        int n1 = N1, n2 = N2;
        void *args[] = {&grid, &result, &bx, &by, &n1, &n2};
        DRV(cuLaunchKernel(g_decim[v], gs2, gs1, 1, kBlockXY, kBlockXY, 1, 0, 0, args, nullptr), -6);
        RT(cudaDeviceSynchronize(), -7);
    }
    RT(cudaFree(bx), -11);
    RT(cudaFree(by), -11);
    RT(cudaFree(grid), -11);
    const auto t1 = std::chrono::steady_clock::now();
    if (total_ms) *total_ms = std::chrono::duration<float, std::milli>(t1 - t0).count();
    return 0;
}

}  // namespace

extern "C" {

const char *ref_last_error(void) { return g_err; }

// Loads the device-linked cubin into the current (primary) context and
// resolves the kernels by their mangled names.  Returns 0 or a negative code.
int ref_load(const char *cubin_path) {
    if (g_mod) return 0;
    RT(cudaFree(nullptr), -1);  // make the runtime's primary context current
    if (cuModuleLoad(&g_mod, cubin_path) != CUDA_SUCCESS) {
        g_mod = nullptr;
        return fail("cuModuleLoad", -12);
    }
    unsigned count = 0;
    DRV(cuModuleGetFunctionCount(&count, g_mod), -13);
    if (count == 0 || count > 64) return fail("unexpected kernel count", -13);
    CUfunction fns[64];
    const char *names[64];
    DRV(cuModuleEnumerateFunctions(fns, count, g_mod), -13);
    for (unsigned i = 0; i < count; ++i) DRV(cuFuncGetName(&names[i], fns[i]), -13);
    const bool ok = find_fn(names, fns, count, "Kernel_BesselIf", "", &g_bessel[0]) &&
                    find_fn(names, fns, count, "Kernel_BesselId", "", &g_bessel[1]) &&
                    find_fn(names, fns, count, "Interpolation_NFFT2_2D_GPUKernel", "6float2", &g_interp[0]) &&
                    find_fn(names, fns, count, "Interpolation_NFFT2_2D_GPUKernel", "7double2", &g_interp[1]) &&
                    find_fn(names, fns, count, "fftshift_2DI6float2", "", &g_shift[0]) &&
                    find_fn(names, fns, count, "fftshift_2DI7double2", "", &g_shift[1]) &&
                    find_fn(names, fns, count, "Decimation_and_Scaling", "6float2", &g_decim[0]) &&
                    find_fn(names, fns, count, "Decimation_and_Scaling", "7double2", &g_decim[1]);
    if (!ok) {
        cuModuleUnload(g_mod);
        g_mod = nullptr;
        return fail("kernel not found in cubin", -14);
    }
    return 0;
}

// The reference's NFFT2_2D_GPU, float and double overloads: type 1 with
// sign -1 on grid-unit coordinates.  M_alloc is the element count of x, y
// and data (>= iDivUp(M, 256) * 256).  interp_ms: CUDA-event time of the
// interpolation launch with its child grids; total_ms: host time of the
// whole call (per-call constants, allocations and synchronisations included).
int ref_nfft2_2d_gpu_f32(void *result, const void *data, const float *x, const float *y, int N1, int N2, int M,
                         long long M_alloc, float *interp_ms, float *total_ms) {
    return run<float, float2>(static_cast<float2 *>(result), static_cast<const float2 *>(data), x, y, N1, N2, M,
                              M_alloc, interp_ms, total_ms);
}

int ref_nfft2_2d_gpu_f64(void *result, const void *data, const double *x, const double *y, int N1, int N2, int M,
                         long long M_alloc, float *interp_ms, float *total_ms) {
    return run<double, double2>(static_cast<double2 *>(result), static_cast<const double2 *>(data), x, y, N1, N2, M,
                                M_alloc, interp_ms, total_ms);
}

}  // extern "C"
