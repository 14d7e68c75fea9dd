// nfft2d_compat.cu -- the reference's own call surface (NFFT/NFFT2_2D.cuh:4-11,
// NFFT/NDFT2_2D.cuh:4-6) implemented over the C ABI, so reference callers
// relink unchanged.  See include/NFFT2_2D.cuh for the kept semantics and the
// deliberate differences.
#include <cuda_runtime.h>
#include <cufft.h>

#include <cstdio>
#include <mutex>

#include "../../include/NDFT2_2D.cuh"
#include "../../include/NFFT2_2D.cuh"
#include "../../include/nfft2d_gb300.h"
#include "nfft2d_internal.h"

cufftHandle NFFT2_2D_GPUplan = 0;

namespace {

// The reference fixes c = 2 and K = 6 at compile time (NFFT2_2D.cu:20-21).
constexpr double kRefSigma = 2.0;
constexpr int kRefK = 6;

struct CachedPlan {
    nfft2d_plan plan = nullptr;
    int N1 = 0, N2 = 0;
};

std::mutex g_mu;
CachedPlan g_plans[2];  // [NFFT2D_F32], [NFFT2D_F64]

void report(const char *what, int st) {
    if (st != NFFT2D_OK) std::fprintf(stderr, "nfft2d_gb300: %s failed: %s\n", what, nfft2d_status_string(st));
}

// Caller holds g_mu.
nfft2d_plan get_plan(int precision, int N1, int N2, bool recreate) {
    CachedPlan &c = g_plans[precision];
    if (c.plan && (recreate || c.N1 != N1 || c.N2 != N2)) {
        nfft2d_plan_destroy(c.plan);
        c.plan = nullptr;
    }
    if (!c.plan) {
        nfft2d_plan p = nullptr;
        const int st = nfft2d_plan_create(&p, N1, N2, kRefSigma, kRefK, precision, nullptr);
        report("plan creation", st);
        if (st != NFFT2D_OK) return nullptr;
        c.plan = p;
        c.N1 = N1;
        c.N2 = N2;
        NFFT2_2D_GPUplan = p->fft;
    }
    return c.plan;
}

template <int PREC>
void run_nfft2(void *result, const void *data, const void *x, const void *y, int N1, int N2, int M) {
    std::lock_guard<std::mutex> lock(g_mu);
    nfft2d_plan p = get_plan(PREC, N1, N2, false);
    if (!p) return;
    const int cd = PREC == NFFT2D_F64 ? NFFT2D_COORD_F64 : NFFT2D_COORD_F32;
    int st = nfft2d_set_points(p, M, x, y, cd, NFFT2D_UNITS_GRID);
    report("NFFT2_2D_GPU set_points", st);
    if (st != NFFT2D_OK) return;
    st = nfft2d_spread_ref(p, data, result);
    report("NFFT2_2D_GPU", st);
    if (st != NFFT2D_OK) return;
    report("NFFT2_2D_GPU synchronize", nfft2d_synchronize(p));
}

}  // namespace

// Reference NFFT2_2D.cu:49 -- cufftPlan2d(&NFFT2_2D_GPUplan, c*N1, c*N2, C2C).
void Calculate_cuFFT_plan_C2C_NFFT2_2D(const int N1, const int N2) {
    std::lock_guard<std::mutex> lock(g_mu);
    get_plan(NFFT2D_F32, N1, N2, true);
}

// Reference NFFT2_2D.cu:50 -- Z2Z twin.
void Calculate_cuFFT_plan_Z2Z_NFFT2_2D(const int N1, const int N2) {
    std::lock_guard<std::mutex> lock(g_mu);
    get_plan(NFFT2D_F64, N1, N2, true);
}

// Reference NFFT2_2D.cu:55.
void Destroy_cuFFT_plan_NFFT2_2D() {
    std::lock_guard<std::mutex> lock(g_mu);
    for (auto &c : g_plans) {
        if (c.plan) nfft2d_plan_destroy(c.plan);
        c = CachedPlan{};
    }
    NFFT2_2D_GPUplan = 0;
}

// Reference NFFT2_2D.cu:329-411 (float) and :413-495 (double).
void NFFT2_2D_GPU(float2 *__restrict__ result, const float2 *__restrict__ data, const float *__restrict__ x,
                  const float *__restrict__ y, const int N1, const int N2, const int M) {
    run_nfft2<NFFT2D_F32>(result, data, x, y, N1, N2, M);
}

void NFFT2_2D_GPU(double2 *__restrict__ result, const double2 *__restrict__ data, const double *__restrict__ x,
                  const double *__restrict__ y, const int N1, const int N2, const int M) {
    run_nfft2<NFFT2D_F64>(result, data, x, y, N1, N2, M);
}

// Reference NDFT2_2D.cu:37-72 (the cuBLAS handle is unused).
extern "C" void NDFT2_2D_GPU(cublasHandle_t, const double *__restrict__ d_X, const double *__restrict__ d_Y,
                             const double *__restrict__ d_u, const double *__restrict__ d_v,
                             const NFFT2D_DOUBLE2_T *__restrict__ d_in, NFFT2D_DOUBLE2_T *__restrict__ d_out,
                             const int Nu, const int Nv, const int M, const int N) {
    int st = nfft2d_ndft2d_f64(d_X, d_Y, d_u, d_v, d_in, d_out, Nu, Nv, M, N, -1, nullptr);
    report("NDFT2_2D_GPU", st);
    if (st == NFFT2D_OK && cudaStreamSynchronize(nullptr) != cudaSuccess) report("NDFT2_2D_GPU", NFFT2D_ERR_CUDA);
}
