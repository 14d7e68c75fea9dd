// compat_driver.cpp -- a reference-style caller of the compatibility
// headers.  It uses only the reference's own signatures (NFFT/NFFT2_2D.cuh,
// NFFT/NDFT2_2D.cuh), called the way Synthesis/PSO/Synthesis.cu:393-398 and
// :506-510 call them, and links against libnfft2d_gb300.so.  Deterministic
// inputs; all inputs and outputs are written to one binary file for the
// parity test to compare with the oracle.
//
// usage: nfft2d_compat_driver N1 N2 M seed out.bin
// file:  int32 N1, N2, M; float64 x[M], y[M]; complex128 data[M];
//        complex64 res_f32[N1*N2]; complex128 res_f64[N1*N2]; complex128 res_ndft[N1*N2]
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "NDFT2_2D.cuh"
#include "NFFT2_2D.cuh"

namespace {

uint64_t g_state = 0;
double next_uniform() {  // splitmix64 -> [0, 1)
    uint64_t z = (g_state += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z ^= z >> 31;
    return static_cast<double>(z >> 11) * (1.0 / 9007199254740992.0);
}

#define CK(x)                                                                   \
    do {                                                                        \
        cudaError_t e_ = (x);                                                   \
        if (e_ != cudaSuccess) {                                                \
            std::fprintf(stderr, "CUDA error %s at %d\n", cudaGetErrorString(e_), __LINE__); \
            return 2;                                                           \
        }                                                                       \
    } while (0)

}  // namespace

int main(int argc, char **argv) {
    if (argc != 6) {
        std::fprintf(stderr, "usage: %s N1 N2 M seed out.bin\n", argv[0]);
        return 1;
    }
    const int N1 = std::atoi(argv[1]), N2 = std::atoi(argv[2]), M = std::atoi(argv[3]);
    g_state = std::strtoull(argv[4], nullptr, 10);
    const char *path = argv[5];

    // points in grid units, uniform over one period; data uniform complex
    // (as Test_NFFT2_2D.m:15-18)
    std::vector<float> xf(M), yf(M);
    std::vector<float2> df(M);
    std::vector<double> xd(M), yd(M);
    std::vector<double2> dd(M);
    for (int p = 0; p < M; ++p) {
        xf[p] = static_cast<float>((next_uniform() - 0.5) * N1);
        yf[p] = static_cast<float>((next_uniform() - 0.5) * N2);
        df[p] = make_float2(static_cast<float>(next_uniform() - 0.5), static_cast<float>(next_uniform() - 0.5));
        xd[p] = xf[p];
        yd[p] = yf[p];
        dd[p] = make_double2(df[p].x, df[p].y);
    }
    const size_t NN = static_cast<size_t>(N1) * N2;

    // ---- single precision, as Synthesis.cu:395 ----
    float *d_xf, *d_yf;
    float2 *d_df, *d_rf;
    CK(cudaMalloc(&d_xf, sizeof(float) * M));
    CK(cudaMalloc(&d_yf, sizeof(float) * M));
    CK(cudaMalloc(&d_df, sizeof(float2) * M));
    CK(cudaMalloc(&d_rf, sizeof(float2) * NN));
    CK(cudaMemcpy(d_xf, xf.data(), sizeof(float) * M, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_yf, yf.data(), sizeof(float) * M, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_df, df.data(), sizeof(float2) * M, cudaMemcpyHostToDevice));
    Calculate_cuFFT_plan_C2C_NFFT2_2D(N1, N2);
    NFFT2_2D_GPU(d_rf, d_df, d_xf, d_yf, N1, N2, M);
    std::vector<float2> rf(NN);
    CK(cudaMemcpy(rf.data(), d_rf, sizeof(float2) * NN, cudaMemcpyDeviceToHost));

    // ---- double precision, as Synthesis.cu:506-508 ----
    double *d_xd, *d_yd;
    double2 *d_dd, *d_rd;
    CK(cudaMalloc(&d_xd, sizeof(double) * M));
    CK(cudaMalloc(&d_yd, sizeof(double) * M));
    CK(cudaMalloc(&d_dd, sizeof(double2) * M));
    CK(cudaMalloc(&d_rd, sizeof(double2) * NN));
    CK(cudaMemcpy(d_xd, xd.data(), sizeof(double) * M, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_yd, yd.data(), sizeof(double) * M, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_dd, dd.data(), sizeof(double2) * M, cudaMemcpyHostToDevice));
    Calculate_cuFFT_plan_Z2Z_NFFT2_2D(N1, N2);
    NFFT2_2D_GPU(d_rd, d_dd, d_xd, d_yd, N1, N2, M);
    std::vector<double2> rd(NN);
    CK(cudaMemcpy(rd.data(), d_rd, sizeof(double2) * NN, cudaMemcpyDeviceToHost));

    // ---- direct sum at the same frequencies, as Synthesis.cu:510 ----
    std::vector<double> u(NN), v(NN);
    for (int i = 0; i < N1; ++i)
        for (int j = 0; j < N2; ++j) {
            u[static_cast<size_t>(i) * N2 + j] = i - N1 / 2;
            v[static_cast<size_t>(i) * N2 + j] = j - N2 / 2;
        }
    double *d_u, *d_v;
    double2 *d_out;
    CK(cudaMalloc(&d_u, sizeof(double) * NN));
    CK(cudaMalloc(&d_v, sizeof(double) * NN));
    CK(cudaMalloc(&d_out, sizeof(double2) * NN));
    CK(cudaMemcpy(d_u, u.data(), sizeof(double) * NN, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_v, v.data(), sizeof(double) * NN, cudaMemcpyHostToDevice));
    NDFT2_2D_GPU(nullptr, d_xd, d_yd, d_u, d_v, d_dd, d_out, N1, N2, M, static_cast<int>(NN));
    std::vector<double2> rn(NN);
    CK(cudaMemcpy(rn.data(), d_out, sizeof(double2) * NN, cudaMemcpyDeviceToHost));
    Destroy_cuFFT_plan_NFFT2_2D();

    FILE *fp = std::fopen(path, "wb");
    if (!fp) return 3;
    const int32_t hdr[3] = {N1, N2, M};
    std::fwrite(hdr, sizeof(int32_t), 3, fp);
    std::fwrite(xd.data(), sizeof(double), M, fp);
    std::fwrite(yd.data(), sizeof(double), M, fp);
    std::fwrite(dd.data(), sizeof(double2), M, fp);
    std::fwrite(rf.data(), sizeof(float2), NN, fp);
    std::fwrite(rd.data(), sizeof(double2), NN, fp);
    std::fwrite(rn.data(), sizeof(double2), NN, fp);
    std::fclose(fp);
    cudaFree(d_xf); cudaFree(d_yf); cudaFree(d_df); cudaFree(d_rf);
    cudaFree(d_xd); cudaFree(d_yd); cudaFree(d_dd); cudaFree(d_rd);
    cudaFree(d_u); cudaFree(d_v); cudaFree(d_out);
    std::printf("ok\n");
    return 0;
}
