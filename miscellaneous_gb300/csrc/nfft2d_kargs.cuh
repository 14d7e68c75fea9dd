// nfft2d_kargs.cuh -- kernel argument block shared by the gather and spread
// translation units.
#pragma once

#include "nfft2d_internal.h"

namespace nfft2d {

struct KArgs {
    Geom g;
    float alpha, cn, kp;     // window constants, FP32 kernels
    double alpha_d, cn_d;    // window constants, FP64 kernels
    float ds1, ds2;          // dt/dx of the caller's coordinate units (sigma * unit scale)
    double ds1_d, ds2_d;
    int n_chunks;            // work items (tiled kernels)
    int M;                   // points (direct kernels)
    int chunk;               // maximum points per work item of the chunk list
    int compensated;         // FP32 gathers: compensated (TwoSum) sum over the rows
    int binned_io;           // per-point arrays in the plan's binned order (else the caller's)
    int *status;             // [1]: latched error bits
    WinPoly poly;            // FP32 window polynomials (kernel parameter space)
};

inline KArgs make_kargs(const nfft2d_plan_s *p) {
    KArgs a{};
    a.g = p->g;
    a.alpha = static_cast<float>(p->w.alpha);
    a.cn = static_cast<float>(p->w.cn);
    a.kp = static_cast<float>(p->w.kp);
    a.alpha_d = p->w.alpha;
    a.cn_d = p->w.cn;
    a.ds1 = static_cast<float>(p->xscale1);
    a.ds2 = static_cast<float>(p->xscale2);
    a.ds1_d = p->xscale1;
    a.ds2_d = p->xscale2;
    a.n_chunks = static_cast<int>(p->n_chunks);
    a.M = static_cast<int>(p->M);
    a.compensated = p->compensated;
    a.binned_io = p->binned_io;
    a.chunk = p->chunk;
    a.status = p->d_status;
    a.poly = p->poly;
    return a;
}

// Patch buffers are 128-byte aligned in shared memory (TMA destination rule).
__host__ __device__ inline int patch_stride_elems(const Geom &g) { return ((g.PR * g.PC + 15) / 16) * 16; }

}  // namespace nfft2d
