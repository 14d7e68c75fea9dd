/*
 * nfft2d_gb300.h -- C ABI of the GB300 (sm_103a) 2D NFFT.
 *
 * One shared library, libnfft2d_gb300.so, exports every function declared
 * here with C linkage: plain pointers, sizes and status codes, no C++ or
 * torch types.  Array arguments are DEVICE pointers owned by the caller
 * (as in the reference, NFFT/NFFT2_2D.cuh:8-11 and NFFT/NDFT2_2D.cuh:4-6;
 * nfft2d_set_points also takes page-locked host coordinates);
 * work buffers are owned by a plan, allocated once at plan creation /
 * set_points, never per call.
 *
 * Conventions (shared with the reference, NFFT/NFFT2_2D.cu:23,66,124-125 and
 * BP_FBP_FFBP/NFFT1_2D.m:17-18,29-30,55):
 *   - a coefficient array F is N1 x N2 complex, row-major, element
 *     F[i*N2 + j] holds frequency (k1, k2) = (i - N1/2, j - N2/2);
 *   - point p has coordinates (x1_p, x2_p); x1 pairs with N1 (rows);
 *   - in GRID units a coordinate spans one period over [-N/2, N/2) (the
 *     reference's units); in UNIT units over [-0.5, 0.5); in RADIANS over
 *     [-pi, pi).  Any real value is accepted and wrapped periodically;
 *   - complex values are interleaved (re, im): float2 for NFFT2D_F32 plans,
 *     double2 for NFFT2D_F64 plans.
 *
 * Transforms (x in grid units):
 *   type 2 ("forward", reference NFFT1_2D, non-equispaced results):
 *       f_p = sum_k F_k exp(sign * 2 pi i (k1 x1_p / N1 + k2 x2_p / N2))
 *   type 1 (spreading, reference NFFT2_2D, non-equispaced data):
 *       F_k = sum_p f_p exp(sign * 2 pi i (k1 x1_p / N1 + k2 x2_p / N2))
 * The reference uses sign = -1 for both (NFFT2_2D.m:63, NFFT1_2D.m:55), so
 * its NFFT2_2D is the transpose of NFFT1_2D; the Hermitian adjoint of the
 * forward is type 1 with sign = +1.
 *
 * Every function returns an int status (NFFT2D_OK = 0, negative on error)
 * and never exits the process.  Transforms are asynchronous on the plan's
 * stream; device-side faults that a kernel detects itself (a bounded wait
 * that ran out, a corrupted bin record) are latched in the plan and
 * reported by the next nfft2d_synchronize(), which then clears them: each
 * such error is reported once, and a later correct run reports NFFT2D_OK.
 */
#ifndef NFFT2D_GB300_H
#define NFFT2D_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define NFFT2D_OK                   0
#define NFFT2D_ERR_INVALID_ARG     -1  /* bad size, null pointer, bad enum       */
#define NFFT2D_ERR_OOM             -2  /* device or host allocation failed        */
#define NFFT2D_ERR_CUDA            -3  /* a CUDA runtime call failed              */
#define NFFT2D_ERR_CUFFT           -4  /* a cuFFT call failed                     */
#define NFFT2D_ERR_NO_POINTS       -5  /* transform called before set_points      */
#define NFFT2D_ERR_NONFINITE       -6  /* a coordinate was NaN or +-Inf           */
#define NFFT2D_ERR_DEVICE_TIMEOUT  -7  /* a bounded device-side wait ran out      */
#define NFFT2D_ERR_DEVICE_BOUNDS   -8  /* a kernel rejected an out-of-tile record */
#define NFFT2D_ERR_UNSUPPORTED     -9  /* valid request this build does not serve */
#define NFFT2D_ERR_INTERNAL       -10
#define NFFT2D_ERR_SCRATCH_LIMIT  -11  /* size beyond the fixed scratch of the no-allocation entry point */

/* ---- enums ------------------------------------------------------------ */
#define NFFT2D_F32 0   /* complex64 data, FP32 kernels (FP64 plan-time math) */
#define NFFT2D_F64 1   /* complex128 data, FP64 kernels                      */

#define NFFT2D_COORD_F32 0
#define NFFT2D_COORD_F64 1

#define NFFT2D_UNITS_GRID    0  /* reference units: period N_d             */
#define NFFT2D_UNITS_UNIT    1  /* period 1, [-0.5, 0.5)                   */
#define NFFT2D_UNITS_RADIANS 2  /* period 2*pi, [-pi, pi)                  */

/* Kernel variants for the gather (type 2) and the spread (type 1).  AUTO:
 * FP32 spreads are TILED; the FP32 gather is chosen at set_points (DIRECT
 * from 128 points per 16 x 16 tile or 2^18 points up, else TILED);
 * FP64 uses DIRECT. */
#define NFFT2D_VARIANT_AUTO   0
#define NFFT2D_VARIANT_TILED  1  /* binned tiles staged by TMA in shared memory */
#define NFFT2D_VARIANT_DIRECT 2  /* sorted points, taps read straight from L2   */

typedef struct nfft2d_plan_s *nfft2d_plan;

typedef struct {
    int N1, N2;            /* coefficient grid                                  */
    double sigma;          /* oversampling factor (reference c)                 */
    int K;                 /* window half-width: 2K+1 taps per dimension        */
    int precision;         /* NFFT2D_F32 / NFFT2D_F64                           */
    int n1, n2;            /* oversampled grid sigma*N1 x sigma*N2              */
    int halo;              /* periodic halo cells around the oversampled grid   */
    int rows, cols;        /* padded grid allocation: whole tiles + halo each side */
    int tile;              /* bin tile edge, in oversampled cells               */
    int tiles1, tiles2;    /* number of tiles per dimension                     */
    int patch_rows, patch_cols; /* shared-memory patch of one tile with halo    */
    int chunk;             /* maximum points per work item                      */
    int gather_variant, spread_variant;
    long long M;           /* points currently set (0 before set_points)        */
    long long n_chunks;    /* work items built by the last set_points           */
    size_t workspace_bytes;/* device bytes owned by the plan                    */
    int fft_mode;          /* oversampled FFT in use: 0 2D cuFFT plan, 1 cuFFT
                              passes, 2 fused passes (see nfft2d_tuning)       */
} nfft2d_info;

typedef struct {
    int tile;              /* 0 or -1 = keep; else 8, 16, 32 or 64              */
    int chunk;             /* 0 or -1 = keep; else points per work item (>= 32):
                              a tile's points are cut into items of this many;
                              the tiled gather stages one patch per item and
                              the tiled spread gives each item to one warp     */
    int gather_variant;    /* -1 = keep; NFFT2D_VARIANT_* (AUTO: chosen at
                              set_points from the bin density)                  */
    int spread_variant;    /* -1 = keep; NFFT2D_VARIANT_*                       */
    int compensated;       /* -1 = default (on); 0 off; 1 on (FP32 gather)      */
    int fft_mode;          /* -1 = keep.  Initially automatic: 2 below 2048 x
                              2048 oversampled cells where it applies, else 1
                              from 2048 x 2048 cells up, else 0.
                              0: one 2D cuFFT plan; 1: two 1D cuFFT passes, the
                              column pass only over the columns the band needs
                              (1.5 instead of 2 passes at sigma = 2); 2: the
                              library's own FFT passes fused with deapodize/pad,
                              halo fill, halo fold and crop (FP32 plans, grid
                              sides powers of two from 64 to 4096, else
                              NFFT2D_ERR_UNSUPPORTED)                           */
    int io_order;          /* -1 = keep.  NFFT2D_ORDER_CALLER (initially): the
                              per-point arrays (f of type 2 / type 1, v, g1,
                              g2 of grad_x) follow the caller's point order.
                              NFFT2D_ORDER_BINNED: they follow the plan's
                              binned order instead -- entry i belongs to the
                              caller's point perm[i] of nfft2d_get_permutation
                              -- so the gather writes and the spread reads
                              them contiguously (a caller that keeps its
                              vectors in that order, an iterative solver, saves
                              the random 8-byte accesses of the caller's
                              order).  Set it before set_points or after. */
} nfft2d_tuning;

#define NFFT2D_ORDER_CALLER 0
#define NFFT2D_ORDER_BINNED 1

/* Stage times in milliseconds, from CUDA events recorded on the plan's
 * stream while timing is enabled.  Each field holds the most recent run of
 * that stage: a type-2 call refreshes pad / fft_type2 / halo_fill / gather,
 * a type-1 call refreshes spread / fold / fft_type1 / crop, set_points
 * refreshes sort; fields of stages that never ran are 0. */
typedef struct {
    float sort_ms;         /* set_points: binning + counting sort               */
    float pad_ms;          /* type 2: deapodize + zero-pad                      */
    float fft_type2_ms;    /* type 2: cuFFT on the oversampled grid             */
    float halo_fill_ms;    /* type 2: periodic halo fill                        */
    float gather_ms;       /* type 2: windowed gather (or coordinate gradient)  */
    float spread_ms;       /* type 1: zero the grid + windowed spread           */
    float fold_ms;         /* type 1: fold the halo onto the interior           */
    float fft_type1_ms;    /* type 1: cuFFT on the oversampled grid             */
    float crop_ms;         /* type 1: crop + deapodize                          */
} nfft2d_timings;

/* ---- plan life cycle --------------------------------------------------
 * Replaces the reference's process-global cuFFT plan
 * (NFFT/NFFT2_2D.cu:11,49-55: Calculate_cuFFT_plan_C2C_NFFT2_2D,
 * Calculate_cuFFT_plan_Z2Z_NFFT2_2D, Destroy_cuFFT_plan_NFFT2_2D) and the
 * per-call cudaMalloc/Kernel_Bessel work of NFFT2_2D_GPU (:333-367).
 * sigma*N1 and sigma*N2 must be even integers >= N and >= 2K+2; N1, N2 even;
 * 2 <= K <= 8; sigma >= 1.25.  stream may be NULL (legacy default stream). */
int nfft2d_plan_create(nfft2d_plan *plan, int N1, int N2, double sigma, int K, int precision, void *stream);
int nfft2d_plan_destroy(nfft2d_plan plan);
int nfft2d_set_stream(nfft2d_plan plan, void *stream);
int nfft2d_set_tuning(nfft2d_plan plan, const nfft2d_tuning *tuning);
int nfft2d_get_info(nfft2d_plan plan, nfft2d_info *info);

/* The binned order of the points set last: perm[i] = the caller's index of
 * the point at binned position i (M ints, DEVICE).  Asynchronous on the
 * plan's stream.  No reference counterpart. */
int nfft2d_get_permutation(nfft2d_plan plan, int *perm);

/* Host-only: the layout a plan with these parameters would use (no GPU
 * needed).  tile = 0 picks the default. */
int nfft2d_layout_query(int N1, int N2, double sigma, int K, int precision, int tile, nfft2d_info *info);

/* ---- points -------------------------------------------------------------
 * Bins and sorts the M points into tiles of the oversampled grid (the
 * reference recomputes mu = rint(c*x) per call inside
 * Interpolation_NFFT2_2D_GPUKernel, NFFT2_2D.cu:163-173).  The coordinate
 * reduction runs in FP64.  Synchronizes the plan's stream.  M = 0 is valid
 * (transforms then produce zeros).  x1, x2 may be device memory or
 * page-locked host memory (read over the host link by the binning pass
 * itself, no separate upload); other host memory only where the device can
 * read pageable memory, else NFFT2D_ERR_INVALID_ARG. */
int nfft2d_set_points(nfft2d_plan plan, long long M, const void *x1, const void *x2, int coord_dtype, int units);

/* As nfft2d_set_points, but returns once the binning is enqueued on the
 * plan's stream, without a host round trip (no reference counterpart: the
 * reference re-derives the bins inside every transform).  The transforms
 * that follow read the work-item count from device memory; x1 and x2 must
 * stay valid until the stream has run the binning.  A non-finite coordinate
 * is reported by the next nfft2d_synchronize (NFFT2D_ERR_NONFINITE, which
 * also drops the point set); transforms enqueued before that produce
 * unspecified values but stay in bounds.  nfft2d_get_info reports n_chunks
 * = -1 until nfft2d_synchronize has read the count back. */
int nfft2d_set_points_async(nfft2d_plan plan, long long M, const void *x1, const void *x2, int coord_dtype,
                            int units);

/* nfft2d_set_points_async followed by nfft2d_forward (type 2, sign -1) in one
 * call, with the same result: the forward's padding and FFT, which read only
 * F, run on a second stream while the binning reads the coordinates (from
 * page-locked host memory over the host link, or from the device) and sorts
 * them; the gather follows both on the plan's stream.  F may be device
 * memory or page-locked host memory; from the host it is copied (into a
 * device buffer the plan keeps) once the coordinates have been read, so the
 * two uploads do not share the link and the copy overlaps the rest of the
 * binning.  inputs_read_event (a cudaEvent_t, or NULL) is recorded once the
 * call's inputs have been read -- the coordinates, and a host F -- so their
 * buffers and the host link are free from there (e.g. to upload the next
 * inputs).
 * Pageable host memory returns NFFT2D_ERR_INVALID_ARG.  Not for plans of a
 * batch.  No reference counterpart. */
int nfft2d_bin_and_forward(nfft2d_plan plan, long long M, const void *x1, const void *x2, int coord_dtype, int units,
                           const void *F, void *f, void *inputs_read_event);

/* ---- transforms ---------------------------------------------------------
 * nfft2d_forward   : type 2, sign -1  (BP_FBP_FFBP/NFFT1_2D.m:1-69)
 * nfft2d_adjoint   : type 1, sign +1  (Hermitian adjoint of nfft2d_forward)
 * nfft2d_spread_ref: type 1, sign -1  (NFFT/NFFT2_2D.cu:329-495 and
 *                    NFFT/NFFT2/Matlab/NFFT2_2D.m:1-72)
 * f has M entries in the caller's point order; F has N1*N2 entries. */
int nfft2d_forward(nfft2d_plan plan, const void *F, void *f);
int nfft2d_adjoint(nfft2d_plan plan, const void *f, void *F);
int nfft2d_spread_ref(nfft2d_plan plan, const void *f, void *F);
int nfft2d_type2(nfft2d_plan plan, int sign, const void *F, void *f);
int nfft2d_type1(nfft2d_plan plan, int sign, const void *f, void *F);

/* Gradient of a type-2 transform w.r.t. the point coordinates, contracted
 * with a cotangent v (M complex):
 *     g1[p] = Re( conj(v_p) * d f_p / d x1_p ),  g2 likewise for x2,
 * in the units given to set_points; g1, g2 are M reals of the plan's
 * precision.  For L = ||f - y||^2 pass v = 2 (f - y).  No reference
 * counterpart (added differentiation of the forward gather). */
int nfft2d_grad_x(nfft2d_plan plan, int sign, const void *F, const void *v, void *g1, void *g2);

/* ---- status / timing ---------------------------------------------------- */
int nfft2d_synchronize(nfft2d_plan plan);
int nfft2d_enable_timing(nfft2d_plan plan, int on);
int nfft2d_get_timings(nfft2d_plan plan, nfft2d_timings *t);
const char *nfft2d_status_string(int status);
int nfft2d_device_count(void);
/* Self-test of the bounded device-side waits (no reference counterpart): one
 * thread polls an mbarrier phase that nothing completes, gives up after
 * spin_limit polls -- as the tiled kernels do after their own limit -- and
 * the call returns NFFT2D_ERR_DEVICE_TIMEOUT with the context intact.
 * Synchronizes `stream`. */
int nfft2d_selftest_wait_timeout(int spin_limit, void *stream);
/* The same bounded wait enqueued on a plan's stream, latching its timeout in
 * the plan's status word as the plan's own kernels do: the next
 * nfft2d_synchronize returns NFFT2D_ERR_DEVICE_TIMEOUT (once).  Asynchronous. */
int nfft2d_plan_selftest_wait_timeout(nfft2d_plan plan, int spin_limit);

/* ---- exact direct sum ----------------------------------------------------
 * Matrix-free FP64 replacement of NDFT2_2D_GPU (NFFT/NDFT2_2D.cu:37-72):
 *     out[q] = sum_p in[p] exp(sign * 2 pi i (u_q X_p / Nu + v_q Y_p / Nv))
 * for M points and N frequencies (u_q, v_q arbitrary reals); in/out are
 * double2.  The reference uses sign = -1, builds an explicit M x N matrix
 * and dumps it to a file; this builds no matrix and writes no file. */
int nfft2d_ndft2d_f64(const double *X, const double *Y, const double *u, const double *v,
                      const void *in, void *out, int Nu, int Nv, long long M, long long N,
                      int sign, void *stream);

/* ---- batches: many transforms of uneven size in one go ------------------
 * No reference counterpart: the reference runs one NFFT2_2D_GPU per PSO
 * particle in a host loop (Synthesis/PSO/PSO.cu:348, Synthesis.cu:395).
 * A batch holds `count` FP32 transforms (N1[t] x N2[t], shared sigma and K
 * -- or a K per transform with nfft2d_batch_create_k --, 16 x 16 tiles).  Grids of equal size share one batched cuFFT plan; every
 * other stage covers all transforms with one launch (a gather with one
 * thread per binned point of all transforms, a persistent spread over the
 * work items of all transforms); the stage sequence
 * is captured into a CUDA graph on first use and replayed (set_graph(0) runs
 * it eagerly instead).  set_points binds per-transform point arrays (FP32 or
 * FP64 coordinates, as nfft2d_set_points) and synchronizes; forward/adjoint
 * take host arrays of `count` device pointers and are asynchronous with
 * respect to the host, ordered after prior work on `stream`. */
typedef struct nfft2d_batch_s *nfft2d_batch;
int nfft2d_batch_create(nfft2d_batch *batch, int count, const int *N1, const int *N2, double sigma, int K,
                        void *stream);
/* As nfft2d_batch_create with a window half-width per transform (K[t], 2 to
 * 8; uneven N and K in one batch).  Transforms are grouped internally by K:
 * the gather and the spread run once per distinct K, every other stage
 * once for the whole batch.  All other calls keep the caller's transform
 * order. */
int nfft2d_batch_create_k(nfft2d_batch *batch, int count, const int *N1, const int *N2, const int *K, double sigma,
                          void *stream);
int nfft2d_batch_destroy(nfft2d_batch batch);
int nfft2d_batch_set_points(nfft2d_batch batch, const long long *M, const void *const *x1, const void *const *x2,
                            int coord_dtype, int units);
int nfft2d_batch_forward(nfft2d_batch batch, const void *const *F, void *const *f);
int nfft2d_batch_adjoint(nfft2d_batch batch, const void *const *f, void *const *F);
/* Type 1 with the reference's sign (NFFT2_2D_GPU, NFFT/NFFT2_2D.cu:329-495)
 * for every transform of the batch: the per-particle far-field call of the
 * PSO synthesis (Synthesis/PSO/Synthesis.cu:395) done for all particles at
 * once. */
int nfft2d_batch_spread_ref(nfft2d_batch batch, const void *const *f, void *const *F);
/* The far-field step of the reflectarray PSO synthesis for every particle of
 * the batch at once (Synthesis/PSO/Synthesis.cu:385-405, raFarFieldCalculation
 * around its NFFT2_2D_GPU call; the reference runs it once per particle,
 * PSO.cu:348): per transform t,
 *   X' = X[t] * scale_x,  Y' = Y[t] * scale_y        (FP32, :388-389; the
 *        reference's scales are 2 Nu (pi / a') / (2 pi) and 2 Nv (pi / b') / (2 pi))
 *   far_field[t] = type 1, sign -1, at (X', Y')      (NFFT2_2D_GPU, :395)
 *   far_field[t] .*= filter                          (farFieldFiltering, :402)
 * M points per transform; X, Y: host arrays of `count` device pointers to M
 * floats; excitations: count device pointers to M float2; filter: DEVICE,
 * N1 N2 floats (NULL: none; every transform must then have the same size);
 * far_field: count device pointers to N1 N2 float2.  Binds the points
 * (synchronizes, as nfft2d_batch_set_points), then runs asynchronously on
 * the batch's stream. */
int nfft2d_batch_far_field(nfft2d_batch batch, long long M, const float *const *X, const float *const *Y,
                           float scale_x, float scale_y, const void *const *excitations, const float *filter,
                           void *const *far_field);
int nfft2d_batch_set_graph(nfft2d_batch batch, int on);
/* Waits for the batch's work and reports a latched device-side error once
 * (cleared after it is read), as nfft2d_synchronize does for plans. */
int nfft2d_batch_synchronize(nfft2d_batch batch);
/* Bounded-wait self-test on the batch's stream; the next
 * nfft2d_batch_synchronize returns NFFT2D_ERR_DEVICE_TIMEOUT (once). */
int nfft2d_batch_selftest_wait_timeout(nfft2d_batch batch, int spin_limit);

/* ---- forward transform that allocates nothing ----------------------------
 * No counterpart in the reference: an addition for callers that must not
 * allocate device memory while they run -- a host application that owns all
 * device memory through its own pool (a MATLAB MEX gateway working on
 * gpuArray data, for instance), or a latency-critical loop that cannot afford
 * cudaMalloc's implicit synchronisation.
 *
 * Same result as nfft2d_forward on a plan (N1, N2, sigma = 2, K), computed
 * without a plan: f_p = sum_k F_k exp(-2 pi i (k1 x1_p / N1 + k2 x2_p / N2)).
 * x1, x2: M FP32 coordinates in `units`; F: N1 x N2 complex64; f: M complex64;
 * all device pointers owned by the caller; runs asynchronously on `stream`.
 *
 * Limits: N1, N2 even and <= 128, 2 <= K <= 8; larger grids return
 * NFFT2D_ERR_SCRATCH_LIMIT.  Every work buffer lives in one fixed 1.12 MB
 * device array inside the library (held on each GPU that loads it until the
 * process exits); no cudaMalloc, cudaFree or allocating library call is made.
 * The first call on a device looks up that array's device address
 * (cudaGetSymbolAddress) and caches it for the life of the process, so make
 * it before any stream capture begins; a cudaDeviceReset (or other teardown
 * of the device's primary context) invalidates the cached address, and the
 * entry point must not be called again in that process afterwards.  All
 * calls share the array and it keeps the last call's contents: calls that
 * overlap on the GPU (other streams, other host threads) race and must be
 * serialised by the caller.  The call reads no status back from the GPU: a
 * non-finite coordinate gives NaN for that point's output (no error code),
 * where a plan's set_points would return NFFT2D_ERR_NONFINITE. */
int nfft2d_forward_small_noalloc(int N1, int N2, int K, long long M, const float *x1, const float *x2, int units,
                                 const void *F, void *f, void *stream);

/* ---- Knab-window band-limited regridding ---------------------------------
 * Replaces BP_FBP_FFBP/knabNFFT2D.m:1-79 (with
 * NFFT_Based_Selvas_Approach_for_Signal_Interp_2D.m:4-28, KnabWindow.m:11-47,
 * ConvWindow.m:5-11), the SAR back-projection code's caller of the forward
 * NFFT.  A raster sampled on a rectilinear grid is interpolated to arbitrary
 * output points as a band-limited trigonometric polynomial:
 *
 *   data     Nrows x Ncols complex (float2 / double2 by precision), row-major,
 *            DEVICE; row i sits at cos_in[i], column j at rho_in[j]
 *            (INPUT_DATA with COSALPHA_IN(:,1) and RHO_IN(1,:));
 *   rho_in   Ncols reals, cos_in  Nrows reals: the raster axes, HOST arrays;
 *            T1 = mean(diff(rho_in)), T2 = mean(diff(cos_in));
 *   B1, B2   bilateral bandwidths of the signal along rho and cos alpha
 *            (0 < B < 1/T);
 *   rho_out, cos_out  len1 x len2 output coordinates, row-major, DEVICE;
 *   out      len1 x len2 complex, DEVICE.
 *
 * As in the reference: the Knab windows use P = 18; the oversampling factors
 * a, b >= 2 are detected from the output points' extent (knabNFFT2D.m:34-60);
 * the interpolation is a type-2 NFFT with sign +1 (sigma = 2, K = 6) on the
 * (b Nrows) x (a Ncols) zero-padded windowed spectrum; output columns whose
 * rho_out[0][j] and rows whose cos_out[i][0] lie outside the input axes get
 * the extrapolation value (:75-78).  Returns NFFT2D_ERR_INVALID_ARG where
 * the reference's NFFT1_2D cannot run (odd b Nrows or a Ncols). */
typedef struct nfft2d_knab_s *nfft2d_knab;

typedef struct {
    int Nrows, Ncols;      /* raster                                              */
    int kgn, kgm;          /* window half-lengths along rho / cos alpha           */
    double T1, T2;         /* mean input spacings                                 */
    int a, b;              /* detected oversampling (0 before set_points)         */
    int N1, N2;            /* internal NFFT grid: b*Nrows x a*Ncols               */
    int len1, len2;        /* output raster                                       */
    int masked_lines;      /* output rows + columns set to the extrapolation value */
} nfft2d_knab_info;

/* Host only (no GPU): the Knab window of KnabWindow.m, G[0 .. 2kg] over
 * frequencies -kg .. kg.  With G = NULL only *kg is returned; otherwise
 * G_len must be >= 2*kg + 1. */
int nfft2d_knab_window(double T, double B, int P, int N, double *G, int G_len, int *kg);

int nfft2d_knab_create(nfft2d_knab *knab, int Nrows, int Ncols, const double *rho_in, const double *cos_in,
                       double B1, double B2, int precision, void *stream);
int nfft2d_knab_destroy(nfft2d_knab knab);
/* Bind the output points (FP32 or FP64 coordinates): reads their extents
 * back (synchronizes) and enqueues their binning on the regridder's stream,
 * whose errors nfft2d_knab_synchronize reports. */
int nfft2d_knab_set_points(nfft2d_knab knab, int len1, int len2, const void *rho_out, const void *cos_out,
                           int coord_dtype);
/* Asynchronous on the stream given at creation. */
int nfft2d_knab_execute(nfft2d_knab knab, double extrap_re, double extrap_im, const void *data, void *out);
int nfft2d_knab_get_info(nfft2d_knab knab, nfft2d_knab_info *info);
int nfft2d_knab_synchronize(nfft2d_knab knab);
/* The internal NFFT plan (for nfft2d_enable_timing / nfft2d_get_timings);
 * NULL before set_points.  Owned by the regridder. */
nfft2d_plan nfft2d_knab_plan(nfft2d_knab knab);
/* The whole knabNFFT2D call: create, set_points (FP64 coordinates), execute,
 * synchronize, destroy. */
int nfft2d_knab_nfft2d(double extrap_re, double extrap_im, const double *rho_in, int Ncols, const double *cos_in,
                       int Nrows, const void *data, const double *rho_out, const double *cos_out, int len1, int len2,
                       double B1, double B2, int precision, void *out, void *stream);

/* ---- type-3 NUFFT (nonuniform points to nonuniform frequencies) -----------
 * Replaces NUFFT_2D_CPU (NFFT/NFFT3/C/NFFT3_2D_C.h, NFFT3_2D_C.cpp:199-312),
 * same argument order:
 *     F[k] = sum_j f[j] exp(-i (s[k] x[j] + t[k] y[j])),  j < len_in, k < len_out,
 * by Gaussian gridding at the reference's R = 2.2 and Gaussian width for the
 * accuracy eps (0 < eps < 1): a spread onto an Mry x Mrx grid sized from the
 * extents of both point sets, a 2D FFT and a Gaussian gather with the
 * reference's pre- and post-compensation.  x, y, s, t: FP64 DEVICE arrays;
 * f, F: DEVICE complex (float2 for NFFT2D_F32, double2 for NFFT2D_F64; the
 * weights are FP64 either way).  The work grid is allocated per call.
 * Synchronous on `stream`.  NFFT2D_ERR_INVALID_ARG when all x or all y are
 * equal (the reference divides by that extent). */
int nfft2d_nufft3_2d(const double *x, const double *y, const double *s, const double *t, const void *f, void *F,
                     double eps, long long len_in, long long len_out, int precision, void *stream);

/* ---- fast factorized back-projection (FFBP) -------------------------------
 * Replaces the NFFT-interpolated branch of BP_FBP_FFBP/FFBP_POLAR_NFFT.m:1-158
 * (with BP_POLAR_NFFT.m:1-25 and NFFT1_1D.m at the leaves): the SAR image of
 * pulses a..b (0-based, inclusive) at len1 x len2 output points given in the
 * polar frame of antenna a (rho_out: range from antenna a; cos_out: cosine of
 * the angle to the track direction; FFBP.m:10-22 builds them from a Cartesian
 * scene).  The aperture is split in two at floor((a + b) / 2) until at most
 * three pulses remain; each half's image is formed on its own polar raster
 * (sample counts and padded axes as FFBP_POLAR_NFFT.m:58-64), brought to
 * baseband, regridded onto the parent's points by the Knab-window NFFT
 * interpolator (knabNFFT2D, extrapolation NaN) and re-modulated; the two
 * halves are summed.  A leaf back-projects each pulse through a 1D type-2
 * NFFT of its nf frequency samples (sigma 2, K 6).
 *
 *   sar               propagation speed, centre frequency fc, bandwidth and
 *                     maximum frequency f2 (the reference's globals c, fc,
 *                     BW, f2);
 *   ant_x/y/z, r0     np antenna positions and reference ranges, HOST arrays
 *                     (a straight track, as the recursion's polar shift
 *                     assumes);
 *   phdata            np x nf complex (pulse n's samples at phdata[n nf + k],
 *                     the reference's data.phdata column n), DEVICE;
 *   rho_out, cos_out  len1 x len2 FP64, DEVICE;  image: len1 x len2 complex,
 *                     DEVICE.
 * Complex data are float2 for NFFT2D_F32 (coordinates and phases are always
 * FP64) and double2 for NFFT2D_F64.  Synchronous on `stream`.  Returns
 * NFFT2D_ERR_INVALID_ARG where the reference cannot run (a sub-aperture whose
 * range extent gives fewer than two samples, or a regridding its NFFT1_2D
 * cannot take, see nfft2d_knab_set_points). */
typedef struct {
    double c;       /* propagation speed [m/s]         */
    double fc;      /* centre frequency [Hz]           */
    double bw;      /* bandwidth [Hz]                  */
    double f_max;   /* maximum frequency f2 [Hz]       */
} nfft2d_sar;

/* Work done by one nfft2d_ffbp_polar call (stats may be NULL). */
typedef struct {
    int depth;                  /* levels of the recursion below the top       */
    int regrids;                /* Knab regriddings                            */
    int leaves;                 /* leaf back-projections                       */
    long long leaf_points;      /* points of the leaves' 1D NFFTs (per pulse)  */
    long long regrid_points;    /* output points of all regriddings            */
    long long raster_cells;     /* cells of all sub-aperture rasters           */
} nfft2d_ffbp_stats;

int nfft2d_ffbp_polar(const nfft2d_sar *sar, int np, const double *ant_x, const double *ant_y, const double *ant_z,
                      const double *r0, int nf, const void *phdata, int a, int b, int len1, int len2,
                      const double *rho_out, const double *cos_out, int precision, void *image, void *stream,
                      nfft2d_ffbp_stats *stats);

#ifdef __cplusplus
}
#endif

#endif /* NFFT2D_GB300_H */
