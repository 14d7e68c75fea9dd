/*
 * nfft2d_oracle.c -- CPU restatement of the reference's 2D NFFT path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker, never the product:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline /
 * reference legs load it.  The shipped library (miscellaneous_gb300) never
 * links, loads or calls anything here, and fails loudly when its CUDA
 * extension is missing instead of falling back to this code.
 *
 * Everything is FP64, single source, plain C99 + OpenMP.  Coordinates are in
 * the reference's "grid units": a point x in [-N/2, N/2) spans one period and
 * the phase of frequency k is 2*pi*k*x/N (BP_FBP_FFBP/NFFT1_2D.m:29-30,55,64;
 * NFFT/NFFT2/Matlab/NDFT2_2D.m:14).  Complex arrays are interleaved (re, im)
 * doubles; 2D arrays are row-major with row index <-> first coordinate x1 and
 * N1 (NFFT/NFFT2_2D.cu:23 IDX2R), frequency index k = i - N/2.
 *
 * `sign` selects the exponent: sign = -1 is the reference's own convention
 * (exp(-i...), NFFT1_2D.m:55 fft2, NFFT2_2D.m:63 fft2, NDFT2_2D.m:14);
 * sign = +1 gives the conjugate-exponent transform (the Hermitian adjoint of
 * the forward is type-1 with sign +1).
 *
 * What pins this oracle (no golden vectors ship with the reference; its
 * MATLAB code cannot run here and its CUDA code needs a GPU and headers that
 * are not vendored):
 *   (1) the reference's own acceptance test, Test_NFFT2_2D.m:24-29
 *       (NFFT2_2D vs the NDFT2_2D direct sum, % rel-L2), restated in tests/;
 *   (2) golden fixtures made by an independent numpy transliteration of the
 *       MATLAB files (tests/golden/make_golden.py);
 *   (3) analytic known answers (single point, single frequency, shifts) and
 *       the adjoint identity.
 */
#include <math.h>
#include <float.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_PI 3.141592653589793238462643383279502884

typedef struct { double re, im; } cplx;

static inline cplx cmul(cplx a, cplx b) {
    cplx r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
    return r;
}

int oracle_version(void) { return 3; }

void oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int oracle_get_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* Window pair                                                              */
/* ------------------------------------------------------------------------ */

/* Modified Bessel function I0 by its power series
 *   I0(x) = sum_j ((x/2)^j / j!)^2         (Abramowitz & Stegun 9.6.12).
 * All terms are positive, so the sum is accurate to a few ulp for the
 * arguments used here (|x| <= K*alpha < 60).  Replaces besseli(0, .) of
 * NFFT1_2D.m:21-22 and bessi0 of NFFT2_2D.cu:67. */
double oracle_bessel_i0(double x) {
    const double q = 0.25 * x * x;
    double term = 1.0, sum = 1.0;
    for (int j = 1; j < 500; ++j) {
        term *= q / ((double)j * (double)j);
        sum += term;
        if (term < 1e-18 * sum) break;
    }
    return sum;
}

/* alfa = (2 - 1/c)*pi - 0.01 : NFFT1_2D.m:11, NFFT2_2D.m:8, NFFT2_2D.cu:27. */
double oracle_kb_alpha(double c) { return (2.0 - 1.0 / c) * OR_PI - 0.01; }

/* Spatial (interpolation) window, NFFT1_2D.m:34-36 / NFFT2_2D.m:19-21 /
 * NFFT2_2D.cu:112-116:
 *   phi_hat(t) = (1/pi) sinh(alpha*sqrt(K^2-t^2)) / sqrt(K^2-t^2),
 * continued analytically as (1/pi) sin(alpha*sqrt(t^2-K^2))/sqrt(t^2-K^2)
 * for |t| > K, and alpha/pi at |t| = K. */
double oracle_phi_hat(double t, int K, double alpha) {
    const double P = (double)K * K - t * t;
    if (P > 0) {
        const double s = sqrt(P);
        return sinh(alpha * s) / (OR_PI * s);
    } else if (P < 0) {
        const double s = sqrt(-P);
        return sin(alpha * s) / (OR_PI * s);
    }
    return alpha / OR_PI;
}

/* d phi_hat / dt.  g(P) = sinh(alpha*sqrt(P))/sqrt(P) = sum_n alpha^(2n+1) P^n/(2n+1)!
 * is entire in P = K^2 - t^2, so d phi_hat/dt = -(2t/pi) g'(P).  Near P = 0
 * the series is used; elsewhere the closed forms of both branches. */
double oracle_phi_hat_deriv(double t, int K, double alpha) {
    const double P = (double)K * K - t * t;
    if (fabs(alpha * alpha * P) < 1.0) {
        /* g'(P) = sum_{n>=1} n alpha^(2n+1) P^(n-1) / (2n+1)! */
        double gp = 0.0;
        double a2 = alpha * alpha;
        double term = alpha * a2 / 6.0; /* n = 1: alpha^3 / 3! */
        for (int n = 1; n < 30; ++n) {
            gp += (double)n * term;
            term *= a2 * P / ((2.0 * n + 2.0) * (2.0 * n + 3.0));
        }
        return -2.0 * t * gp / OR_PI;
    }
    if (P > 0) {
        const double s = sqrt(P), as = alpha * s;
        /* d/ds [sinh(as)/s] = (as cosh(as) - sinh(as))/s^2 ; ds/dt = -t/s */
        return ((as * cosh(as) - sinh(as)) / (s * s)) * (-t / s) / OR_PI;
    } else {
        const double s = sqrt(-P), as = alpha * s;
        /* d/ds [sin(as)/s] = (as cos(as) - sin(as))/s^2 ; ds/dt = t/s */
        return ((as * cos(as) - sin(as)) / (s * s)) * (t / s) / OR_PI;
    }
}

/* Spectral (deapodization) window phi(xi) = I0(K sqrt(alpha^2 - xi^2)),
 * NFFT1_2D.m:19-22, NFFT2_2D.m:33-39, NFFT2_2D.cu:66-67. */
double oracle_phi(double xi, int K, double alpha) {
    return oracle_bessel_i0((double)K * sqrt(alpha * alpha - xi * xi));
}

/* MATLAB round(): half away from zero (NFFT1_2D.m:29-30, NFFT2_2D.m:14-15). */
static inline double matlab_round(double v) { return v < 0 ? -floor(-v + 0.5) : floor(v + 0.5); }

static inline long pos_mod(long a, long n) {
    long r = a % n;
    return r < 0 ? r + n : r;
}

/* ------------------------------------------------------------------------ */
/* FFT (own code: iterative radix-2 for powers of two, exact-twiddle direct   */
/* DFT otherwise).  sign = -1 is MATLAB fft; sign = +1 the unnormalised       */
/* inverse.                                                                   */
/* ------------------------------------------------------------------------ */

static int is_pow2(long n) { return n > 0 && (n & (n - 1)) == 0; }

/* twiddle table w[j] = exp(sign*2*pi*i*j/n), j < n, angle reduced exactly. */
static cplx *make_twiddles(long n, int sign) {
    cplx *w = (cplx *)malloc(sizeof(cplx) * (size_t)n);
    for (long j = 0; j < n; ++j) {
        const double ang = 2.0 * OR_PI * (double)j / (double)n;
        w[j].re = cos(ang);
        w[j].im = sign * sin(ang);
    }
    return w;
}

static void fft1d_pow2(cplx *a, long n, const cplx *w) {
    /* bit reversal */
    for (long i = 1, j = 0; i < n; ++i) {
        long bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) { cplx t = a[i]; a[i] = a[j]; a[j] = t; }
    }
    for (long len = 2; len <= n; len <<= 1) {
        const long half = len >> 1, step = n / len;
        for (long i = 0; i < n; i += len) {
            for (long k = 0; k < half; ++k) {
                cplx u = a[i + k];
                cplx v = cmul(a[i + k + half], w[k * step]);
                a[i + k].re = u.re + v.re; a[i + k].im = u.im + v.im;
                a[i + k + half].re = u.re - v.re; a[i + k + half].im = u.im - v.im;
            }
        }
    }
}

static void dft1d_direct(cplx *a, long n, const cplx *w, cplx *tmp) {
    for (long k = 0; k < n; ++k) {
        double sr = 0, si = 0;
        for (long j = 0; j < n; ++j) {
            const cplx t = w[(k * j) % n];
            sr += a[j].re * t.re - a[j].im * t.im;
            si += a[j].re * t.im + a[j].im * t.re;
        }
        tmp[k].re = sr; tmp[k].im = si;
    }
    memcpy(a, tmp, sizeof(cplx) * (size_t)n);
}

static void fft1d(cplx *a, long n, const cplx *w, cplx *tmp) {
    if (is_pow2(n)) fft1d_pow2(a, n, w);
    else dft1d_direct(a, n, w, tmp);
}

/* In-place 2D FFT of an n1 x n2 row-major array (MATLAB fft2 for sign -1). */
void oracle_fft2d(double *data, long n1, long n2, int sign) {
    cplx *a = (cplx *)data;
    cplx *w2 = make_twiddles(n2, sign);
    cplx *w1 = make_twiddles(n1, sign);
#pragma omp parallel
    {
        cplx *tmp = (cplx *)malloc(sizeof(cplx) * (size_t)(n1 > n2 ? n1 : n2));
        cplx *col = (cplx *)malloc(sizeof(cplx) * (size_t)n1);
#pragma omp for schedule(static)
        for (long r = 0; r < n1; ++r) fft1d(a + r * n2, n2, w2, tmp);
#pragma omp for schedule(static)
        for (long c = 0; c < n2; ++c) {
            for (long r = 0; r < n1; ++r) col[r] = a[r * n2 + c];
            fft1d(col, n1, w1, tmp);
            for (long r = 0; r < n1; ++r) a[r * n2 + c] = col[r];
        }
        free(tmp);
        free(col);
    }
    free(w1);
    free(w2);
}

/* ifftshift / fftshift for even sizes: cyclic shift by n/2 in both dims. */
static void half_shift2d(cplx *a, long n1, long n2) {
    const long h1 = n1 / 2, h2 = n2 / 2;
    for (long r = 0; r < h1; ++r) {
        for (long c = 0; c < n2; ++c) {
            const long r2 = r + h1, c2 = (c + h2) % n2;
            cplx t = a[r * n2 + c];
            a[r * n2 + c] = a[r2 * n2 + c2];
            a[r2 * n2 + c2] = t;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Window tables shared by the restated NFFTs                                 */
/* ------------------------------------------------------------------------ */

/* deapodization values phi(2*pi*k/(cN)), k = i - N/2, i < N (NFFT1_2D.m:17-22). */
static double *deapod_table(long N, double c, int K, double alpha) {
    double *t = (double *)malloc(sizeof(double) * (size_t)N);
    for (long i = 0; i < N; ++i) {
        const double xi = 2.0 * OR_PI * (double)(i - N / 2) / (c * (double)N);
        t[i] = oracle_phi(xi, K, alpha);
    }
    return t;
}

static int check_grid(long N, double c, long *n_out) {
    const double cn = c * (double)N;
    const long n = (long)llround(cn);
    if (N <= 0 || (N & 1) || fabs(cn - (double)n) > 1e-9 || (n & 1) || n < N) return -1;
    *n_out = n;
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Restated NFFT1_2D (forward, type 2): BP_FBP_FFBP/NFFT1_2D.m:1-69           */
/* ------------------------------------------------------------------------ */
int oracle_nfft1_2d(const double *F, long N1, long N2, const double *x1, const double *x2, long M,
                    double c, int K, int sign, double *out) {
    long n1, n2;
    if (check_grid(N1, c, &n1) || check_grid(N2, c, &n2) || K < 1) return -1;
    const double alpha = oracle_kb_alpha(c);
    double *phi1 = deapod_table(N1, c, K, alpha); /* :17-23 */
    double *phi2 = deapod_table(N2, c, K, alpha);

    /* STEP 1: scaling and zero padding into the centered c*N grid (:48-49).
     * The MATLAB block (c-1)*N/2+1 : (c+1)*N/2 starts at 0-based n/2 - N/2. */
    cplx *u = (cplx *)calloc((size_t)(n1 * n2), sizeof(cplx));
    const cplx *Fc = (const cplx *)F;
    const long o1 = n1 / 2 - N1 / 2, o2 = n2 / 2 - N2 / 2;
    for (long i = 0; i < N1; ++i)
        for (long j = 0; j < N2; ++j) {
            const double s = 1.0 / (phi1[i] * phi2[j]);
            u[(o1 + i) * n2 + (o2 + j)].re = Fc[i * N2 + j].re * s;
            u[(o1 + i) * n2 + (o2 + j)].im = Fc[i * N2 + j].im * s;
        }

    /* STEP 2: U = fft2(ifftshift(u)) (:55). */
    half_shift2d(u, n1, n2);
    oracle_fft2d((double *)u, n1, n2, sign);

    /* STEP 3: per point, (2K+1)^2 windowed gather (:29-42, :61-67). */
    cplx *o = (cplx *)out;
    const int W = 2 * K + 1;
#pragma omp parallel
    {
        double *ph1 = (double *)malloc(sizeof(double) * W);
        double *ph2 = (double *)malloc(sizeof(double) * W);
#pragma omp for schedule(static)
        for (long l = 0; l < M; ++l) {
            const double mu1 = matlab_round(c * x1[l]), mu2 = matlab_round(c * x2[l]);
            for (int m = -K; m <= K; ++m) {
                ph1[m + K] = oracle_phi_hat(c * x1[l] - (mu1 + m), K, alpha);
                ph2[m + K] = oracle_phi_hat(c * x2[l] - (mu2 + m), K, alpha);
            }
            double sr = 0, si = 0;
            for (int m1 = -K; m1 <= K; ++m1) {
                const long r = pos_mod((long)mu1 + m1, n1);
                double rr = 0, ri = 0;
                for (int m2 = -K; m2 <= K; ++m2) {
                    const long cc = pos_mod((long)mu2 + m2, n2);
                    rr += ph2[m2 + K] * u[r * n2 + cc].re;
                    ri += ph2[m2 + K] * u[r * n2 + cc].im;
                }
                sr += ph1[m1 + K] * rr;
                si += ph1[m1 + K] * ri;
            }
            o[l].re = sr;
            o[l].im = si;
        }
        free(ph1);
        free(ph2);
    }
    free(u);
    free(phi1);
    free(phi2);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Restated NFFT1_1D (forward, type 2, one dimension): BP_FBP_FFBP/NFFT1_1D.m */
/* ------------------------------------------------------------------------ */
/* result_l = sum_k data_k exp(sign 2 pi i k x_l / N), k = -N/2 .. N/2-1, x in
 * grid units.  Both windows of NFFT1_1D.m are divided by I0(K alpha)
 * (:16,:30); the factor cancels and is left out. */
int oracle_nfft1_1d(const double *data, long N, const double *x, long M, double c, int K, int sign, double *out) {
    long n;
    if (check_grid(N, c, &n) || K < 1) return -1;
    const double alpha = oracle_kb_alpha(c);
    double *phi = deapod_table(N, c, K, alpha); /* :14-16 */
    /* STEP 1 (:36-37): data ./ phi into the centered block of u */
    cplx *u = (cplx *)calloc((size_t)n, sizeof(cplx));
    const cplx *d = (const cplx *)data;
    const long o = n / 2 - N / 2;
    for (long i = 0; i < N; ++i) {
        u[o + i].re = d[i].re / phi[i];
        u[o + i].im = d[i].im / phi[i];
    }
    /* STEP 2 (:43): U = fft(ifftshift(u)); for even n ifftshift swaps halves */
    cplx *U = (cplx *)malloc(sizeof(cplx) * (size_t)n);
    for (long k = 0; k < n; ++k) U[k] = u[(k + n / 2) % n];
    oracle_fft2d((double *)U, 1, n, sign);
    /* STEP 3 (:22-30, :49-50): (2K+1)-tap windowed gather */
    cplx *res = (cplx *)out;
#pragma omp parallel for schedule(static)
    for (long l = 0; l < M; ++l) {
        const double mu = matlab_round(c * x[l]);
        double sr = 0, si = 0;
        for (int m = -K; m <= K; ++m) {
            const double w = oracle_phi_hat(c * x[l] - (mu + m), K, alpha);
            const long r = pos_mod((long)mu + m, n);
            sr += w * U[r].re;
            si += w * U[r].im;
        }
        res[l].re = sr;
        res[l].im = si;
    }
    free(U);
    free(u);
    free(phi);
    return 0;
}

/* Derivative of the restated forward w.r.t. the point coordinates (grid
 * units): d f / d x1 = c * sum phi_hat'(c x1 - n1) phi_hat(c x2 - n2) U[n].
 * Same steps 1-2 as oracle_nfft1_2d; step 3 uses the window derivative. */
int oracle_nfft1_2d_grad(const double *F, long N1, long N2, const double *x1, const double *x2, long M,
                         double c, int K, int sign, double *dfdx1, double *dfdx2) {
    long n1, n2;
    if (check_grid(N1, c, &n1) || check_grid(N2, c, &n2) || K < 1) return -1;
    const double alpha = oracle_kb_alpha(c);
    double *phi1 = deapod_table(N1, c, K, alpha);
    double *phi2 = deapod_table(N2, c, K, alpha);
    cplx *u = (cplx *)calloc((size_t)(n1 * n2), sizeof(cplx));
    const cplx *Fc = (const cplx *)F;
    const long o1 = n1 / 2 - N1 / 2, o2 = n2 / 2 - N2 / 2;
    for (long i = 0; i < N1; ++i)
        for (long j = 0; j < N2; ++j) {
            const double s = 1.0 / (phi1[i] * phi2[j]);
            u[(o1 + i) * n2 + (o2 + j)].re = Fc[i * N2 + j].re * s;
            u[(o1 + i) * n2 + (o2 + j)].im = Fc[i * N2 + j].im * s;
        }
    half_shift2d(u, n1, n2);
    oracle_fft2d((double *)u, n1, n2, sign);
    cplx *g1 = (cplx *)dfdx1, *g2 = (cplx *)dfdx2;
    const int W = 2 * K + 1;
#pragma omp parallel
    {
        double *ph1 = (double *)malloc(sizeof(double) * W), *dp1 = (double *)malloc(sizeof(double) * W);
        double *ph2 = (double *)malloc(sizeof(double) * W), *dp2 = (double *)malloc(sizeof(double) * W);
#pragma omp for schedule(static)
        for (long l = 0; l < M; ++l) {
            const double mu1 = matlab_round(c * x1[l]), mu2 = matlab_round(c * x2[l]);
            for (int m = -K; m <= K; ++m) {
                const double t1 = c * x1[l] - (mu1 + m), t2 = c * x2[l] - (mu2 + m);
                ph1[m + K] = oracle_phi_hat(t1, K, alpha);
                ph2[m + K] = oracle_phi_hat(t2, K, alpha);
                dp1[m + K] = oracle_phi_hat_deriv(t1, K, alpha);
                dp2[m + K] = oracle_phi_hat_deriv(t2, K, alpha);
            }
            double ar = 0, ai = 0, br = 0, bi = 0;
            for (int m1 = -K; m1 <= K; ++m1) {
                const long r = pos_mod((long)mu1 + m1, n1);
                double rr = 0, ri = 0, dr = 0, di = 0;
                for (int m2 = -K; m2 <= K; ++m2) {
                    const cplx v = u[r * n2 + pos_mod((long)mu2 + m2, n2)];
                    rr += ph2[m2 + K] * v.re; ri += ph2[m2 + K] * v.im;
                    dr += dp2[m2 + K] * v.re; di += dp2[m2 + K] * v.im;
                }
                ar += dp1[m1 + K] * rr; ai += dp1[m1 + K] * ri;
                br += ph1[m1 + K] * dr; bi += ph1[m1 + K] * di;
            }
            g1[l].re = c * ar; g1[l].im = c * ai;
            g2[l].re = c * br; g2[l].im = c * bi;
        }
        free(ph1); free(dp1); free(ph2); free(dp2);
    }
    free(u);
    free(phi1);
    free(phi2);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Restated NFFT2_2D (spreading, type 1): NFFT/NFFT2/Matlab/NFFT2_2D.m:1-72,  */
/* same steps as NFFT/NFFT2_2D.cu:329-411 (scatter, fftshift/fft/fftshift,    */
/* crop + scale).  Output N1 x N2, row i <-> k1 = i - N1/2.                   */
/* ------------------------------------------------------------------------ */
int oracle_nfft2_2d(const double *d, const double *x1, const double *x2, long M, long N1, long N2,
                    double c, int K, int sign, double *out) {
    long n1, n2;
    if (check_grid(N1, c, &n1) || check_grid(N2, c, &n2) || K < 1) return -1;
    const double alpha = oracle_kb_alpha(c);
    const cplx *dc = (const cplx *)d;
    const int W = 2 * K + 1;
    int nthreads = oracle_get_threads();
    /* STEP 1 (:47-56): scatter into the centered grid; every thread owns a
     * private grid, summed afterwards (order-independent up to rounding). */
    cplx **grids = (cplx **)calloc((size_t)nthreads, sizeof(cplx *));
#pragma omp parallel num_threads(nthreads)
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        cplx *g = (cplx *)calloc((size_t)(n1 * n2), sizeof(cplx));
        grids[tid] = g;
        double *ph1 = (double *)malloc(sizeof(double) * W);
        double *ph2 = (double *)malloc(sizeof(double) * W);
#pragma omp for schedule(static)
        for (long k = 0; k < M; ++k) {
            const double mu1 = matlab_round(c * x1[k]), mu2 = matlab_round(c * x2[k]);
            for (int m = -K; m <= K; ++m) {
                ph1[m + K] = oracle_phi_hat(c * x1[k] - (mu1 + m), K, alpha); /* :14-21 */
                ph2[m + K] = oracle_phi_hat(c * x2[k] - (mu2 + m), K, alpha); /* :23-27 */
            }
            for (int l1 = -K; l1 <= K; ++l1) {
                const long p1 = pos_mod((long)mu1 + l1 + n1 / 2, n1); /* :51 */
                for (int l2 = -K; l2 <= K; ++l2) {
                    const long p2 = pos_mod((long)mu2 + l2 + n2 / 2, n2); /* :52 */
                    const double w = ph1[l1 + K] * ph2[l2 + K];
                    g[p1 * n2 + p2].re += dc[k].re * w; /* :53 */
                    g[p1 * n2 + p2].im += dc[k].im * w;
                }
            }
        }
        free(ph1);
        free(ph2);
    }
    cplx *u = grids[0];
    for (int t = 1; t < nthreads; ++t) {
        if (!grids[t]) continue;
        for (long i = 0; i < n1 * n2; ++i) { u[i].re += grids[t][i].re; u[i].im += grids[t][i].im; }
        free(grids[t]);
    }
    free(grids);
    /* STEP 2 (:63): FFT_Mc = fftshift(fft2(ifftshift(u))). */
    half_shift2d(u, n1, n2);
    oracle_fft2d((double *)u, n1, n2, sign);
    half_shift2d(u, n1, n2);
    /* STEP 3 (:70): crop the center N1 x N2 and divide by PHI1.*PHI2 (:33-41). */
    double *phi1 = deapod_table(N1, c, K, alpha);
    double *phi2 = deapod_table(N2, c, K, alpha);
    cplx *o = (cplx *)out;
    const long o1 = n1 / 2 - N1 / 2, o2 = n2 / 2 - N2 / 2;
    for (long i = 0; i < N1; ++i)
        for (long j = 0; j < N2; ++j) {
            const double s = 1.0 / (phi1[i] * phi2[j]);
            o[i * N2 + j].re = u[(o1 + i) * n2 + (o2 + j)].re * s;
            o[i * N2 + j].im = u[(o1 + i) * n2 + (o2 + j)].im * s;
        }
    free(u);
    free(phi1);
    free(phi2);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Exact direct sums (FP64, exact phase reduction)                            */
/* ------------------------------------------------------------------------ */

/* e[k - kmin] = exp(sign*2*pi*i*k*x/N) for k in [-N/2, N/2).  k*x is exact in
 * FP64 for x carrying <= 41 significant bits (every FP32 input does), /N is
 * exact for power-of-two N, and the fraction is reduced before sincos. */
static void phase_row(double x, long N, int sign, cplx *e) {
    for (long i = 0; i < N; ++i) {
        const double k = (double)(i - N / 2);
        const double r = k * x / (double)N;
        const double f = r - nearbyint(r);
        const double ang = 2.0 * OR_PI * f;
        e[i].re = cos(ang);
        e[i].im = sign * sin(ang);
    }
}

/* out[p] = sum_{i,j} F[i,j] exp(sign*2*pi*i*((i-N1/2) x1_p/N1 + (j-N2/2) x2_p/N2)) */
void oracle_ndft_type2(const double *F, long N1, long N2, const double *x1, const double *x2, long M,
                       int sign, double *out) {
    const cplx *Fc = (const cplx *)F;
    cplx *o = (cplx *)out;
#pragma omp parallel
    {
        cplx *e1 = (cplx *)malloc(sizeof(cplx) * (size_t)N1);
        cplx *e2 = (cplx *)malloc(sizeof(cplx) * (size_t)N2);
#pragma omp for schedule(dynamic, 16)
        for (long p = 0; p < M; ++p) {
            phase_row(x1[p], N1, sign, e1);
            phase_row(x2[p], N2, sign, e2);
            double sr = 0, si = 0;
            for (long i = 0; i < N1; ++i) {
                double rr = 0, ri = 0;
                const cplx *row = Fc + i * N2;
                for (long j = 0; j < N2; ++j) {
                    rr += row[j].re * e2[j].re - row[j].im * e2[j].im;
                    ri += row[j].re * e2[j].im + row[j].im * e2[j].re;
                }
                sr += rr * e1[i].re - ri * e1[i].im;
                si += rr * e1[i].im + ri * e1[i].re;
            }
            o[p].re = sr;
            o[p].im = si;
        }
        free(e1);
        free(e2);
    }
}

/* d out[p] / d x1_p and d out[p] / d x2_p of oracle_ndft_type2 (grid units). */
void oracle_ndft_type2_grad(const double *F, long N1, long N2, const double *x1, const double *x2, long M,
                            int sign, double *dfdx1, double *dfdx2) {
    const cplx *Fc = (const cplx *)F;
    cplx *g1 = (cplx *)dfdx1, *g2 = (cplx *)dfdx2;
#pragma omp parallel
    {
        cplx *e1 = (cplx *)malloc(sizeof(cplx) * (size_t)N1);
        cplx *e2 = (cplx *)malloc(sizeof(cplx) * (size_t)N2);
#pragma omp for schedule(dynamic, 16)
        for (long p = 0; p < M; ++p) {
            phase_row(x1[p], N1, sign, e1);
            phase_row(x2[p], N2, sign, e2);
            double ar = 0, ai = 0, br = 0, bi = 0;
            for (long i = 0; i < N1; ++i) {
                const cplx *row = Fc + i * N2;
                double rr = 0, ri = 0, kr = 0, ki = 0;
                for (long j = 0; j < N2; ++j) {
                    const double vr = row[j].re * e2[j].re - row[j].im * e2[j].im;
                    const double vi = row[j].re * e2[j].im + row[j].im * e2[j].re;
                    const double k2 = (double)(j - N2 / 2);
                    rr += vr; ri += vi;
                    kr += k2 * vr; ki += k2 * vi;
                }
                const double k1 = (double)(i - N1 / 2);
                /* term for d/dx1: k1 * e1 * rowsum ; d/dx2: e1 * k-weighted rowsum */
                ar += k1 * (rr * e1[i].re - ri * e1[i].im);
                ai += k1 * (rr * e1[i].im + ri * e1[i].re);
                br += kr * e1[i].re - ki * e1[i].im;
                bi += kr * e1[i].im + ki * e1[i].re;
            }
            /* multiply by sign*2*pi*i/N */
            const double s1 = sign * 2.0 * OR_PI / (double)N1, s2 = sign * 2.0 * OR_PI / (double)N2;
            g1[p].re = -s1 * ai; g1[p].im = s1 * ar;
            g2[p].re = -s2 * bi; g2[p].im = s2 * br;
        }
        free(e1);
        free(e2);
    }
}

/* out[i,j] = sum_p d_p exp(sign*2*pi*i*((i-N1/2) x1_p/N1 + (j-N2/2) x2_p/N2)) */
void oracle_ndft_type1(const double *d, const double *x1, const double *x2, long M, long N1, long N2,
                       int sign, double *out) {
    const cplx *dc = (const cplx *)d;
    cplx *o = (cplx *)out;
    const long CH = 256;
    cplx *E1 = (cplx *)malloc(sizeof(cplx) * (size_t)(CH * N1));
    cplx *E2 = (cplx *)malloc(sizeof(cplx) * (size_t)(CH * N2));
    memset(out, 0, sizeof(cplx) * (size_t)(N1 * N2));
    for (long p0 = 0; p0 < M; p0 += CH) {
        const long np = (M - p0) < CH ? (M - p0) : CH;
#pragma omp parallel for schedule(static)
        for (long q = 0; q < np; ++q) {
            phase_row(x1[p0 + q], N1, sign, E1 + q * N1);
            phase_row(x2[p0 + q], N2, sign, E2 + q * N2);
            /* fold the data value into the first factor */
            for (long i = 0; i < N1; ++i) E1[q * N1 + i] = cmul(E1[q * N1 + i], dc[p0 + q]);
        }
#pragma omp parallel for schedule(static)
        for (long i = 0; i < N1; ++i) {
            for (long q = 0; q < np; ++q) {
                const cplx a = E1[q * N1 + i];
                const cplx *e2 = E2 + q * N2;
                cplx *row = o + i * N2;
                for (long j = 0; j < N2; ++j) {
                    row[j].re += a.re * e2[j].re - a.im * e2[j].im;
                    row[j].im += a.re * e2[j].im + a.im * e2[j].re;
                }
            }
        }
    }
    free(E1);
    free(E2);
}

/* NDFT2_2D_GPU semantics (NFFT/NDFT2_2D.cu:15-32, 67): arbitrary frequencies
 *   out[q] = sum_p in[p] exp(-2*pi*i*(u_q X_p / Nu + v_q Y_p / Nv)),
 * M points, N frequencies.  Phase reduced to [-1/2, 1/2] turns before sincos. */
void oracle_ndft2_2d_general(const double *X, const double *Y, const double *u, const double *v,
                             const double *in, long Nu, long Nv, long M, long N, double *out) {
    const cplx *ic = (const cplx *)in;
    cplx *o = (cplx *)out;
#pragma omp parallel for schedule(static)
    for (long q = 0; q < N; ++q) {
        double sr = 0, si = 0;
        for (long p = 0; p < M; ++p) {
            const double a = u[q] * X[p] / (double)Nu, b = v[q] * Y[p] / (double)Nv;
            const double f = (a - nearbyint(a)) + (b - nearbyint(b));
            const double ang = -2.0 * OR_PI * (f - nearbyint(f));
            const double cr = cos(ang), ci = sin(ang);
            sr += ic[p].re * cr - ic[p].im * ci;
            si += ic[p].re * ci + ic[p].im * cr;
        }
        o[q].re = sr;
        o[q].im = si;
    }
}

/* ------------------------------------------------------------------------ */
/* Type-3 2D NUFFT (non-uniform to non-uniform)                              */
/* ------------------------------------------------------------------------ */
/* Exact sum F_k = sum_j f_j exp(-i (s_k x_j + t_k y_j)). */
void oracle_ndft3_2d(const double *x, const double *y, const double *f, long M, const double *s, const double *t,
                     long N, double *F) {
    const cplx *fc = (const cplx *)f;
    cplx *o = (cplx *)F;
#pragma omp parallel for schedule(static)
    for (long k = 0; k < N; ++k) {
        double sr = 0, si = 0;
        for (long j = 0; j < M; ++j) {
            const double ang = -(s[k] * x[j] + t[k] * y[j]);
            const double cr = cos(ang), ci = sin(ang);
            sr += fc[j].re * cr - fc[j].im * ci;
            si += fc[j].re * ci + fc[j].im * cr;
        }
        o[k].re = sr;
        o[k].im = si;
    }
}

static double minmax_d(const double *v, long n, int want_max) {
    double m = want_max ? -FLT_MAX : FLT_MAX; /* the reductions' initial values (:214-232) */
    for (long i = 0; i < n; ++i) m = want_max ? (v[i] > m ? v[i] : m) : (v[i] < m ? v[i] : m);
    return m;
}

/* Restated NUFFT_2D_CPU (NFFT/NFFT3/C/NFFT3_2D_C.cpp:199-312) with its
 * gridding (:38-85), shifts (:135-151) and spectral gridding with
 * compensation (:156-194): Gaussian gridding at R = 2.2 for accuracy eps.
 * R is a parameter (the C++ uses 2.2).  info (may be NULL) receives
 * Mrx, Mry, msp.  Returns 0, or -1 for a degenerate input extent. */
int oracle_nufft3_2d(const double *x_in, const double *y_in, const double *f, long len_in, const double *s_in,
                     const double *t_in, long len_out, double eps, double R, double *F, long *info) {
    double Max_x = minmax_d(x_in, len_in, 1), min_x = minmax_d(x_in, len_in, 0);
    double xb = (Max_x + min_x) / 2, X1 = fabs(Max_x - xb);
    double Max_y = minmax_d(y_in, len_in, 1), min_y = minmax_d(y_in, len_in, 0);
    double yb = (Max_y + min_y) / 2, Y1 = fabs(Max_y - yb);
    double Max_s = minmax_d(s_in, len_out, 1), min_s = minmax_d(s_in, len_out, 0);
    double sb = (Max_s + min_s) / 2, S = fabs(Max_s - sb);
    double Max_t = minmax_d(t_in, len_out, 1), min_t = minmax_d(t_in, len_out, 0);
    double tb = (Max_t + min_t) / 2, T = fabs(Max_t - tb);
    if (!(X1 > 0) || !(Y1 > 0)) return -1;
    double msp = 2 + 2 * (R * R) * (-log(eps / 76)) / (OR_PI * (R * R - 2)); /* :235 */
    const long Mrx = 2 * (long)ceil((X1 * S / OR_PI) * R * R + R * msp);  /* :237-238 */
    const long Mry = 2 * (long)ceil((Y1 * T / OR_PI) * R * R + R * msp);
    const double Dx = 2 * OR_PI / (double)Mrx, Ds = 1, Dy = 2 * OR_PI / (double)Mry, Dt = 1; /* :240-241 */
    const double kk_x = X1 / (OR_PI / 2), kk_y = Y1 / (OR_PI / 2);                            /* :243 */
    double *x = (double *)malloc(sizeof(double) * (size_t)len_in), *y = (double *)malloc(sizeof(double) * (size_t)len_in);
    double *s = (double *)malloc(sizeof(double) * (size_t)len_out), *t = (double *)malloc(sizeof(double) * (size_t)len_out);
    for (long i = 0; i < len_in; ++i) { x[i] = x_in[i] / kk_x; y[i] = y_in[i] / kk_y; }      /* :245-246 */
    for (long i = 0; i < len_out; ++i) { s[i] = s_in[i] * kk_x; t[i] = t_in[i] * kk_y; }     /* :247-248 */
    Max_x = Max_x / kk_x; min_x = min_x / kk_x; xb = (Max_x + min_x) / 2;                     /* :250-264 */
    Max_s = Max_s * kk_x; min_s = min_s * kk_x; sb = (Max_s + min_s) / 2;
    Max_y = Max_y / kk_y; min_y = min_y / kk_y; yb = (Max_y + min_y) / 2;
    Max_t = Max_t * kk_y; min_t = min_t * kk_y; tb = (Max_t + min_t) / 2;
    const double b = (msp - 2) / (4 * OR_PI), t1 = 1 / (4 * b);                                /* :267 */
    const int ms = (int)floor(msp - 2);
    if (info) { info[0] = Mrx; info[1] = Mry; info[2] = ms; }

    /* STEP 1 (:38-85): pre-phase, Gaussian spread with pre-compensation */
    cplx *ft = (cplx *)calloc((size_t)(Mrx * Mry), sizeof(cplx));
    const cplx *fc = (const cplx *)f;
    const double fact0 = 1. / (4. * OR_PI * b), fact = fact0 * fact0;
    for (long kk = 0; kk < len_in; ++kk) { /* serial: the sum order is fixed */
        const double arg = sb * x[kk] + tb * y[kk];
        const double re = fc[kk].re * cos(arg) + fc[kk].im * sin(arg);
        const double im = fc[kk].im * cos(arg) - fc[kk].re * sin(arg);
        const double x_temp = (x[kk] - xb) / Dx, y_temp = (y[kk] - yb) / Dy;
        const long nn_offset = (long)floor(Mrx / 2 + x_temp), mm_offset = (long)floor(Mry / 2 + y_temp);
        for (int mm = -ms; mm <= ms; ++mm) {
            const long j = mm + mm_offset;
            const double d_n_sj = (double)(j - Mry / 2);
            for (int nn = -ms; nn <= ms; ++nn) {
                const long i = nn + nn_offset;
                const double d_n_si = (double)(i - Mrx / 2);
                const double e = fact * exp(b * (Dy * Dy * d_n_sj * d_n_sj + Dx * Dx * d_n_si * d_n_si) -
                                            t1 * ((x_temp - d_n_si) * (x_temp - d_n_si) + (y_temp - d_n_sj) * (y_temp - d_n_sj)));
                ft[j * Mrx + i].re += re * e;
                ft[j * Mrx + i].im += im * e;
            }
        }
    }
    /* STEP 2 (:283-292): forward 2D FFT of the Mry x Mrx grid */
    oracle_fft2d((double *)ft, Mry, Mrx, -1);
    /* shifts (:135-151): out[(j + Mry/2) % Mry][(i + Mrx/2) % Mrx] = (-1)^(i+j) in[j][i] */
    cplx *Fs = (cplx *)malloc(sizeof(cplx) * (size_t)(Mrx * Mry));
    for (long i = 0; i < Mrx; ++i)
        for (long j = 0; j < Mry; ++j) {
            const long ii = (i + Mrx / 2) % Mrx, jj = (j + Mry / 2) % Mry;
            const double sg = ((i + j) & 1) ? -1.0 : 1.0;
            Fs[jj * Mrx + ii].re = sg * ft[j * Mrx + i].re;
            Fs[jj * Mrx + ii].im = sg * ft[j * Mrx + i].im;
        }
    /* STEP 3 (:156-194): Gaussian gather and post-compensation */
    cplx *o = (cplx *)F;
#pragma omp parallel for schedule(static)
    for (long kk = 0; kk < len_out; ++kk) {
        const long nsn = (long)floor(Mrx / 2 + (s[kk] - sb) / Ds);
        const double difs = (Mrx / 2 + (s[kk] - sb) / Ds) - nsn;
        const long ntn = (long)floor(Mry / 2 + (t[kk] - tb) / Dt);
        const double dift = (Mry / 2 + (t[kk] - tb) / Dt) - ntn;
        double a0 = 0, a1 = 0;
        double tmp1 = Dy * (t[kk] - tb); tmp1 = tmp1 * tmp1;
        double tmp2 = Dx * (s[kk] - sb); tmp2 = tmp2 * tmp2;
        const double comp = exp(b * (tmp1 + tmp2));
        for (long nn = nsn - ms; nn <= nsn + ms; ++nn)
            for (long mm = ntn - ms; mm <= ntn + ms; ++mm) {
                const double n_pi = (double)(mm - ntn), n_pj = (double)(nn - nsn);
                const double e = exp(-t1 * ((dift - n_pi) * (dift - n_pi) + (difs - n_pj) * (difs - n_pj)));
                a0 += Fs[mm * Mrx + nn].re * e;
                a1 += Fs[mm * Mrx + nn].im * e;
            }
        const double arg = (s[kk] - sb) * xb + (t[kk] - tb) * yb;
        o[kk].re = (a0 * cos(arg) + a1 * sin(arg)) * comp;
        o[kk].im = (a1 * cos(arg) - a0 * sin(arg)) * comp;
    }
    free(ft); free(Fs); free(x); free(y); free(s); free(t);
    return 0;
}

/* Literal NDFT2_2D.m:1-16, including its layout (output N x M, column-major
 * in MATLAB; element (r, s) pairs v(r) with the y-term and u(s) with the
 * x-term) and its division of BOTH phase terms by N (:14).  Returned here
 * row-major as out[r * M + s] for r < N (rows) and s < M. */
void oracle_ndft2_2d_matlab(const double *data, const double *x, const double *y, long P, long N, long M,
                            double *out) {
    const cplx *dc = (const cplx *)data;
    cplx *o = (cplx *)out;
    /* vec[q], q = a + M*b (a < M: v index, b < N: u index); reshape(vec, N, M)
     * puts vec[r + N*s] at (r, s). */
    cplx *vec = (cplx *)malloc(sizeof(cplx) * (size_t)(N * M));
#pragma omp parallel for schedule(static)
    for (long q = 0; q < N * M; ++q) {
        const long a = q % M, b = q / M;
        const double U = (double)(b - N / 2), V = (double)(a - M / 2);
        double sr = 0, si = 0;
        for (long p = 0; p < P; ++p) {
            const double ang = -2.0 * OR_PI * (x[p] * U / (double)N + y[p] * V / (double)N);
            sr += dc[p].re * cos(ang) - dc[p].im * sin(ang);
            si += dc[p].re * sin(ang) + dc[p].im * cos(ang);
        }
        vec[q].re = sr;
        vec[q].im = si;
    }
    for (long r = 0; r < N; ++r)
        for (long s = 0; s < M; ++s) o[r * M + s] = vec[r + N * s];
    free(vec);
}

/* ------------------------------------------------------------------------ */
/* Knab-window band-limited regridding (the SAR code's NFFT caller):         */
/*   BP_FBP_FFBP/knabNFFT2D.m:1-79                                          */
/*   BP_FBP_FFBP/NFFT_Based_Selvas_Approach_for_Signal_Interp_2D.m:4-28     */
/*   BP_FBP_FFBP/KnabWindow.m:11-47, ConvWindow.m:5-11,                     */
/*   IntervalIntersection.m:4-22                                            */
/* ------------------------------------------------------------------------ */

/* ConvWindow.m:5-11: W(f) = I0(pi B (T/2) sqrt(1 - (2f/B)^2)) / (B sinc(i B T/2))
 * on |f| < B/2, else 0; MATLAB's sinc(i y) = sinh(pi y) / (pi y). */
double oracle_conv_window(double f, double B, double T) {
    if (!(fabs(f) < B / 2)) return 0.0;
    const double q = 2.0 * f / B;
    const double y = B * T / 2.0;
    const double snc = (y == 0.0) ? 1.0 : sinh(OR_PI * y) / (OR_PI * y);
    return oracle_bessel_i0(OR_PI * B * (T / 2.0) * sqrt(1.0 - q * q)) / (B * snc);
}

/* Adaptive Simpson quadrature with Richardson correction and tolerance
 * halving on subdivision (Lyness 1969; the method of MATLAB's quad, which
 * KnabWindow.m:40 calls with tolerance 1e-12). */
static double simpson_step(double B1, double T, double a, double b, double fa, double fc, double fb, double tol,
                           int depth) {
    const double c = 0.5 * (a + b), h = b - a;
    const double d = 0.5 * (a + c), e = 0.5 * (c + b);
    const double fd = oracle_conv_window(d, B1, T), fe = oracle_conv_window(e, B1, T);
    const double q1 = h / 6.0 * (fa + 4.0 * fc + fb);
    const double q2 = h / 12.0 * (fa + 4.0 * fd + 2.0 * fc + 4.0 * fe + fb);
    const double q = q2 + (q2 - q1) / 15.0;
    if (depth >= 50 || fabs(q2 - q) <= tol || h <= 1e-300) return q;
    return simpson_step(B1, T, a, c, fa, fd, fc, tol / 2, depth + 1) +
           simpson_step(B1, T, c, b, fc, fe, fb, tol / 2, depth + 1);
}

double oracle_conv_window_integral(double lo, double hi, double B1, double T, double tol) {
    if (!(hi > lo)) return 0.0;
    /* three unequal starting panels keep the first estimate off symmetric
     * cancellations */
    const double h = 0.13579 * (hi - lo);
    const double x[7] = {lo, lo + h, lo + 2 * h, 0.5 * (lo + hi), hi - 2 * h, hi - h, hi};
    double y[7];
    for (int i = 0; i < 7; ++i) y[i] = oracle_conv_window(x[i], B1, T);
    return simpson_step(B1, T, x[0], x[2], y[0], y[1], y[2], tol, 0) +
           simpson_step(B1, T, x[2], x[4], y[2], y[3], y[4], tol, 0) +
           simpson_step(B1, T, x[4], x[6], y[4], y[5], y[6], tol, 0);
}

/* KnabWindow.m:11-47.  Returns kg; with G != NULL also fills G[0 .. 2kg]
 * (frequencies -kg .. kg).  The operation order of kg and f(k) follows the
 * MATLAB lines, since kg is a floor() of a quotient. */
long oracle_knab_window(double T, double B, int P, long N, double *G) {
    const double df = 1.0 / ((double)N * T);                       /* :16 */
    const long kg = (long)floor((1.0 / T - B / 2.0) / df);          /* :19 */
    if (!G || kg < 0) return kg;
    const double B0 = 1.0 / T;                                      /* :24 */
    const double B1 = B0 - B;                                       /* :25 */
    const long n = 2 * kg + 1;
    for (long i = 0; i < n; ++i) G[i] = 0.0;                        /* :29 */
    long last = -1;
    for (long k = 0; k <= kg; ++k) {
        const double f = -df * (double)kg + df * (double)k;         /* :22 */
        if (B1 / 2.0 <= f + B0 / 2.0)                               /* :26 */
            G[k] = 1.0;                                             /* :32 */
        else
            last = k;
    }
    for (long k = 0; k <= last; ++k) {                              /* :36 */
        const double f = -df * (double)kg + df * (double)k;
        const double ia0 = -B1 / 2.0, ia1 = B1 / 2.0;               /* IntervalIntersection.m */
        const double ib0 = f - B0 / 2.0, ib1 = f + B0 / 2.0;
        if (ia1 < ib0 || ib1 < ia0) continue;                       /* :6-11 */
        double lo, hi;
        if (ib1 < ia1) {                                            /* :13-18 */
            lo = ia0;
            hi = ib1;
        } else {                                                    /* :20 */
            lo = ib0;
            hi = ia1;
        }
        G[k] = oracle_conv_window_integral(lo, hi, B1, 2.0 * P * T, 1e-12);  /* :34,40 */
    }
    double *g2 = (double *)malloc(sizeof(double) * (size_t)n);
    for (long i = 0; i < n; ++i) g2[i] = G[i] + G[n - 1 - i];      /* :45 */
    g2[kg] -= 1.0;                                                  /* :46 */
    for (long i = 0; i < n; ++i) G[i] = g2[i] / (double)N;          /* :47 */
    free(g2);
    return kg;
}

static double matlab_mean_diff(const double *v, long n) {
    double s = 0.0;
    for (long i = 0; i + 1 < n; ++i) s += v[i + 1] - v[i];
    return s / (double)(n - 1);
}

/* knabNFFT2D.m:1-79 with the interpolation of
 * NFFT_Based_Selvas_Approach_for_Signal_Interp_2D.m:4-28.
 *
 *   rho_in[Ncols], cos_in[Nrows]: the input raster's axes (RHO_IN(1,:),
 *     COSALPHA_IN(:,1));
 *   data: Nrows x Ncols complex, row <-> cos, column <-> rho (INPUT_DATA);
 *   rho_out, cos_out: len1 x len2 (RHO_OUT, COSALPHA_OUT), row-major;
 *   out: len1 x len2 complex.
 *   info (may be NULL): {a, b, kgn, kgm}.
 *   direct != 0 replaces the NFFT1_2D call by the exact direct sum of the
 *   same trigonometric polynomial (to pin the NFFT's approximation).
 * Returns 0, or -1 where the MATLAB code would fail (fewer than 2 x 2
 * samples, an odd NFFT1_2D size, a spectrum wider than the padded grid). */
int oracle_knab_nfft2d(double ev_re, double ev_im, const double *rho_in, long Ncols, const double *cos_in,
                       long Nrows, const double *data, const double *rho_out, const double *cos_out, long len1,
                       long len2, double B1, double B2, int direct, double *out, long *info) {
    if (Nrows < 2 || Ncols < 2 || len1 < 1 || len2 < 1) return -1;  /* :15-20 */
    const double T1 = matlab_mean_diff(rho_in, Ncols);               /* :6 */
    const double T2 = matlab_mean_diff(cos_in, Nrows);               /* :7 */
    const long Mo = len1 * len2;
    /* :23-35 shifted outputs and their extent */
    double mnr = INFINITY, mxr = -INFINITY, mnc = INFINITY, mxc = -INFINITY;
    for (long p = 0; p < Mo; ++p) {
        const double r = rho_out[p] - rho_in[0], c = cos_out[p] - cos_in[0];
        if (r < mnr) mnr = r;
        if (r > mxr) mxr = r;
        if (c < mnc) mnc = c;
        if (c > mxc) mxc = c;
    }
    double Nn = (mxr - mnr) / (T1 * (1.0 - 1.0 / (double)len2));     /* :34 */
    double Mm = (mxc - mnc) / (T2 * (1.0 - 1.0 / (double)len1));     /* :35 */
    if (Nn < 1 || isnan(Nn)) Nn = 1;                                 /* :37-42 */
    if (Mm < 1 || isnan(Mm)) Mm = 1;
    long a = (long)matlab_round((double)len2 / Nn);                  /* :45 */
    long b = (long)matlab_round((double)len1 / Mm);                  /* :46 */
    if (a < 2) a = 2;  /* :48-53; the zero-coordinate points appended there */
    if (b < 2) b = 2;  /* :55-60   are cropped away again at :72            */
    const int P = 18;                                                /* :63 */
    const long kgn = oracle_knab_window(T1, B1, P, Ncols, NULL);     /* :64 */
    const long kgm = oracle_knab_window(T2, B2, P, Nrows, NULL);     /* :65 */
    if (info) {
        info[0] = a;
        info[1] = b;
        info[2] = kgn;
        info[3] = kgm;
    }
    const long NA = Ncols * a, MB = Nrows * b;  /* Interp_2D: N = Ncols, M = Nrows (INPUT_DATA.') */
    if (kgn < 0 || kgm < 0 || (NA & 1) || (MB & 1) || NA / 2 - kgn - 1 < 0 || MB / 2 - kgm - 1 < 0) return -1;
    double *Gn = (double *)malloc(sizeof(double) * (size_t)(2 * kgn + 1));
    double *Gm = (double *)malloc(sizeof(double) * (size_t)(2 * kgm + 1));
    oracle_knab_window(T1, B1, P, Ncols, Gn);
    oracle_knab_window(T2, B2, P, Nrows, Gm);

    /* Interp_2D:9  sF = fft2(INPUT_DATA.'): an Ncols x Nrows array */
    cplx *sF = (cplx *)malloc(sizeof(cplx) * (size_t)(Ncols * Nrows));
    const cplx *dc = (const cplx *)data;
    for (long j = 0; j < Ncols; ++j)
        for (long i = 0; i < Nrows; ++i) sF[j * Nrows + i] = dc[i * Ncols + j];
    oracle_fft2d((double *)sF, Ncols, Nrows, -1);
    /* Interp_2D:10-25: periodic repetition, window, (N a)(M b) factor, and
     * the centered zero padding to NA x MB (even sizes: frequency k at
     * index NA/2 + k) */
    cplx *S = (cplx *)calloc((size_t)(NA * MB), sizeof(cplx));
    const double scale = (double)NA * (double)MB;
    for (long k1 = -kgn; k1 <= kgn; ++k1)
        for (long k2 = -kgm; k2 <= kgm; ++k2) {
            const cplx v = sF[pos_mod(k1, Ncols) * Nrows + pos_mod(k2, Nrows)];
            const double g = Gn[k1 + kgn] * Gm[k2 + kgm] * scale;
            S[(NA / 2 + k1) * MB + (MB / 2 + k2)].re = v.re * g;
            S[(NA / 2 + k1) * MB + (MB / 2 + k2)].im = v.im * g;
        }
    /* Interp_2D:28  sUp = conj(NFFT1_2D(conj(S), rho_s/(T1/a), cos_s/(T2/b))) / (a b N M) */
    double *x1 = (double *)malloc(sizeof(double) * (size_t)Mo);
    double *x2 = (double *)malloc(sizeof(double) * (size_t)Mo);
    for (long p = 0; p < Mo; ++p) {
        x1[p] = (rho_out[p] - rho_in[0]) / (T1 / (double)a);
        x2[p] = (cos_out[p] - cos_in[0]) / (T2 / (double)b);
    }
    for (long q = 0; q < NA * MB; ++q) S[q].im = -S[q].im;
    cplx *o = (cplx *)out;
    if (direct) {
        oracle_ndft_type2((const double *)S, NA, MB, x1, x2, Mo, -1, out);
    } else {
        if (oracle_nfft1_2d((const double *)S, NA, MB, x1, x2, Mo, 2.0, 6, -1, out) != 0) {
            free(Gn), free(Gm), free(sF), free(S), free(x1), free(x2);
            return -1;
        }
    }
    const double inv = 1.0 / ((double)a * (double)b * (double)Ncols * (double)Nrows);
    for (long p = 0; p < Mo; ++p) {
        o[p].re = o[p].re * inv;
        o[p].im = -o[p].im * inv;
    }
    /* :75-78 extrapolation: columns whose RHO_OUT(1, :) and rows whose
     * COSALPHA_OUT(:, 1) lie outside the input axes' range */
    double rmin = INFINITY, rmax = -INFINITY, cmin = INFINITY, cmax = -INFINITY;
    for (long j = 0; j < Ncols; ++j) {
        if (rho_in[j] < rmin) rmin = rho_in[j];
        if (rho_in[j] > rmax) rmax = rho_in[j];
    }
    for (long i = 0; i < Nrows; ++i) {
        if (cos_in[i] < cmin) cmin = cos_in[i];
        if (cos_in[i] > cmax) cmax = cos_in[i];
    }
    for (long j = 0; j < len2; ++j)
        if (rho_out[j] < rmin || rho_out[j] > rmax)
            for (long i = 0; i < len1; ++i) o[i * len2 + j].re = ev_re, o[i * len2 + j].im = ev_im;
    for (long i = 0; i < len1; ++i)
        if (cos_out[i * len2] < cmin || cos_out[i * len2] > cmax)
            for (long j = 0; j < len2; ++j) o[i * len2 + j].re = ev_re, o[i * len2 + j].im = ev_im;
    free(Gn), free(Gm), free(sF), free(S), free(x1), free(x2);
    return 0;
}
