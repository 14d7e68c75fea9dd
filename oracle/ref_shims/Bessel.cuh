/*
 * Stand-in for the reference's Bessel.cuh (not shipped; NFFT/NFFT2_2D.cu:6).
 * bessi0(x) = I0(x), the modified Bessel function of the first kind, order
 * 0, by its power series (Abramowitz & Stegun 9.6.12):
 *     I0(x) = sum_k ((x/2)^(2k)) / (k!)^2,
 * summed in FP64 until the term no longer changes the sum, then returned in
 * the caller's type.  TEST INFRASTRUCTURE ONLY.
 */
#ifndef ORACLE_REF_SHIM_BESSEL_CUH
#define ORACLE_REF_SHIM_BESSEL_CUH

template <class T>
__host__ __device__ inline T bessi0(T x)
{
    const double q = 0.25 * (double)x * (double)x;
    double term = 1.0, sum = 1.0;
    for (int k = 1; k < 500; ++k) {
        term *= q / ((double)k * (double)k);
        const double next = sum + term;
        if (next == sum) break;
        sum = next;
    }
    return (T)sum;
}

#endif
