/*
 * oracle/wem_oracle.c -- TEST INFRASTRUCTURE (CPU oracle), never the product path.
 *
 * Instantiates the restatement in wem_oracle_impl.h twice:
 *   wemo_port_wem  -- the reference's own mixed float/double arithmetic;
 *   wemo_fp64_wem  -- the same operator in double precision.
 * and the FFT of fft_core.h in float (of_*) and double (od_*), plus a few
 * entry points the tests use to check the FFT itself.
 */
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define FFTC_T float
#define FFTC_NAME(x) of_##x
#include "fft_core.h"
#undef FFTC_T
#undef FFTC_NAME

#define FFTC_T double
#define FFTC_NAME(x) od_##x
#include "fft_core.h"
#undef FFTC_T
#undef FFTC_NAME

#define ORC_FP64 0
#include "wem_oracle_impl.h"
#undef ORC_FP64

#define ORC_FP64 1
#include "wem_oracle_impl.h"
#undef ORC_FP64

/* 1-D unnormalised complex FFT of `howmany` contiguous rows of length n (interleaved
   re/im), in place; sign -1 forward. Used by the tests to pin the FFT. */
int wemo_fft_f32(float *data, int n, int howmany, int sign)
{
    if (n < 1 || howmany < 0) return -1;
    of_plan *p = of_plan_create(n);
    of_cpx *work = (of_cpx *)malloc(sizeof(of_cpx) * (size_t)n);
    for (int h = 0; h < howmany; h++) of_exec(p, sign, (of_cpx *)data + (size_t)h * n, work);
    free(work);
    of_plan_destroy(p);
    return 0;
}

int wemo_fft_f64(double *data, int n, int howmany, int sign)
{
    if (n < 1 || howmany < 0) return -1;
    od_plan *p = od_plan_create(n);
    od_cpx *work = (od_cpx *)malloc(sizeof(od_cpx) * (size_t)n);
    for (int h = 0; h < howmany; h++) od_exec(p, sign, (od_cpx *)data + (size_t)h * n, work);
    free(work);
    od_plan_destroy(p);
    return 0;
}

/* OpenMP threads a parallel region of this process gets (the reference's
   omp_thread_count(), wem.c:539-544); tests pass it to the port so both reduce
   their per-thread image slices identically. */
int wemo_omp_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
