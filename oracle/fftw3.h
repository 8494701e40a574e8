/*
 * oracle/fftw3.h -- TEST INFRASTRUCTURE (CPU oracle), never the product path.
 *
 * Declares the subset of the FFTW 3.3.4 single-precision API that the reference
 * C core uses (src/Imaging/c/wem.c, src/API/c/seismic.h:13), so that those
 * sources compile unmodified against oracle/fftw_subset.c. Names, argument
 * meaning and the sign/flag constants follow FFTW's published interface; the
 * type of fftwf_complex follows FFTW's rule (C99 float _Complex when
 * <complex.h> was included first, float[2] otherwise).
 */
#ifndef ORACLE_FFTW3_SUBSET_H
#define ORACLE_FFTW3_SUBSET_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

#if defined(_Complex_I) && defined(complex) && defined(I)
typedef float _Complex fftwf_complex;
#else
typedef float fftwf_complex[2];
#endif

typedef struct oracle_fftwf_plan_s *fftwf_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_DESTROY_INPUT (1U << 0)
#define FFTW_PRESERVE_INPUT (1U << 4)
#define FFTW_ESTIMATE (1U << 6)

fftwf_plan fftwf_plan_dft(int rank, const int *n, fftwf_complex *in, fftwf_complex *out,
                          int sign, unsigned flags);
fftwf_plan fftwf_plan_dft_1d(int n, fftwf_complex *in, fftwf_complex *out, int sign,
                             unsigned flags);
fftwf_plan fftwf_plan_dft_2d(int n0, int n1, fftwf_complex *in, fftwf_complex *out,
                             int sign, unsigned flags);
fftwf_plan fftwf_plan_dft_r2c_1d(int n, float *in, fftwf_complex *out, unsigned flags);
fftwf_plan fftwf_plan_dft_c2r_1d(int n, fftwf_complex *in, float *out, unsigned flags);
void fftwf_execute(const fftwf_plan p);
void fftwf_execute_dft(const fftwf_plan p, fftwf_complex *in, fftwf_complex *out);
void fftwf_destroy_plan(fftwf_plan p);
void *fftwf_malloc(size_t n);
void fftwf_free(void *p);

#ifdef __cplusplus
}
#endif
#endif
