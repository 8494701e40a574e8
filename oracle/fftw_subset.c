/*
 * oracle/fftw_subset.c -- TEST INFRASTRUCTURE (CPU oracle), never the product path.
 *
 * Restates the FFTW 3.3.4 single-precision API subset used by the reference C core
 * (call sites: src/Imaging/c/wem.c:98-110 plan_dft + warm-up execute, :334 :348
 * :426 :441 execute_dft from OpenMP threads, :492-497 r2c, :504-509 c2r) on top of
 * the Stockham FFT in oracle/fft_core.h. Contract kept from FFTW's manual:
 *   - transforms are unnormalised; FFTW_FORWARD = -1 uses e^{-2 pi i jk/n};
 *   - rank-k arrays are row-major (last dimension contiguous);
 *   - fftwf_execute_dft(p, in, out) is re-entrant: it may run concurrently from
 *     several threads on different arrays (it allocates its own work space);
 *   - r2c writes n/2+1 outputs; c2r reads n/2+1 inputs and returns the real part
 *     of the inverse transform of their Hermitian extension (imaginary parts of
 *     the DC and, for even n, Nyquist bins do not contribute), unnormalised.
 * Plans are created from the main thread only (as the reference does).
 */
#include <complex.h>
#include <stdlib.h>
#include <string.h>
#include "fftw3.h"

#define FFTC_T float
#define FFTC_NAME(x) fsub_##x
#include "fft_core.h"
#undef FFTC_T
#undef FFTC_NAME

enum { KIND_DFT = 0, KIND_R2C = 1, KIND_C2R = 2 };

struct oracle_fftwf_plan_s {
    int kind;
    int rank;
    int n[8];
    int sign;
    fsub_plan *axis[8];
    void *in, *out; /* arrays bound at planning time (fftwf_execute) */
};

void *fftwf_malloc(size_t n) { return malloc(n ? n : 1); }
void fftwf_free(void *p) { free(p); }

static fftwf_plan make_plan(int kind, int rank, const int *n, int sign, void *in, void *out)
{
    if (rank < 1 || rank > 8) return NULL;
    fftwf_plan p = (fftwf_plan)calloc(1, sizeof(*p));
    if (!p) return NULL;
    p->kind = kind; p->rank = rank; p->sign = sign; p->in = in; p->out = out;
    for (int d = 0; d < rank; d++) {
        p->n[d] = n[d];
        p->axis[d] = fsub_plan_create(n[d]);
    }
    return p;
}

fftwf_plan fftwf_plan_dft(int rank, const int *n, fftwf_complex *in, fftwf_complex *out,
                          int sign, unsigned flags)
{
    (void)flags;
    return make_plan(KIND_DFT, rank, n, sign, in, out);
}

fftwf_plan fftwf_plan_dft_1d(int n, fftwf_complex *in, fftwf_complex *out, int sign, unsigned flags)
{
    return fftwf_plan_dft(1, &n, in, out, sign, flags);
}

fftwf_plan fftwf_plan_dft_2d(int n0, int n1, fftwf_complex *in, fftwf_complex *out, int sign,
                             unsigned flags)
{
    int n[2] = { n0, n1 };
    return fftwf_plan_dft(2, n, in, out, sign, flags);
}

fftwf_plan fftwf_plan_dft_r2c_1d(int n, float *in, fftwf_complex *out, unsigned flags)
{
    (void)flags;
    return make_plan(KIND_R2C, 1, &n, FFTW_FORWARD, in, out);
}

fftwf_plan fftwf_plan_dft_c2r_1d(int n, fftwf_complex *in, float *out, unsigned flags)
{
    (void)flags;
    return make_plan(KIND_C2R, 1, &n, FFTW_BACKWARD, in, out);
}

void fftwf_destroy_plan(fftwf_plan p)
{
    if (!p) return;
    for (int d = 0; d < p->rank; d++) fsub_plan_destroy(p->axis[d]);
    free(p);
}

/* complex rank-k transform of buf (row-major) in place */
static void exec_dft_inplace(const fftwf_plan p, fsub_cpx *buf)
{
    size_t total = 1;
    int nmax = 1;
    for (int d = 0; d < p->rank; d++) { total *= (size_t)p->n[d]; if (p->n[d] > nmax) nmax = p->n[d]; }
    fsub_cpx *line = (fsub_cpx *)malloc(sizeof(fsub_cpx) * (size_t)nmax);
    fsub_cpx *work = (fsub_cpx *)malloc(sizeof(fsub_cpx) * (size_t)nmax);
    size_t stride = 1;
    for (int d = p->rank - 1; d >= 0; d--) {
        const int nd = p->n[d];
        const size_t outer = total / ((size_t)nd * stride);
        for (size_t o = 0; o < outer; o++)
            for (size_t s = 0; s < stride; s++) {
                fsub_cpx *base = buf + o * (size_t)nd * stride + s;
                if (stride == 1) {
                    fsub_exec(p->axis[d], p->sign, base, work);
                } else {
                    for (int i = 0; i < nd; i++) line[i] = base[(size_t)i * stride];
                    fsub_exec(p->axis[d], p->sign, line, work);
                    for (int i = 0; i < nd; i++) base[(size_t)i * stride] = line[i];
                }
            }
        stride *= (size_t)nd;
    }
    free(line);
    free(work);
}

static void exec_any(const fftwf_plan p, void *in, void *out)
{
    if (p->kind == KIND_DFT) {
        size_t total = 1;
        for (int d = 0; d < p->rank; d++) total *= (size_t)p->n[d];
        if (out != in) memcpy(out, in, sizeof(fsub_cpx) * total);
        exec_dft_inplace(p, (fsub_cpx *)out);
    } else if (p->kind == KIND_R2C) {
        const int n = p->n[0];
        fsub_cpx *buf = (fsub_cpx *)malloc(sizeof(fsub_cpx) * (size_t)n);
        const float *x = (const float *)in;
        for (int i = 0; i < n; i++) { buf[i].re = x[i]; buf[i].im = 0.0f; }
        exec_dft_inplace(p, buf);
        memcpy(out, buf, sizeof(fsub_cpx) * (size_t)(n / 2 + 1));
        free(buf);
    } else {
        const int n = p->n[0], nh = n / 2 + 1;
        fsub_cpx *buf = (fsub_cpx *)malloc(sizeof(fsub_cpx) * (size_t)n);
        const fsub_cpx *X = (const fsub_cpx *)in;
        for (int k = 0; k < nh && k < n; k++) buf[k] = X[k];
        for (int k = nh; k < n; k++) { buf[k].re = X[n - k].re; buf[k].im = -X[n - k].im; }
        buf[0].im = 0.0f;
        if (n % 2 == 0) buf[n / 2].im = 0.0f;
        exec_dft_inplace(p, buf);
        float *y = (float *)out;
        for (int i = 0; i < n; i++) y[i] = buf[i].re;
        free(buf);
    }
}

void fftwf_execute(const fftwf_plan p) { exec_any(p, p->in, p->out); }

void fftwf_execute_dft(const fftwf_plan p, fftwf_complex *in, fftwf_complex *out)
{
    exec_any(p, (void *)in, (void *)out);
}
