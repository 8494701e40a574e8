/*
 * oracle/fft_core.h -- TEST INFRASTRUCTURE (CPU oracle), never the product path.
 *
 * A mixed-radix Stockham autosort FFT used by the oracle tier:
 *   - oracle/fftw_subset.c exposes it through the FFTW 3.3.4 single-precision API
 *     subset that the reference C core calls (src/Imaging/c/wem.c:98-110, 334, 348,
 *     426, 441, 492-497, 504-509), so the reference sources compile unmodified;
 *   - oracle/wem_oracle_impl.h calls it directly (float for the reference-semantics
 *     port, double for the FP64 oracle).
 *
 * FFTW itself (www.fftw.org, version 3.3.4, named by the reference's
 * src/Imaging/c/Makefile.hungabee:5-6) is not vendored in the reference and not
 * installed here. What the reference relies on is FFTW's published contract:
 * unnormalised transforms, forward sign e^{-2 pi i jk/n} (FFTW_FORWARD = -1),
 * backward e^{+2 pi i jk/n}, row-major multi-dimensional layout, r2c producing
 * n/2+1 outputs and c2r consuming them. This file restates that contract with
 * the Stockham decimation-in-time formulation published by Govindaraju et al.,
 * "High performance discrete Fourier transforms on graphics processors"
 * (SC 2008), one pass per radix:
 *     for j in [0, n/R):  k = j mod Ns
 *         v[r] = in[j + r n/R] * W_{Ns R}^{r k}      (r = 0..R-1)
 *         v    = DFT_R(v)
 *         out[(j/Ns) Ns R + k + r Ns] = v[r]
 * with Ns the product of the radices of the earlier passes. Twiddles are
 * computed in double and rounded to the working type.
 *
 * Instantiate by defining FFTC_T (float|double) and FFTC_NAME(x) before
 * including this header; it may be included several times.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifndef FFTC_T
#error "define FFTC_T and FFTC_NAME before including fft_core.h"
#endif

#define FFTC_MAXPASS 40

typedef struct { FFTC_T re, im; } FFTC_NAME(cpx);

typedef struct {
    int n;
    int npass;
    int radix[FFTC_MAXPASS];
    int span[FFTC_MAXPASS];          /* Ns of each pass */
    FFTC_NAME(cpx) *tw[FFTC_MAXPASS]; /* [Ns][R-1] forward twiddles W^{r k} */
    FFTC_NAME(cpx) *root[FFTC_MAXPASS]; /* generic radix: W_R^q, q in [0,R) */
} FFTC_NAME(plan);

static int FFTC_NAME(factor)(int n, int *radix)
{
    int np = 0;
    while (n % 4 == 0) { radix[np++] = 4; n /= 4; }
    while (n % 2 == 0) { radix[np++] = 2; n /= 2; }
    while (n % 3 == 0) { radix[np++] = 3; n /= 3; }
    while (n % 5 == 0) { radix[np++] = 5; n /= 5; }
    for (int f = 7; n > 1; f += 2) {
        while (n % f == 0) { radix[np++] = f; n /= f; }
        if (f * f > n && n > 1) { radix[np++] = n; n = 1; }
    }
    return np;
}

static FFTC_NAME(plan) *FFTC_NAME(plan_create)(int n)
{
    FFTC_NAME(plan) *p = (FFTC_NAME(plan) *)calloc(1, sizeof(*p));
    if (!p) return NULL;
    p->n = n;
    p->npass = (n > 1) ? FFTC_NAME(factor)(n, p->radix) : 0;
    int ns = 1;
    const double two_pi = 6.283185307179586476925286766559;
    for (int ip = 0; ip < p->npass; ip++) {
        int R = p->radix[ip];
        p->span[ip] = ns;
        p->tw[ip] = (FFTC_NAME(cpx) *)malloc(sizeof(FFTC_NAME(cpx)) * (size_t)ns * (size_t)(R > 1 ? R - 1 : 1));
        for (int k = 0; k < ns; k++)
            for (int r = 1; r < R; r++) {
                long long e = ((long long)r * k) % ((long long)ns * R);
                double a = -two_pi * (double)e / ((double)ns * R);
                p->tw[ip][(size_t)k * (R - 1) + (r - 1)].re = (FFTC_T)cos(a);
                p->tw[ip][(size_t)k * (R - 1) + (r - 1)].im = (FFTC_T)sin(a);
            }
        if (R != 2 && R != 3 && R != 4 && R != 5) {
            p->root[ip] = (FFTC_NAME(cpx) *)malloc(sizeof(FFTC_NAME(cpx)) * (size_t)R);
            for (int q = 0; q < R; q++) {
                double a = -two_pi * (double)q / (double)R;
                p->root[ip][q].re = (FFTC_T)cos(a);
                p->root[ip][q].im = (FFTC_T)sin(a);
            }
        }
        ns *= R;
    }
    return p;
}

static void FFTC_NAME(plan_destroy)(FFTC_NAME(plan) *p)
{
    if (!p) return;
    for (int ip = 0; ip < p->npass; ip++) { free(p->tw[ip]); free(p->root[ip]); }
    free(p);
}

/* One Stockham pass. sign = -1 forward, +1 backward (twiddles conjugated). */
static void FFTC_NAME(pass)(const FFTC_NAME(plan) *p, int ip, int sign,
                            const FFTC_NAME(cpx) *restrict in, FFTC_NAME(cpx) *restrict out)
{
    typedef FFTC_NAME(cpx) C;
    const int n = p->n, R = p->radix[ip], ns = p->span[ip], m = n / R;
    const C *tw = p->tw[ip];
    const FFTC_T sg = (FFTC_T)sign; /* multiplies the imaginary part of roots */
    for (int jb = 0; jb < m; jb += ns) {
        C *o = out + (size_t)(jb / ns) * ns * R;
        for (int k = 0; k < ns; k++) {
            const int j = jb + k;
            const C *t = tw + (size_t)k * (R - 1);
            if (R == 4) {
                C a = in[j], b = in[j + m], c = in[j + 2 * m], d = in[j + 3 * m];
                if (k) {
                    FFTC_T w1r = t[0].re, w1i = sg * -t[0].im;
                    FFTC_T w2r = t[1].re, w2i = sg * -t[1].im;
                    FFTC_T w3r = t[2].re, w3i = sg * -t[2].im;
                    /* stored twiddles are forward (sign -1); sg*-im restores them
                       for sign=-1 and conjugates them for sign=+1 */
                    C bb = { b.re * w1r - b.im * w1i, b.re * w1i + b.im * w1r };
                    C cc = { c.re * w2r - c.im * w2i, c.re * w2i + c.im * w2r };
                    C dd = { d.re * w3r - d.im * w3i, d.re * w3i + d.im * w3r };
                    b = bb; c = cc; d = dd;
                }
                C s0 = { a.re + c.re, a.im + c.im }, d0 = { a.re - c.re, a.im - c.im };
                C s1 = { b.re + d.re, b.im + d.im }, d1 = { b.re - d.re, b.im - d.im };
                /* X1 = d0 + sign*i*d1 ; X3 = d0 - sign*i*d1 (forward: sign=-1) */
                C id1 = { -sg * d1.im, sg * d1.re };
                o[k]          = (C){ s0.re + s1.re, s0.im + s1.im };
                o[k + ns]     = (C){ d0.re + id1.re, d0.im + id1.im };
                o[k + 2 * ns] = (C){ s0.re - s1.re, s0.im - s1.im };
                o[k + 3 * ns] = (C){ d0.re - id1.re, d0.im - id1.im };
            } else if (R == 2) {
                C a = in[j], b = in[j + m];
                if (k) {
                    FFTC_T wr = t[0].re, wi = sg * -t[0].im;
                    C bb = { b.re * wr - b.im * wi, b.re * wi + b.im * wr };
                    b = bb;
                }
                o[k]      = (C){ a.re + b.re, a.im + b.im };
                o[k + ns] = (C){ a.re - b.re, a.im - b.im };
            } else if (R == 3) {
                C v[3] = { in[j], in[j + m], in[j + 2 * m] };
                if (k)
                    for (int r = 1; r < 3; r++) {
                        FFTC_T wr = t[r - 1].re, wi = sg * -t[r - 1].im;
                        C x = { v[r].re * wr - v[r].im * wi, v[r].re * wi + v[r].im * wr };
                        v[r] = x;
                    }
                const FFTC_T c3 = (FFTC_T)-0.5, s3 = (FFTC_T)(0.86602540378443864676 * sign);
                C s = { v[1].re + v[2].re, v[1].im + v[2].im }, df = { v[1].re - v[2].re, v[1].im - v[2].im };
                C mid = { v[0].re + c3 * s.re, v[0].im + c3 * s.im };
                C rot = { -s3 * df.im, s3 * df.re };
                o[k]          = (C){ v[0].re + s.re, v[0].im + s.im };
                o[k + ns]     = (C){ mid.re + rot.re, mid.im + rot.im };
                o[k + 2 * ns] = (C){ mid.re - rot.re, mid.im - rot.im };
            } else if (R == 5) {
                C v[5] = { in[j], in[j + m], in[j + 2 * m], in[j + 3 * m], in[j + 4 * m] };
                if (k)
                    for (int r = 1; r < 5; r++) {
                        FFTC_T wr = t[r - 1].re, wi = sg * -t[r - 1].im;
                        C x = { v[r].re * wr - v[r].im * wi, v[r].re * wi + v[r].im * wr };
                        v[r] = x;
                    }
                const FFTC_T c1 = (FFTC_T)0.30901699437494742410, c2 = (FFTC_T)-0.80901699437494742410;
                const FFTC_T s1 = (FFTC_T)(0.95105651629515357212 * sign), s2 = (FFTC_T)(0.58778525229247312917 * sign);
                C a1 = { v[1].re + v[4].re, v[1].im + v[4].im }, b1 = { v[1].re - v[4].re, v[1].im - v[4].im };
                C a2 = { v[2].re + v[3].re, v[2].im + v[3].im }, b2 = { v[2].re - v[3].re, v[2].im - v[3].im };
                C m1 = { v[0].re + c1 * a1.re + c2 * a2.re, v[0].im + c1 * a1.im + c2 * a2.im };
                C m2 = { v[0].re + c2 * a1.re + c1 * a2.re, v[0].im + c2 * a1.im + c1 * a2.im };
                /* i*(s1*b1 + s2*b2) and i*(s2*b1 - s1*b2) */
                C r1 = { -(s1 * b1.im + s2 * b2.im), s1 * b1.re + s2 * b2.re };
                C r2 = { -(s2 * b1.im - s1 * b2.im), s2 * b1.re - s1 * b2.re };
                o[k]          = (C){ v[0].re + a1.re + a2.re, v[0].im + a1.im + a2.im };
                o[k + ns]     = (C){ m1.re + r1.re, m1.im + r1.im };
                o[k + 4 * ns] = (C){ m1.re - r1.re, m1.im - r1.im };
                o[k + 2 * ns] = (C){ m2.re + r2.re, m2.im + r2.im };
                o[k + 3 * ns] = (C){ m2.re - r2.re, m2.im - r2.im };
            } else {
                /* generic prime radix: direct DFT of length R */
                C v[64];
                C *vv = v;
                C *heap = NULL;
                if (R > 64) { heap = (C *)malloc(sizeof(C) * (size_t)R); vv = heap; }
                vv[0] = in[j];
                for (int r = 1; r < R; r++) {
                    C x = in[j + (size_t)r * m];
                    if (k) {
                        FFTC_T wr = t[r - 1].re, wi = sg * -t[r - 1].im;
                        C y = { x.re * wr - x.im * wi, x.re * wi + x.im * wr };
                        x = y;
                    }
                    vv[r] = x;
                }
                const C *rt = p->root[ip];
                for (int q = 0; q < R; q++) {
                    FFTC_T sr = 0, si = 0;
                    for (int r = 0; r < R; r++) {
                        int e = (int)(((long long)r * q) % R);
                        FFTC_T wr = rt[e].re, wi = sg * -rt[e].im;
                        sr += vv[r].re * wr - vv[r].im * wi;
                        si += vv[r].re * wi + vv[r].im * wr;
                    }
                    o[k + (size_t)q * ns] = (C){ sr, si };
                }
                free(heap);
            }
        }
    }
}

/* Unnormalised 1-D transform of data[0..n) in place; work holds n entries. */
static void FFTC_NAME(exec)(const FFTC_NAME(plan) *p, int sign, FFTC_NAME(cpx) *data,
                            FFTC_NAME(cpx) *work)
{
    FFTC_NAME(cpx) *cur = data, *dst = work;
    for (int ip = 0; ip < p->npass; ip++) {
        FFTC_NAME(pass)(p, ip, sign, cur, dst);
        FFTC_NAME(cpx) *t = cur; cur = dst; dst = t;
    }
    if (cur != data) memcpy(data, cur, sizeof(*data) * (size_t)p->n);
}
