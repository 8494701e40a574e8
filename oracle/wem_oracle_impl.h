/*
 * oracle/wem_oracle_impl.h -- TEST INFRASTRUCTURE (CPU oracle), never the product path.
 *
 * CPU restatement of the reference's shot-profile one-way wave-equation
 * migration/demigration operator, src/Imaging/c/wem.c. Included twice by
 * oracle/wem_oracle.c:
 *
 *   ORC_FP64 == 0  "port": the reference's own arithmetic, type by type. FFTs in
 *                  float (FFTW single precision in the reference), wavefields held
 *                  as double _Complex (seismic.h:11 makes `complex` double),
 *                  cexpf/cexp exactly where the reference calls them, image in
 *                  float. Linked against the same FFT as oracle/_ref it agrees
 *                  with the compiled reference bit for bit (checked by
 *                  tests/test_oracle_ref.py). This is the CPU baseline that
 *                  bench.py times where the reference sources are absent.
 *   ORC_FP64 == 1  "fp64": the same operator evaluated in double throughout
 *                  (FFTs, phases, image sums); integer decisions (frequency
 *                  band, source cell, reference-velocity indices) are made with
 *                  the reference's float arithmetic so that both variants apply
 *                  the same operator.
 *
 * Both variants take `interp`:
 *   0 = "ref"    PSPI exactly as the reference: wem.c:450-460 with
 *                linear_interp (wem.c:473-478) returning float, i.e. the real part
 *                of the nearest-lower reference wavefield wherever
 *                vref2 - vref1 > 10, the complex value elsewhere;
 *   1 = "linear" the interpolation the commented line wem.c:476 describes,
 *                y1 + (y2 - y1)(v - vref1)/(vref2 - vref1), in complex arithmetic.
 *
 * Array layouts follow the reference's float** (n1 fastest):
 * vel[ix*nz + iz], m[ix*nz + iz], d[ix*nt + it], ix = imx*nmy + imy.
 */

#if ORC_FP64
#define ORC(x) wemo_fp64_##x
#define FR double            /* FFT working type */
#define FFT_PLAN od_plan
#define FFT_CPX od_cpx
#define FFT_CREATE od_plan_create
#define FFT_DESTROY od_plan_destroy
#define FFT_EXEC od_exec
#define IMG_T double         /* image / data element type */
#define WT double            /* angular frequency type */
#else
#define ORC(x) wemo_port_##x
#define FR float
#define FFT_PLAN of_plan
#define FFT_CPX of_cpx
#define FFT_CREATE of_plan_create
#define FFT_DESTROY of_plan_destroy
#define FFT_EXEC of_exec
#define IMG_T float
#define WT float
#endif

/* everything one (shot, frequency) extrapolation needs; shared read-only by threads */
typedef struct {
    int nmx, nmy, nkx, nky, nz, nref, ntfft, nw, ifmin, ifmax, interp, pspi;
    float oz, dz, gz, sz, dw, dkx, dky;
    const float *vel;      /* [nmx*nmy][nz] */
    float *po;             /* [nz]  */
    float *pd;             /* [nmx*nmy][nz] */
    float *vref;           /* [nref][nz] */
    int *iref1, *iref2;    /* [nmx*nmy][nz] */
#if ORC_FP64
    double *po64, *pd64, *vref64;
    double dkx64, dky64;
#endif
    FFT_PLAN *px, *py;     /* 1-D plans along x and y (2-D transform = rows + columns) */
} ORC(ctx);

/* 2-D (nkx x nky, y fastest) unnormalised transform in place, wem.c:103-104 p1/p2 */
static void ORC(fft2)(const ORC(ctx) *c, int sign, FFT_CPX *a, FFT_CPX *work, FFT_CPX *line)
{
    const int nkx = c->nkx, nky = c->nky;
    if (nky > 1)
        for (int ix = 0; ix < nkx; ix++) FFT_EXEC(c->py, sign, a + (size_t)ix * nky, work);
    if (nkx > 1)
        for (int iy = 0; iy < nky; iy++) {
            for (int ix = 0; ix < nkx; ix++) line[ix] = a[(size_t)ix * nky + iy];
            FFT_EXEC(c->px, sign, line, work);
            for (int ix = 0; ix < nkx; ix++) a[(size_t)ix * nky + iy] = line[ix];
        }
}

/* wavenumber of FFT bin ik, wem.c:336-337 */
static inline float ORC(kfloat)(int ik, int nk, float dk)
{
    if (ik <= (int)nk / 2) return (float)dk * ik;
    return -((float)dk * nk - dk * ik);
}

/* taper, wem.c:546-564 */
static void ORC(taper)(double _Complex *dx, int nmx, int lmx, int nmy, int lmy)
{
    float tmx = 1.f, tmy = 1.f;
    for (int imx = 0; imx < nmx; imx++) {
        if (imx >= 0 && imx < lmx) tmx = expf(-powf(0.015 * ((float)lmx - imx), 2.));
        if (imx >= lmx && imx <= nmx - lmx) tmx = 1.;
        if (imx > nmx - lmx && imx < nmx) tmx = expf(-powf(0.015 * ((float)imx - nmx + lmx), 2.));
        for (int imy = 0; imy < nmy; imy++) {
            if (imy >= 0 && imy < lmy) tmy = expf(-powf(0.015 * ((float)lmy - imy), 2.));
            if (imy >= lmy && imy <= nmy - lmy) tmy = 1.;
            if (imy > nmy - lmy && imy < nmy) tmy = expf(-powf(0.015 * ((float)imy - nmy + lmy), 2.));
            dx[imx * nmy + imy] *= tmx * tmy;
        }
    }
}

/* per-thread scratch for one extrapolation step */
typedef struct {
    FFT_CPX *a, *b, *work, *line;
    double _Complex *dref; /* [n][nref] */
} ORC(scratch);

static inline double _Complex ORC(cmul)(double _Complex x, double _Complex y)
{
    double a = creal(x), b = cimag(x), c = creal(y), d = cimag(y);
    return (a * c - b * d) + I * (a * d + b * c);
}

/*
 * Split-step operator, wem.c:289-378. dz carries the sign (source -dz, receiver +dz);
 * adj selects migration (phase-shift then split-step correction and taper) or
 * modelling (taper and correction first).
 */
static void ORC(ssop)(const ORC(ctx) *c, ORC(scratch) *s, double _Complex *dx, WT w, float dz,
                      int iz, int adj)
{
    const int nmx = c->nmx, nmy = c->nmy, nkx = c->nkx, nky = c->nky;
    const int lmx = nmx > 100 ? 30 : 0, lmy = nmy > 100 ? 30 : 0;
    FFT_CPX *a = s->a;
    const float sqn = sqrtf((float)nkx * nky);
    if (!adj) ORC(taper)(dx, nmx, lmx, nmy, lmy);
    for (int imx = 0; imx < nkx; imx++)
        for (int imy = 0; imy < nky; imy++) {
            FFT_CPX v = { 0, 0 };
            if (imx < nmx && imy < nmy) {
                double _Complex u = dx[imx * nmy + imy];
                if (!adj) {
#if ORC_FP64
                    double th = (double)w * c->pd64[(size_t)(imx * nmy + imy) * c->nz + iz] * dz;
                    u = ORC(cmul)(u, cos(th) + I * sin(th));
#else
                    float th = w * c->pd[(size_t)(imx * nmy + imy) * c->nz + iz] * dz;
                    float sn, cs;
                    sincosf(th, &sn, &cs);
                    u = ORC(cmul)(u, (double)cs + I * (double)sn);
#endif
                }
                v.re = (FR)creal(u);
                v.im = (FR)cimag(u);
            }
            a[(size_t)imx * nky + imy] = v;
        }
    ORC(fft2)(c, -1, a, s->work, s->line);
    for (int ikx = 0; ikx < nkx; ikx++)
        for (int iky = 0; iky < nky; iky++) {
            FFT_CPX *p = &a[(size_t)ikx * nky + iky];
#if ORC_FP64
            double kx = ikx <= nkx / 2 ? (double)ikx * c->dkx64 : -(double)(nkx - ikx) * c->dkx64;
            double ky = iky <= nky / 2 ? (double)iky * c->dky64 : -(double)(nky - iky) * c->dky64;
            double wd = (double)w;
            double sq = wd * wd * c->po64[iz] * c->po64[iz] - kx * kx - ky * ky;
            double Lr, Li;
            if (sq >= 0) { Lr = cos(sqrt(sq) * dz); Li = sin(sqrt(sq) * dz); }
            else { Lr = exp(-0.2 * sqrt(-sq) * fabs((double)dz)); Li = 0; }
            double re = (p->re * Lr - p->im * Li) / (double)nkx / (double)nky;
            double im = (p->re * Li + p->im * Lr) / (double)nkx / (double)nky;
            /* fp64 folds both 1/sqrt(N) factors here */
            p->re = re; p->im = im;
#else
            float kx = ORC(kfloat)(ikx, nkx, c->dkx), ky = ORC(kfloat)(iky, nky, c->dky);
            float sq = (w * w) * (c->po[iz] * c->po[iz]) - (kx * kx) - (ky * ky);
            double Lr, Li;
            if (sq >= 0) { float th = sqrtf(sq) * dz; Lr = cos((double)th); Li = sin((double)th); }
            else { Lr = exp(-0.2 * sqrtf(fabs(sq)) * fabs(dz)); Li = 0.0; }
            double ar = p->re, ai = p->im;
            double re = (ar * Lr - ai * Li) / sqn, im = (ar * Li + ai * Lr) / sqn;
            p->re = (float)re; p->im = (float)im;
#endif
        }
    ORC(fft2)(c, +1, a, s->work, s->line);
    for (int imx = 0; imx < nmx; imx++)
        for (int imy = 0; imy < nmy; imy++) {
            FFT_CPX v = a[(size_t)imx * nky + imy];
#if ORC_FP64
            double _Complex u = v.re + I * v.im;
            if (adj) {
                double th = (double)w * c->pd64[(size_t)(imx * nmy + imy) * c->nz + iz] * dz;
                u = ORC(cmul)(u, cos(th) + I * sin(th));
            }
#else
            double _Complex u = ((double)v.re + I * (double)v.im);
            if (adj) {
                float th = w * c->pd[(size_t)(imx * nmy + imy) * c->nz + iz] * dz;
                float sn, cs;
                sincosf(th, &sn, &cs);
                u = ORC(cmul)(u, (double)cs + I * (double)sn);
            }
            u = creal(u) / sqn + I * (cimag(u) / sqn);
#endif
            dx[imx * nmy + imy] = u;
        }
    (void)sqn;
    if (adj) ORC(taper)(dx, nmx, lmx, nmy, lmy);
}

/* PSPI operator, wem.c:380-471 (adj does not change its arithmetic) */
static void ORC(pspiop)(const ORC(ctx) *c, ORC(scratch) *s, double _Complex *dx, WT w, float dz,
                        int iz)
{
    const int nmx = c->nmx, nmy = c->nmy, nkx = c->nkx, nky = c->nky, nref = c->nref;
    FFT_CPX *a = s->a, *b = s->b;
    const float sqn = sqrtf((float)nkx * nky);
    (void)sqn;
    for (int imx = 0; imx < nkx; imx++)
        for (int imy = 0; imy < nky; imy++) {
            FFT_CPX v = { 0, 0 };
            if (imx < nmx && imy < nmy) {
                v.re = (FR)creal(dx[imx * nmy + imy]);
                v.im = (FR)cimag(dx[imx * nmy + imy]);
            }
            a[(size_t)imx * nky + imy] = v;
        }
    ORC(fft2)(c, -1, a, s->work, s->line);
    for (int iref = 0; iref < nref; iref++) {
        for (int ikx = 0; ikx < nkx; ikx++)
            for (int iky = 0; iky < nky; iky++) {
                const FFT_CPX p = a[(size_t)ikx * nky + iky];
                FFT_CPX *q = &b[(size_t)ikx * nky + iky];
#if ORC_FP64
                double kx = ikx <= nkx / 2 ? (double)ikx * c->dkx64 : -(double)(nkx - ikx) * c->dkx64;
                double ky = iky <= nky / 2 ? (double)iky * c->dky64 : -(double)(nky - iky) * c->dky64;
                double vr = c->vref64[(size_t)iref * c->nz + iz];
                double wd = (double)w;
                double sq = wd * wd / (vr * vr) - kx * kx - ky * ky;
                double Lr, Li;
                if (sq >= 0) { Lr = cos(sqrt(sq) * dz); Li = sin(sqrt(sq) * dz); }
                else { Lr = exp(-0.2 * sqrt(-sq) * fabs((double)dz)); Li = 0; }
                q->re = (p.re * Lr - p.im * Li) / (double)nkx / (double)nky;
                q->im = (p.re * Li + p.im * Lr) / (double)nkx / (double)nky;
#else
                float kx = ORC(kfloat)(ikx, nkx, c->dkx), ky = ORC(kfloat)(iky, nky, c->dky);
                float vr = c->vref[(size_t)iref * c->nz + iz];
                float sq = (w * w) * (1 / (vr * vr)) - (kx * kx) - (ky * ky);
                float Lr, Li;
                if (sq >= 0) { float th = sqrtf(sq) * dz; sincosf(th, &Li, &Lr); }
                else { Lr = expf((float)(-0.2 * sqrtf(fabs(sq)) * fabs(dz))); Li = 0.f; }
                double ar = p.re, ai = p.im;
                double re = (ar * (double)Lr - ai * (double)Li) / sqn;
                double im = (ar * (double)Li + ai * (double)Lr) / sqn;
                q->re = (float)re; q->im = (float)im;
#endif
            }
        ORC(fft2)(c, +1, b, s->work, s->line);
        for (int imx = 0; imx < nmx; imx++)
            for (int imy = 0; imy < nmy; imy++) {
                FFT_CPX v = b[(size_t)imx * nky + imy];
#if ORC_FP64
                s->dref[(size_t)(imx * nmy + imy) * nref + iref] = v.re + I * v.im;
#else
                s->dref[(size_t)(imx * nmy + imy) * nref + iref] = (double)v.re / sqn + I * ((double)v.im / sqn);
#endif
            }
    }
    for (int ix = 0; ix < nmx * nmy; ix++) {
        const int i1 = c->iref1[(size_t)ix * c->nz + iz], i2 = c->iref2[(size_t)ix * c->nz + iz];
        const double _Complex y1 = s->dref[(size_t)ix * nref + i1], y2 = s->dref[(size_t)ix * nref + i2];
#if ORC_FP64
        const double v = c->vel[(size_t)ix * c->nz + iz];
        const double vr1 = c->vref64[(size_t)i1 * c->nz + iz], vr2 = c->vref64[(size_t)i2 * c->nz + iz];
        const float vr1f = c->vref[(size_t)i1 * c->nz + iz], vr2f = c->vref[(size_t)i2 * c->nz + iz];
        if (vr2f - vr1f > 10.0) {
            if (c->interp == 1) dx[ix] = y1 + (y2 - y1) * ((v - vr1) / (vr2 - vr1));
            else dx[ix] = creal(y1);
        } else dx[ix] = y1;
#else
        const float v = c->vel[(size_t)ix * c->nz + iz];
        const float vr1 = c->vref[(size_t)i1 * c->nz + iz], vr2 = c->vref[(size_t)i2 * c->nz + iz];
        if (vr2 - vr1 > 10.0) {
            if (c->interp == 1) dx[ix] = y1 + (y2 - y1) * (double)((v - vr1) / (vr2 - vr1));
            else dx[ix] = (double)(float)creal(y1);
        } else dx[ix] = y1;
#endif
    }
}

static void ORC(step)(const ORC(ctx) *c, ORC(scratch) *s, double _Complex *dx, WT w, float dz, int iz,
                      int adj)
{
    if (c->pspi) ORC(pspiop)(c, s, dx, w, dz, iz);
    else ORC(ssop)(c, s, dx, w, dz, iz, adj);
}

/* unnormalised real <-> half-complex transform of one trace, wem.c:480-514 */
static void ORC(f_op)(double _Complex *mw, IMG_T *d, int nw, int nt, int adj, FFT_PLAN *pt, FFT_CPX *buf,
                      FFT_CPX *work)
{
    const int n = (nw - 1) * 2;
    if (adj) {
        for (int it = 0; it < n; it++) { buf[it].re = it < nt ? (FR)d[it] : 0; buf[it].im = 0; }
        FFT_EXEC(pt, -1, buf, work);
        for (int iw = 0; iw < nw; iw++) mw[iw] = (double)buf[iw].re + I * (double)buf[iw].im;
    } else {
        for (int k = 0; k < nw && k < n; k++) { buf[k].re = (FR)creal(mw[k]); buf[k].im = (FR)cimag(mw[k]); }
        for (int k = nw; k < n; k++) { buf[k].re = buf[n - k].re; buf[k].im = -buf[n - k].im; }
        buf[0].im = 0;
        if (n % 2 == 0) buf[n / 2].im = 0;
        FFT_EXEC(pt, +1, buf, work);
        /* nt > n (padt = 1, odd nt): the reference reads one float past its c2r output there
           (wem.c:505-507); the periodic continuation of the transform stands in */
        for (int it = 0; it < nt; it++) d[it] = (IMG_T)buf[it < n ? it : it - n].re;
    }
}

/*
 * The operator, wem.c:3-204 (+ extrap1f, wem.c:206-287).
 * adj=1: d [nmx*nmy][nt] -> m [nmx*nmy][nz] (m is overwritten)
 * adj=0: m -> d (d is overwritten)
 * Returns 0, or -1 on a bad argument (the reference has no checks; an out-of-range
 * source cell would write out of bounds there).
 */
int ORC(wem)(IMG_T *d, IMG_T *m, const float *wav, int nt, float ot, float dt, int nmx, float omx,
             float dmx, int nmy, float omy, float dmy, float sx, float sy, int nz, float oz, float dz,
             float gz, float sz, const float *vel, int nref, float fmin, float fmax, int padt, int padx,
             int adj, int pspi, int interp, int nthreads)
{
    (void)ot;
    if (nt < 1 || nmx < 1 || nmy < 1 || nz < 1 || padt < 1 || padx < 1) return -1;
    if (pspi && nref < 2) return -1;
    const int n = nmx * nmy;
    ORC(ctx) C;
    memset(&C, 0, sizeof(C));
    C.nmx = nmx; C.nmy = nmy; C.nz = nz; C.nref = pspi ? nref : 1; C.interp = interp; C.pspi = pspi;
    C.oz = oz; C.dz = dz; C.gz = gz; C.sz = sz; C.vel = vel;

    /* a1: slowness split, wem.c:28-36 */
    C.po = (float *)malloc(sizeof(float) * nz);
    C.pd = (float *)malloc(sizeof(float) * (size_t)n * nz);
    for (int iz = 0; iz < nz; iz++) {
        C.po[iz] = 0.;
        for (int ix = 0; ix < n; ix++) C.po[iz] += vel[(size_t)ix * nz + iz];
        C.po[iz] /= (float)nmx * nmy;
        C.po[iz] = 1. / C.po[iz];
        for (int ix = 0; ix < n; ix++) C.pd[(size_t)ix * nz + iz] = 1.0 / vel[(size_t)ix * nz + iz] - C.po[iz];
    }
#if ORC_FP64
    C.po64 = (double *)malloc(sizeof(double) * nz);
    C.pd64 = (double *)malloc(sizeof(double) * (size_t)n * nz);
    for (int iz = 0; iz < nz; iz++) {
        double acc = 0;
        for (int ix = 0; ix < n; ix++) acc += vel[(size_t)ix * nz + iz];
        C.po64[iz] = (double)n / acc;
        for (int ix = 0; ix < n; ix++) C.pd64[(size_t)ix * nz + iz] = 1.0 / (double)vel[(size_t)ix * nz + iz] - C.po64[iz];
    }
#endif
    /* a2: reference velocities and indices, wem.c:40-70 */
    const int nr = C.nref;
    C.vref = (float *)malloc(sizeof(float) * (size_t)nr * nz);
    C.iref1 = (int *)malloc(sizeof(int) * (size_t)n * nz);
    C.iref2 = (int *)malloc(sizeof(int) * (size_t)n * nz);
#if ORC_FP64
    C.vref64 = (double *)malloc(sizeof(double) * (size_t)nr * nz);
#endif
    for (int iz = 0; iz < nz; iz++) {
        float vmin = vel[iz], vmax = vel[(size_t)(nmx - 1) * nz + iz];
        for (int ix = 0; ix < nmx; ix++) if (vel[(size_t)ix * nz + iz] < vmin) vmin = vel[(size_t)ix * nz + iz];
        for (int ix = 0; ix < n; ix++) if (vel[(size_t)ix * nz + iz] > vmax) vmax = vel[(size_t)ix * nz + iz];
        for (int ir = 0; ir < nr; ir++) {
            C.vref[(size_t)ir * nz + iz] = nr > 1 ? vmin + (float)ir * (vmax - vmin) / ((float)nr - 1) : vmin;
#if ORC_FP64
            C.vref64[(size_t)ir * nz + iz] = nr > 1 ? (double)vmin + (double)ir * ((double)vmax - vmin) / (nr - 1) : vmin;
#endif
        }
        for (int ix = 0; ix < n; ix++) {
            float v = vel[(size_t)ix * nz + iz];
            int i1 = 0, i2 = 0;
            if (vmax > vmin + 10) {
                int ir = (int)(nr - 1) * (v - vmin) / (vmax - vmin);
                /* the reference indexes vref[ir] unchecked; for 3-D grids a point slower
                   than the first line's minimum gives ir < 0 there. Clamp instead. */
                if (ir < 0) ir = 0;
                i1 = ir; i2 = ir + 1;
                if (ir > nr - 2) { i1 = nr - 1; i2 = nr - 1; }
            }
            C.iref1[(size_t)ix * nz + iz] = i1;
            C.iref2[(size_t)ix * nz + iz] = i2;
        }
    }

    /* a3: frequency and wavenumber grids, wem.c:79-89 */
    const int ntfft = (int)2 * padt * ((float)nt) / 2;
    const int nw = (int)ntfft / 2 + 1;
    C.nkx = nmx > 1 ? padx * nmx : 1;
    C.nky = nmy > 1 ? padx * nmy : 1;
    C.dkx = 2 * 3.141592653589793 / ((float)C.nkx) / dmx;
    C.dky = 2 * 3.141592653589793 / ((float)C.nky) / dmy;
    C.dw = 2 * 3.141592653589793 / ((float)ntfft) / dt;
#if ORC_FP64
    C.dkx64 = 2 * 3.141592653589793 / ((double)C.nkx * (double)dmx);
    C.dky64 = 2 * 3.141592653589793 / ((double)C.nky * (double)dmy);
#endif
    int ifmax, ifmin;
    if (fmax * dt * ntfft + 1 < nw) ifmax = (int)fmax * dt * ntfft + 1;
    else ifmax = nw;
    if (fmin * dt * ntfft + 1 < ifmax) ifmin = (int)fmin * dt * ntfft;
    else ifmin = 0;
    C.ntfft = ntfft; C.nw = nw; C.ifmin = ifmin; C.ifmax = ifmax;

    const int igx = (int)(sx - omx) / dmx;
    const int igy = (int)(sy - omy) / dmy;
    int rc = 0;
    if (igx < 0 || igx >= nmx || igy < 0 || igy >= nmy) rc = -1;

    C.px = FFT_CREATE(C.nkx);
    C.py = FFT_CREATE(C.nky);
    const int nf = (nw - 1) * 2 > 0 ? (nw - 1) * 2 : 1;
    FFT_PLAN *pt = FFT_CREATE(nf);
    FFT_CPX *tbuf = (FFT_CPX *)malloc(sizeof(FFT_CPX) * (size_t)nf);
    FFT_CPX *twork = (FFT_CPX *)malloc(sizeof(FFT_CPX) * (size_t)nf);
    IMG_T *dtr = (IMG_T *)calloc((size_t)nt, sizeof(IMG_T));
    double _Complex *d_s = (double _Complex *)calloc((size_t)n * nw, sizeof(double _Complex));
    double _Complex *d_g = (double _Complex *)calloc((size_t)n * nw, sizeof(double _Complex));
    double _Complex *dw_ = (double _Complex *)calloc((size_t)nw, sizeof(double _Complex));

    if (adj) memset(m, 0, sizeof(IMG_T) * (size_t)n * nz);
    else memset(d, 0, sizeof(IMG_T) * (size_t)n * nt);
    if (rc) goto done;

    /* a4: source and receiver spectra, wem.c:112-140 */
    for (int it = 0; it < nt; it++) dtr[it] = (IMG_T)wav[it];
    ORC(f_op)(dw_, dtr, nw, nt, 1, pt, tbuf, twork);
    for (int iw = 0; iw < nw; iw++) d_s[(size_t)(igx * nmy + igy) * nw + iw] = dw_[iw];
    if (adj)
        for (int ix = 0; ix < n; ix++) {
            ORC(f_op)(dw_, d + (size_t)ix * nt, nw, nt, 1, pt, tbuf, twork);
            for (int iw = ifmin; iw < ifmax; iw++) {
#if ORC_FP64
                double w = iw * (2 * 3.141592653589793 / (double)ntfft / (double)dt);
                d_g[(size_t)ix * nw + iw] = w * w * dw_[iw];
#else
                float w = iw * C.dw;
                d_g[(size_t)ix * nw + iw] = w * w * dw_[iw];
#endif
            }
        }

    {
        int nthr = nthreads > 0 ? nthreads : 1;
#ifdef _OPENMP
        if (nthreads <= 0) nthr = omp_get_max_threads();
#endif
        const size_t per = (size_t)n * nz;
        IMG_T *mthr = NULL;
        if (adj) mthr = (IMG_T *)calloc(per * (size_t)nthr, sizeof(IMG_T));
        const int nfreq = ifmax - ifmin;
        /* a5: frequencies in parallel, each thread with its own image slice; the slices
           are added in thread order afterwards (wem.c:141-176). Static contiguous
           chunks, as an OpenMP static schedule gives. */
#pragma omp parallel num_threads(nthr)
        {
            int tid = 0, nth = 1;
#ifdef _OPENMP
            tid = omp_get_thread_num();
            nth = omp_get_num_threads();
#endif
            const int q = nfreq / nth, r = nfreq % nth;
            const int lo = ifmin + tid * q + (tid < r ? tid : r);
            const int hi = lo + q + (tid < r ? 1 : 0);
            const int nk = C.nkx * C.nky;
            const int nline = C.nkx > C.nky ? C.nkx : C.nky;
            ORC(scratch) S;
            S.a = (FFT_CPX *)malloc(sizeof(FFT_CPX) * (size_t)nk);
            S.b = (FFT_CPX *)malloc(sizeof(FFT_CPX) * (size_t)nk);
            S.work = (FFT_CPX *)malloc(sizeof(FFT_CPX) * (size_t)nline);
            S.line = (FFT_CPX *)malloc(sizeof(FFT_CPX) * (size_t)nline);
            S.dref = (double _Complex *)malloc(sizeof(double _Complex) * (size_t)n * C.nref);
            double _Complex *xs = (double _Complex *)malloc(sizeof(double _Complex) * (size_t)n);
            double _Complex *xg = (double _Complex *)malloc(sizeof(double _Complex) * (size_t)n);
            double _Complex *smig = adj ? NULL : (double _Complex *)malloc(sizeof(double _Complex) * (size_t)n * nz);
            IMG_T *mt = adj ? mthr + per * (size_t)tid : NULL;
#if ORC_FP64
            const double sqt = sqrt((double)ntfft);
#else
            const float sqt = sqrtf((float)ntfft);
#endif
            for (int iw = lo; iw < hi; iw++) {
                /* a6 / a11: extrap1f, wem.c:206-287 */
                const float factor = iw == 0 ? 1.f : 2.f;
#if ORC_FP64
                const double w = iw * (2 * 3.141592653589793 / (double)ntfft / (double)dt);
#else
                const float w = iw * C.dw;
#endif
                for (int ix = 0; ix < n; ix++) {
                    xs[ix] = d_s[(size_t)ix * nw + iw] / sqt;
                    xg[ix] = adj ? d_g[(size_t)ix * nw + iw] / sqt : 0;
                }
                if (adj) {
                    for (int iz = 0; iz < nz; iz++) {
                        const float z = oz + dz * iz;
                        if (z >= sz) ORC(step)(&C, &S, xs, w, -dz, iz, 1);
                        if (z >= gz) {
                            ORC(step)(&C, &S, xg, w, dz, iz, 1);
                            for (int ix = 0; ix < n; ix++) {
#if ORC_FP64
                                mt[(size_t)ix * nz + iz] += factor * creal(xg[ix] * conj(xs[ix]));
#else
                                double _Complex us = (double _Complex)conjf((float _Complex)xs[ix]);
                                float re = (float)creal(ORC(cmul)(xg[ix], us));
                                mt[(size_t)ix * nz + iz] += factor * re;
#endif
                            }
                        }
                    }
                } else {
                    for (int iz = 0; iz < nz; iz++) {
                        const float z = oz + dz * iz;
                        if (z >= sz) {
                            ORC(step)(&C, &S, xs, w, -dz, iz, 1);
                            for (int ix = 0; ix < n; ix++) smig[(size_t)ix * nz + iz] = xs[ix];
                        } else
                            for (int ix = 0; ix < n; ix++) smig[(size_t)ix * nz + iz] = 0;
                    }
                    for (int iz = nz - 1; iz >= 0; iz--) {
                        const float z = oz + dz * iz;
                        if (z >= gz) {
                            for (int ix = 0; ix < n; ix++)
                                xg[ix] += m[(size_t)ix * nz + iz] * smig[(size_t)ix * nz + iz];
                            ORC(step)(&C, &S, xg, w, -dz, iz, 0);
                        }
                    }
                    for (int ix = 0; ix < n; ix++) d_g[(size_t)ix * nw + iw] = xg[ix] / sqt;
                }
            }
            free(S.a); free(S.b); free(S.work); free(S.line); free(S.dref);
            free(xs); free(xg); free(smig);
        }
        if (adj) {
            for (int ix = 0; ix < n; ix++)
                for (int t = 0; t < nthr; t++)
                    for (int iz = 0; iz < nz; iz++)
                        m[(size_t)ix * nz + iz] += mthr[per * (size_t)t + (size_t)ix * nz + iz];
            free(mthr);
        } else {
            /* data synthesis, wem.c:177-188 */
            for (int ix = 0; ix < n; ix++) {
                for (int iw = 0; iw < nw; iw++) dw_[iw] = 0;
                for (int iw = ifmin; iw < ifmax; iw++) {
#if ORC_FP64
                    double w = iw * (2 * 3.141592653589793 / (double)ntfft / (double)dt);
#else
                    float w = iw * C.dw;
#endif
                    dw_[iw] = w * w * d_g[(size_t)ix * nw + iw];
                }
                ORC(f_op)(dw_, d + (size_t)ix * nt, nw, nt, 0, pt, tbuf, twork);
            }
        }
    }

done:
    FFT_DESTROY(C.px); FFT_DESTROY(C.py); FFT_DESTROY(pt);
    free(tbuf); free(twork); free(dtr); free(d_s); free(d_g); free(dw_);
    free(C.po); free(C.pd); free(C.vref); free(C.iref1); free(C.iref2);
#if ORC_FP64
    free(C.po64); free(C.pd64); free(C.vref64);
#endif
    return rc;
}

#undef ORC
#undef FR
#undef FFT_PLAN
#undef FFT_CPX
#undef FFT_CREATE
#undef FFT_DESTROY
#undef FFT_EXEC
#undef IMG_T
#undef WT
