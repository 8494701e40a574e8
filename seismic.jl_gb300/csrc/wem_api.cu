// wem_api.cu -- host runtime and C ABI of shotwem.so (declared in include/shotwem_gb300.h).
//
// The per-velocity tables are derived on the host with the reference's own float
// arithmetic (wem.c:28-89, compiled with -ffp-contract=off so that no FMA changes a
// rounding), exactly once per wem_prepare; everything per shot and per frequency
// runs on the GPU: trace spectra (wem_spectra_kernel), the fused depth recursion
// (wem_migrate_kernel) and the image reduction (wem_image_reduce_kernel).
// There is no CPU fallback: without a CUDA device every entry point fails.
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <vector>

#include "../../include/shotwem_gb300.h"
#include "wem_internal.h"

using namespace gbwem;

static thread_local char g_err[512] = "";

static int fail(int code, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

#define CK(call)                                                                                      \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess) return fail(WEM_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                                           __FILE__, __LINE__);                                       \
    } while (0)

struct DevBuf {
    void *p = nullptr;
    size_t n = 0;
};

// bumped on every device (re)allocation: a captured launch sequence that was recorded
// before the bump may hold a freed pointer and is re-captured
static std::atomic<unsigned long long> g_alloc_gen{ 0 };

static int ensure(DevBuf &b, size_t bytes)
{
    if (bytes == 0) bytes = 16;
    if (b.n >= bytes) return WEM_OK;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.n = 0;
    cudaError_t e = cudaMalloc(&b.p, bytes);
    if (e != cudaSuccess) return fail(WEM_ERR_NOMEM, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
    b.n = bytes;
    g_alloc_gen++;
    return WEM_OK;
}

template <class T> static T *P(DevBuf &b) { return reinterpret_cast<T *>(b.p); }

struct wem_ctx {
    int device = 0;
    cudaStream_t st = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // pinned staging ring for host buffers that are not pinned (copy_h2d)
    void *stage[2] = { nullptr, nullptr };
    cudaEvent_t stage_ev[2] = { nullptr, nullptr };
    cudaEvent_t evk[4] = { nullptr, nullptr, nullptr, nullptr };  // around spectra / migrate / reduce
    int nsm = 0;
    float last_ms = 0.f;
    float last_kms[3] = { 0.f, 0.f, 0.f };
    int last_kernels = 0;

    bool prepared = false;
    wem_params p{};
    int ntfft = 0, nw = 0, nf = 0, ifmin = 0, ifmax = 0, nwf = 0, nkx = 0, nky = 0;
    float dw = 0.f, dkx = 0.f, dky = 0.f;
    // 2-D rows: the depth kernels' row length nfft (= nkx, or for an nkx that is not a power
    // of two the power of two >= 2 nkx - 1 that carries it in Bluestein's chirp form, blu)
    int nfft = 0;
    bool blu = false;
    int chirp_off = 0, bfft_off = 0;  // offsets of the chirp and G/N tables in twid (blu)

    // per-velocity tables
    DevBuf vref, slow2, po, pd, sel, wlin, taper, zflag, twid, wtab, scale_recv, scale_src, srcw, wav, wav_base;
    DevBuf vref64;                // [nz][nref] reference velocities in double (split16 FP64 phase tables)
    double dkx64 = 0.0;
    DevBuf ssyn_ref, ssyn_exact;  // synthesis weights w^2 * (half-spectrum | image) factor
    DevBuf tapery, twy;           // 3-D: y taper and y-FFT twiddles
    DevBuf tcw, tcerr;            // split16: W operands of the tensor-core DFT stages, timeout word
    DevBuf wposb;                 // [nz][WPOS_STRIDE] points taking their wavefield whole (paired form)
    DevBuf plan3;                 // [nz][PLAN3_STRIDE] 3-D paired planes (empty: one plane per reference)
    DevBuf ang_vol[7];              // 2-D angles: the batch's volumes (u, u_x, u_l, u_r, u_z, u planes) and angles
    DevBuf dsum3;                 // 3-D direct sums: [item][2][WHOLE_MAX][nky] column sums
    bool plan3_ok = false;
    DevBuf selbp;                 // [nz][nmx rounded up to 16] selection rows (precomputed-table path)
    DevBuf wlinp;                 // [nz][nmx rounded up to 4] linear weights (precomputed-table path)
    DevBuf ptab;                  // [nwf][nz][nref][nkx/2 + 2] phase tables (paired form)
    bool use_ptab = true;         // WEM_PHASE_TABLES=0: every CTA builds its own tables
    bool use_tma = true;          // WEM_TMA=0: the precomputed tables by per-thread cp.async, not bulk copies
    bool ptab_ok = false;         // the current migration uses ptab
    int ptab_nc = 0;              // frequencies per sub-band of ptab (alloc_phase_tables)
    int wdot_off = 0;             // offset of the direct-sum table in twid
    DevBuf refmask;               // [2][nz] bit r: some grid point takes its wavefield from reference r
                                  // (all of it, in the second row)
    DevBuf m3_items, m3_U, m3_Y, m3_C, m3_parts;
    // per-call buffers
    DevBuf recv, slots, image, data, tbase, igx, smig, mimg;
    int max_smem = 0;
    // host copies of the last shot metadata (skip re-uploads)
    std::vector<int64_t> h_tbase;
    std::vector<int> h_igx;
    int last_nshot = -1;
    unsigned long long prep_gen = 0;  // bumped by every wem_prepare

    // the launch sequence of the last 2-D migration, captured as a CUDA graph and
    // replayed while nothing it depends on has changed
    bool use_graph = true;
    bool paired = true;  // PSPI nearest-lower mode: the paired inverse transforms (the tuner's choice)
    bool paired_env = true;  // WEM_PAIRED=0: never paired
    bool tma_env = true;     // WEM_TMA=0: never bulk copies
    cudaGraphExec_t gexec = nullptr;
    struct GraphKey {
        int nshot, wide, grid;
        int64_t ntr;
        const float *d;
        float *m;
        unsigned long long alloc_gen, prep_gen;
        bool operator==(const GraphKey &o) const
        {
            return nshot == o.nshot && wide == o.wide && grid == o.grid && ntr == o.ntr && d == o.d && m == o.m &&
                   alloc_gen == o.alloc_gen && prep_gen == o.prep_gen;
        }
    } gkey{};
    // what the last migration launched
    int last_threads = 0, last_S = 0, last_grid = 0, last_replayed = 0, last_tuned = 0;
    int last_form = 0, last_tma = 0;  // the depth kernel's form (MIG_FORM_*) and table copies of the last 2-D call
};

namespace gbwem {
// lets other translation units of the library report through wem_last_error()
int set_error(int code, const char *msg) { return fail(code, "%s", msg); }
}  // namespace gbwem

extern "C" const char *wem_last_error(void) { return g_err; }
extern "C" int wem_version(void) { return 100; }

extern "C" int wem_ctx_create(wem_ctx **out, int device)
{
    if (!out) return fail(WEM_ERR_ARG, "wem_ctx_create: null output pointer");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(WEM_ERR_NODEV, "no CUDA device: the GPU library has no CPU path");
    if (device < 0 || device >= ndev) return fail(WEM_ERR_ARG, "device %d out of range (have %d)", device, ndev);
    wem_ctx *c = new (std::nothrow) wem_ctx();
    if (!c) return fail(WEM_ERR_NOMEM, "host allocation failed");
    c->device = device;
    CK(cudaSetDevice(device));
    CK(cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking));
    CK(cudaEventCreate(&c->ev0));
    CK(cudaEventCreate(&c->ev1));
    for (int i = 0; i < 4; i++) CK(cudaEventCreate(&c->evk[i]));
    CK(cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, device));
    CK(cudaDeviceGetAttribute(&c->max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
    const char *g = getenv("WEM_GRAPH");
    c->use_graph = !(g && !strcmp(g, "0"));
    *out = c;
    return WEM_OK;
}

extern "C" int wem_ctx_destroy(wem_ctx *c)
{
    if (!c) return WEM_OK;
    cudaSetDevice(c->device);
    if (c->st) cudaStreamSynchronize(c->st);
    DevBuf *bufs[] = { &c->vref, &c->slow2, &c->po, &c->pd, &c->sel, &c->wlin, &c->taper, &c->zflag, &c->twid,
                       &c->wtab, &c->scale_recv, &c->scale_src, &c->srcw, &c->wav, &c->wav_base,
                       &c->ssyn_ref, &c->ssyn_exact, &c->recv, &c->slots, &c->image, &c->data,
                       &c->tbase, &c->igx, &c->smig, &c->mimg, &c->tapery, &c->twy, &c->m3_items,
                       &c->m3_U, &c->m3_Y, &c->m3_C, &c->m3_parts, &c->tcw, &c->tcerr, &c->refmask, &c->wposb, &c->selbp, &c->wlinp, &c->ptab, &c->plan3, &c->dsum3, &c->vref64 };
    for (DevBuf *b : bufs)
        if (b->p) cudaFree(b->p);
    for (int i = 0; i < 2; i++) {
        if (c->stage[i]) cudaFreeHost(c->stage[i]);
        if (c->stage_ev[i]) cudaEventDestroy(c->stage_ev[i]);
    }
    for (DevBuf &b : c->ang_vol)
        if (b.p) cudaFree(b.p);
    if (c->gexec) cudaGraphExecDestroy(c->gexec);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    for (int i = 0; i < 4; i++)
        if (c->evk[i]) cudaEventDestroy(c->evk[i]);
    if (c->st) cudaStreamDestroy(c->st);
    delete c;
    return WEM_OK;
}

extern "C" int wem_last_timing(wem_ctx *c, float *ms, int *kernels)
{
    if (!c) return fail(WEM_ERR_ARG, "null context");
    if (ms) *ms = c->last_ms;
    if (kernels) *kernels = c->last_kernels;
    return WEM_OK;
}

extern "C" int wem_last_kernel_times(wem_ctx *c, float *ms_spectra, float *ms_extrapolate, float *ms_reduce)
{
    if (!c) return fail(WEM_ERR_ARG, "null context");
    if (ms_spectra) *ms_spectra = c->last_kms[0];
    if (ms_extrapolate) *ms_extrapolate = c->last_kms[1];
    if (ms_reduce) *ms_reduce = c->last_kms[2];
    return WEM_OK;
}

extern "C" int wem_selftest_wait_timeout(int device, int *timed_out, float *ms)
{
    if (!timed_out) return fail(WEM_ERR_ARG, "wem_selftest_wait_timeout: null argument");
    CK(cudaSetDevice(device));
    int *d = nullptr;
    CK(cudaMalloc(&d, sizeof(int)));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = WEM_OK;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess || cudaMemset(d, 0, sizeof(int)) ||
        cudaEventRecord(e0, 0) || launch_wait_probe(d, 0) || cudaEventRecord(e1, 0) || cudaEventSynchronize(e1) ||
        cudaMemcpy(timed_out, d, sizeof(int), cudaMemcpyDeviceToHost))
        rc = fail(WEM_ERR_CUDA, "wem_selftest_wait_timeout: %s", cudaGetErrorString(cudaGetLastError()));
    if (!rc && ms) cudaEventElapsedTime(ms, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(d);
    return rc;
}

extern "C" int wem_measure_fp32_peak(int device, double *tflops)
{
    if (!tflops) return fail(WEM_ERR_ARG, "wem_measure_fp32_peak: null argument");
    CK(cudaSetDevice(device));
    int nsm = 0;
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device));
    const int grid = 2 * nsm, iters = 20000;  // 2 CTAs of 512 threads per SM, ~40 ms
    float *d = nullptr;
    CK(cudaMalloc(&d, sizeof(float) * (size_t)grid * 512));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = WEM_OK;
    float best = 0.f;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) rc = fail(WEM_ERR_CUDA, "event");
    for (int rep = 0; rep < 4 && !rc; rep++) {  // the first launch warms up; the best of the rest counts
        float ms = 0.f;
        if (cudaEventRecord(e0, 0) || launch_fma_probe(d, iters, grid, 0) || cudaEventRecord(e1, 0) ||
            cudaEventSynchronize(e1) || cudaEventElapsedTime(&ms, e0, e1))
            rc = fail(WEM_ERR_CUDA, "wem_measure_fp32_peak: %s", cudaGetErrorString(cudaGetLastError()));
        else if (rep > 0 && ms > 0.f && (best == 0.f || ms < best))
            best = ms;
    }
    if (!rc) *tflops = 2.0 * 64.0 * iters * (double)grid * 512.0 / (best * 1e-3) / 1e12;
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(d);
    return rc;
}

extern "C" int wem_last_launch(wem_ctx *c, int *threads, int *shots_per_cta, int *grid, int *replayed, int *tuned)
{
    if (!c) return fail(WEM_ERR_ARG, "null context");
    if (threads) *threads = c->last_threads;
    if (shots_per_cta) *shots_per_cta = c->last_S;
    if (grid) *grid = c->last_grid;
    if (replayed) *replayed = c->last_replayed;
    if (tuned) *tuned = c->last_tuned;
    return WEM_OK;
}

extern "C" int wem_last_launch_form(wem_ctx *c, int *form, int *bulk_tables)
{
    if (!c) return fail(WEM_ERR_ARG, "null context");
    if (form) *form = c->last_form;
    if (bulk_tables) *bulk_tables = c->last_tma;
    return WEM_OK;
}

extern "C" int wem_ctx_stream(wem_ctx *c, void **stream)
{
    if (!c || !stream) return fail(WEM_ERR_ARG, "null argument");
    *stream = (void *)c->st;
    return WEM_OK;
}

// read the per-kernel event times of the last (completed) call; in split16 mode also
// the tensor-core timeout word of the depth kernel
static int collect_times(wem_ctx *c)
{
    if (c->prepared && c->p.nmy == 1 && c->tcerr.p) {
        int e = 0;
        CK(cudaMemcpy(&e, c->tcerr.p, sizeof(int), cudaMemcpyDeviceToHost));
        if (e == 2) return fail(WEM_ERR_TIMEOUT, "a wait for the depth kernel's bulk table copies ran out");
        if (e) return fail(WEM_ERR_TIMEOUT, "a tensor-core wait of the depth kernel ran out (split16 mode)");
    }
    CK(cudaEventElapsedTime(&c->last_ms, c->ev0, c->ev1));
    for (int i = 0; i < 3; i++) CK(cudaEventElapsedTime(&c->last_kms[i], c->evk[i], c->evk[i + 1]));
    return WEM_OK;
}

// ---------------------------------------------------------------- derived grids
// Integer decisions with the reference's float expressions (wem.c:79-89, 112-113).
static void freq_grid(const wem_params &p, int *ntfft, int *nw, int *ifmin, int *ifmax, float *dw)
{
    const int nt = p.nt, padt = p.padt;
    const float fmin = p.fmin, fmax = p.fmax, dt = p.dt;
    const int n = (int)2 * padt * ((float)nt) / 2;
    const int w_ = (int)n / 2 + 1;
    int hi, lo;
    if (fmax * dt * n + 1 < w_) hi = (int)fmax * dt * n + 1;
    else hi = w_;
    if (fmin * dt * n + 1 < hi) lo = (int)fmin * dt * n;
    else lo = 0;
    *ntfft = n;
    *nw = w_;
    *ifmin = lo;
    *ifmax = hi;
    *dw = 2 * 3.141592653589793 / ((float)n) / dt;
}

static int is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

// In-place radix-2 FFT of n = re.size() (a power of two) complex doubles, sign -1 forward.
void fft_pow2_double(std::vector<double> &re, std::vector<double> &im, int sign)
{
    const int n = (int)re.size();
    for (int i = 1, j = 0; i < n; i++) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) {
            std::swap(re[i], re[j]);
            std::swap(im[i], im[j]);
        }
    }
    for (int len = 2; len <= n; len <<= 1) {
        const double ang = sign * 6.283185307179586476925286766559 / len;
        for (int k = 0; k < len / 2; k++) {
            const double wr = cos(ang * k), wi = sin(ang * k);
            for (int i = k; i < n; i += len) {
                const int j = i + len / 2;
                const double xr = re[j] * wr - im[j] * wi, xi = re[j] * wi + im[j] * wr;
                re[j] = re[i] - xr;
                im[j] = im[i] - xi;
                re[i] += xr;
                im[i] += xi;
            }
        }
    }
}

// Tables of a length-L transform on N-point rows in Bluestein's chirp form (xform in
// wem_step.cuh): chirp[n] = e^{i pi n^2 / L}, n < L (n^2 reduced mod 2L in integers, then
// the angle in double), and gq = G / N with G the forward N-point FFT (double precision) of
// the chirp placed at n and N - n (N >= 2L - 1, so the two copies do not overlap).
void bluestein_tables(int L, int N, float2 *chirp, float2 *gq)
{
    std::vector<double> gr(N, 0.0), gi(N, 0.0);
    for (int n = 0; n < L; n++) {
        const long long r = ((long long)n * n) % (2LL * L);
        const double ang = 3.14159265358979323846264338327950288 * (double)r / (double)L;
        const double cr = cos(ang), ci = sin(ang);
        chirp[n] = make_float2((float)cr, (float)ci);
        gr[n] = cr;
        gi[n] = ci;
        if (n > 0) {
            gr[N - n] = cr;
            gi[N - n] = ci;
        }
    }
    fft_pow2_double(gr, gi, -1);
    for (int q = 0; q < N; q++) gq[q] = make_float2((float)(gr[q] / N), (float)(gi[q] / N));
}

// The 2-D row length of the depth kernels for a transform of length nkx: nkx itself when it
// is a power of two in [32, 4096]; otherwise (Bluestein) the smallest power of two >= 2 nkx - 1,
// when that is at most 4096; 0 when neither fits.
int row_length_2d(int nkx, bool *blu)
{
    *blu = false;
    if (is_pow2(nkx)) return (nkx >= 32 && nkx <= 4096) ? nkx : 0;
    if (nkx < 9) return 0;
    int n = 32;
    while (n < 2 * nkx - 1) n *= 2;
    if (n > 4096) return 0;
    *blu = true;
    return n;
}

// boundary_condition weights along one axis (wem.c:546-564), in the reference's float
// expressions (lm = 30 points from each edge when the axis has more than 100)
static std::vector<float> taper_of(int nm)
{
    std::vector<float> tp(nm);
    const int lm = nm > 100 ? 30 : 0;
    float tm = 1.f;
    for (int im = 0; im < nm; im++) {
        if (im >= 0 && im < lm) tm = expf(-powf(0.015 * ((float)lm - im), 2.));
        if (im >= lm && im <= nm - lm) tm = 1.;
        if (im > nm - lm && im < nm) tm = expf(-powf(0.015 * ((float)im - nm + lm), 2.));
        tp[im] = tm;
    }
    return tp;
}

extern "C" int wem_prepare(wem_ctx *c, const wem_params *pp, const float *vel, const float *wav)
{
    if (!c || !pp || !vel || !wav) return fail(WEM_ERR_ARG, "wem_prepare: null argument");
    const wem_params p = *pp;
    if (p.nt < 1 || p.nmx < 1 || p.nmy < 1 || p.nz < 1 || p.padt < 1 || p.padx < 1 || !(p.dt > 0) || !(p.dmx > 0))
        return fail(WEM_ERR_ARG, "wem_prepare: invalid grid (nt=%d nmx=%d nmy=%d nz=%d padt=%d padx=%d)", p.nt,
                    p.nmx, p.nmy, p.nz, p.padt, p.padx);
    if (p.pspi && (p.nref < 2 || p.nref > 64))
        return fail(WEM_ERR_ARG, "PSPI needs 2 <= nref <= 64 (nref=%d; the reference divides by nref-1, wem.c:52)",
                    p.nref);
    if (p.interp != WEM_INTERP_REF && p.interp != WEM_INTERP_LINEAR) return fail(WEM_ERR_ARG, "unknown interp %d", p.interp);
    const int nkx = p.nmx > 1 ? p.padx * p.nmx : 1;
    const int nky = p.nmy > 1 ? p.padx * p.nmy : 1;
    if (p.precision != WEM_PREC_FP32 && p.precision != WEM_PREC_SPLIT16)
        return fail(WEM_ERR_ARG, "unknown precision mode %d", p.precision);
    if (p.precision == WEM_PREC_SPLIT16 && (p.nmy != 1 || nkx != 2048))
        return fail(WEM_ERR_SIZE, "split16 (tensor-core) migration is built for 2-D rows of nkx = padx*nmx = 2048 "
                                  "(have nmy=%d, nkx=%d)", p.nmy, nkx);
    bool blu = false;
    const int nfft = p.nmy == 1 ? row_length_2d(nkx, &blu) : nkx;
    if (p.nmy == 1) {
        if (!nfft)
            return fail(WEM_ERR_SIZE, "nkx = padx*nmx = %d: 2-D rows take a power of two in [32, 4096] or any other "
                                      "length in [9, 2048]", nkx);
        if (blu && p.precision != WEM_PREC_FP32)
            return fail(WEM_ERR_SIZE, "nkx = %d is not a power of two: FP32 precision only", nkx);
    } else if (!m3d_supported(nkx, nky)) {
        return fail(WEM_ERR_SIZE, "3-D: padx*nmx = %d and padx*nmy = %d must be powers of two in [64, 1024]", nkx, nky);
    } else if (!(p.dmy > 0)) {
        return fail(WEM_ERR_ARG, "3-D: dmy must be positive");
    }
    CK(cudaSetDevice(c->device));

    int ntfft, nw, ifmin, ifmax;
    float dw;
    freq_grid(p, &ntfft, &nw, &ifmin, &ifmax, &dw);
    const int nwf = ifmax - ifmin;
    const int nmx = p.nmx, nz = p.nz, n = p.nmx * p.nmy;
    const int nref = p.pspi ? p.nref : 1;

    // a1: slowness split (wem.c:28-36); a2: reference velocities (wem.c:40-70).
    // Device layouts are depth-major ([iz][ix]) so that a depth step reads a row.
    std::vector<float> po(nz), pd((size_t)nz * n), vref((size_t)nz * nref), wl((size_t)nz * n, 0.f);
    std::vector<float> slow2((size_t)nz * nref);
    std::vector<double> vref64((size_t)nz * nref);
    std::vector<uint8_t> sel((size_t)nz * n);
    // points taking their wavefield whole, listed where a depth has at most WHOLE_MAX (their
    // references then pair like the others, and the imaginary parts come from direct sums)
    std::vector<int> wpos((size_t)nz * WPOS_STRIDE, 0);
    const char *ds_env = getenv("WEM_DIRECT_SUMS");  // 0: no direct sums
    const bool direct_sums = !(ds_env && !strcmp(ds_env, "0"));
    // reference velocities some grid point of the depth takes its wavefield from: the
    // others' inverse transforms are skipped (their results would not be used); then
    // (from nz on) those some point takes whole in the nearest-lower mode, where the
    // others give real parts only (wem.c:454-458, 473-478)
    std::vector<unsigned long long> used(2 * (size_t)nz, 0ull);
    for (int iz = 0; iz < nz; iz++) {
        float s = 0.;
        for (int ix = 0; ix < n; ix++) s += vel[(size_t)ix * nz + iz];
        s /= (float)p.nmx * p.nmy;
        s = 1. / s;
        po[iz] = s;
        for (int ix = 0; ix < n; ix++) pd[(size_t)iz * n + ix] = 1.0 / vel[(size_t)ix * nz + iz] - po[iz];
        float vmin = vel[iz], vmax = vel[(size_t)(p.nmx - 1) * nz + iz];
        for (int ix = 0; ix < p.nmx; ix++) if (vel[(size_t)ix * nz + iz] < vmin) vmin = vel[(size_t)ix * nz + iz];
        for (int ix = 0; ix < n; ix++) if (vel[(size_t)ix * nz + iz] > vmax) vmax = vel[(size_t)ix * nz + iz];
        for (int ir = 0; ir < nref; ir++) {
            const float vr = nref > 1 ? vmin + (float)ir * (vmax - vmin) / ((float)nref - 1) : vmin;
            vref[(size_t)iz * nref + ir] = vr;
            slow2[(size_t)iz * nref + ir] = 1 / (vr * vr);  // the float expression of wem.c:434
            vref64[(size_t)iz * nref + ir] =
                nref > 1 ? (double)vmin + (double)ir * ((double)vmax - (double)vmin) / (double)(nref - 1) : (double)vmin;
        }
        for (int ix = 0; ix < n; ix++) {
            const float v = vel[(size_t)ix * nz + iz];
            int i1 = 0, i2 = 0;
            if (vmax > vmin + 10) {
                int ir = (int)(nref - 1) * (v - vmin) / (vmax - vmin);
                if (ir < 0) ir = 0;  // unreachable in 2-D (vmin is the row minimum)
                i1 = ir;
                i2 = ir + 1;
                if (ir > nref - 2) { i1 = nref - 1; i2 = nref - 1; }
            }
            const float vr1 = vref[(size_t)iz * nref + i1], vr2 = vref[(size_t)iz * nref + i2];
            uint8_t word = (uint8_t)i1;  // where it interpolates, i2 = i1 + 1
            if (vr2 - vr1 > 10.0) {
                word |= SEL_INTERP;
                wl[(size_t)iz * n + ix] = (v - vr1) / (vr2 - vr1);
            }
            sel[(size_t)iz * n + ix] = word;
            used[iz] |= 1ull << i1;
            if ((word & SEL_INTERP) && p.interp == WEM_INTERP_LINEAR) used[iz] |= 1ull << (i1 + 1);
            if (!(word & SEL_INTERP)) {
                used[(size_t)nz + iz] |= 1ull << i1;
                int &cnt = wpos[(size_t)iz * WPOS_STRIDE];
                if (cnt <= WHOLE_MAX) {
                    if (cnt < WHOLE_MAX) wpos[(size_t)iz * WPOS_STRIDE + 1 + cnt] = ix;
                    cnt++;
                }
            }
        }
        int &cnt = wpos[(size_t)iz * WPOS_STRIDE];
        // 3-D: direct sums where the paired planes' passes reduce within a warp (nkx, nky <= 512)
        const bool sums_here = p.nmy == 1 || (nkx <= 512 && nky <= 512);
        if (cnt > WHOLE_MAX || !sums_here || p.interp != WEM_INTERP_REF || !direct_sums)
            cnt = 0;  // the whole references keep transforms of their own
        else used[(size_t)nz + iz] = 0ull;
        if (!p.pspi) {
            used[iz] = used[(size_t)nz + iz] = 1ull;
            cnt = 0;
        }
    }
    // taper of the split-step operator (wem.c:546-564): tmx(imx) * tmy(imy)
    std::vector<float> taper = taper_of(nmx), tapery = taper_of(p.nmy);
    std::vector<uint8_t> zf(nz);
    for (int iz = 0; iz < nz; iz++) {
        const float z = p.oz + p.dz * iz;
        zf[iz] = (uint8_t)((z >= p.sz ? Z_SRC : 0) | (z >= p.gz ? Z_REC : 0));
    }
    const int ntw = twiddle_table_size(nfft);
    std::vector<float2> tw(ntw > 0 ? ntw : 1);
    twiddle_table_host(nfft, tw.data());
    // then e^{+2 pi i e / nkx}, e = 0 .. nkx/2 (FP64-built): the direct sums of the paired form
    c->wdot_off = (int)tw.size();
    tw.resize(tw.size() + nkx / 2 + 1);
    for (int e = 0; e <= nkx / 2; e++) {
        const double ang = 6.283185307179586476925 * (double)e / (double)nkx;
        tw[(size_t)c->wdot_off + e] = make_float2((float)cos(ang), (float)sin(ang));
    }
    // then, for a row length that is not a power of two, the chirp (nkx entries, padded to an
    // even count) and G/N (nfft entries) of Bluestein's form
    if (blu) {
        c->chirp_off = (int)tw.size();
        c->bfft_off = c->chirp_off + ((nkx + 1) & ~1);
        tw.resize((size_t)c->bfft_off + nfft);
        bluestein_tables(nkx, nfft, &tw[c->chirp_off], &tw[c->bfft_off]);
    }
    const int ntwy = p.nmy > 1 ? twiddle_table_size(nky) : 1;
    std::vector<float2> twy(ntwy > 0 ? ntwy : 1);
    if (p.nmy > 1) twiddle_table_host(nky, twy.data());
    // the real transform of f_op has length (nw-1)*2 (wem.c:487), which is ntfft - 1
    // when padt*nt is odd
    const int nf = (nw - 1) * 2;
    if (nf < 2) return fail(WEM_ERR_ARG, "wem_prepare: trace too short (nt=%d, padt=%d)", p.nt, p.padt);
    std::vector<float2> wtab(nf);
    for (int k = 0; k < nf; k++) {
        const double a = -6.283185307179586476925286766559 * (double)k / (double)nf;
        wtab[k] = make_float2((float)cos(a), (float)sin(a));
    }
    // receiver weights w^2 (wem.c:128-129) and the 1/sqrtf(ntfft) of wem.c:231-232
    std::vector<float> srec(nwf > 0 ? nwf : 1), ssrc(nwf > 0 ? nwf : 1);
    // modelling: D = w^2 d_g (wem.c:179-184) and the weights of the half-spectrum
    // inverse transform (c2r: 1 at DC and Nyquist, 2 elsewhere) -- or, for the exact
    // adjoint of the migration, its image weights (1 at DC, 2 elsewhere, wem.c:226-227)
    std::vector<float> syn_ref(nwf > 0 ? nwf : 1), syn_exact(nwf > 0 ? nwf : 1);
    const float sq = sqrtf((float)ntfft);
    for (int i = 0; i < nwf; i++) {
        const int iw = ifmin + i;
        const float w = iw * dw;
        srec[i] = (float)((double)(w * w) / (double)sq);
        ssrc[i] = (float)(1.0 / (double)sq);
        syn_ref[i] = (w * w) * ((iw == 0 || 2 * iw == (nw - 1) * 2) ? 1.f : 2.f);
        syn_exact[i] = (w * w) * (iw == 0 ? 1.f : 2.f);
    }

    int rc;
    if ((rc = ensure(c->po, sizeof(float) * nz)) || (rc = ensure(c->pd, sizeof(float) * pd.size())) ||
        (rc = ensure(c->vref, sizeof(float) * vref.size())) || (rc = ensure(c->vref64, sizeof(double) * vref64.size())) ||
        (rc = ensure(c->slow2, sizeof(float) * slow2.size())) || (rc = ensure(c->sel, sel.size())) ||
        (rc = ensure(c->wlin, sizeof(float) * wl.size())) || (rc = ensure(c->taper, sizeof(float) * nmx)) ||
        (rc = ensure(c->zflag, nz)) || (rc = ensure(c->twid, sizeof(float2) * tw.size())) ||
        (rc = ensure(c->wtab, sizeof(float2) * nf)) || (rc = ensure(c->scale_recv, sizeof(float) * srec.size())) ||
        (rc = ensure(c->scale_src, sizeof(float) * ssrc.size())) || (rc = ensure(c->srcw, sizeof(float2) * (nwf > 0 ? nwf : 1))) ||
        (rc = ensure(c->wav, sizeof(float) * p.nt)) || (rc = ensure(c->wav_base, sizeof(int64_t))) ||
        (rc = ensure(c->ssyn_ref, sizeof(float) * syn_ref.size())) ||
        (rc = ensure(c->ssyn_exact, sizeof(float) * syn_exact.size())) ||
        (rc = ensure(c->tapery, sizeof(float) * tapery.size())) || (rc = ensure(c->twy, sizeof(float2) * twy.size())) ||
        (rc = ensure(c->tcw, 10240)) || (rc = ensure(c->tcerr, sizeof(int))) ||
        (rc = ensure(c->refmask, sizeof(unsigned long long) * 2 * nz)) ||
        (rc = ensure(c->wposb, sizeof(int) * wpos.size())) ||
        (rc = ensure(c->selbp, (size_t)nz * ((nmx + 15) / 16 * 16))) ||
        (rc = ensure(c->wlinp, sizeof(float) * (size_t)nz * ((nmx + 3) / 4 * 4))))
        return rc;
    cudaStream_t st = c->st;
    std::vector<uint16_t> tcw(5120);
    tc_w_table_host(tcw.data());
    CK(cudaMemcpyAsync(c->tcw.p, tcw.data(), 10240, cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(c->tcerr.p, 0, sizeof(int), st));
    CK(cudaMemcpyAsync(c->refmask.p, used.data(), sizeof(unsigned long long) * 2 * nz, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->wposb.p, wpos.data(), sizeof(int) * wpos.size(), cudaMemcpyHostToDevice, st));
    // 3-D nearest-lower PSPI: the planes of pass B/C per depth -- pairs of references whose
    // every taker keeps the real part, then an odd one and those taken whole, one plane each
    c->plan3_ok = false;
    if (p.nmy > 1 && p.pspi && p.interp == WEM_INTERP_REF && nref <= PLAN3_MAX) {
        const char *pe = getenv("WEM_PAIRED");
        if (!(pe && !strcmp(pe, "0"))) {
            std::vector<int> plan((size_t)nz * PLAN3_STRIDE, 0);
            for (int iz = 0; iz < nz; iz++) {
                int *pr = &plan[(size_t)iz * PLAN3_STRIDE];
                const unsigned long long u = used[iz], cxm = used[(size_t)nz + iz];
                int np = 0, pend = -1;
                for (int r = 0; r < nref; r++) {
                    if (!((u >> r) & 1ull) || ((cxm >> r) & 1ull)) continue;
                    if (pend < 0) {
                        pend = r;
                    } else {
                        pr[1 + 2 * np] = pend;
                        pr[2 + 2 * np] = r;
                        np++;
                        pend = -1;
                    }
                }
                if (pend >= 0) {
                    pr[1 + 2 * np] = pend;
                    pr[2 + 2 * np] = -1;
                    np++;
                }
                for (int r = 0; r < nref; r++) {
                    if (!((u >> r) & 1ull) || !((cxm >> r) & 1ull)) continue;
                    pr[1 + 2 * np] = r;
                    pr[2 + 2 * np] = -1;
                    np++;
                }
                pr[0] = np;
            }
            int rc3;
            if ((rc3 = ensure(c->plan3, sizeof(int) * plan.size()))) return rc3;
            CK(cudaMemcpyAsync(c->plan3.p, plan.data(), sizeof(int) * plan.size(), cudaMemcpyHostToDevice, st));
            CK(cudaStreamSynchronize(st));  // plan is a local
            c->plan3_ok = true;
        }
    }
    CK(cudaMemcpyAsync(c->po.p, po.data(), sizeof(float) * nz, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->pd.p, pd.data(), sizeof(float) * pd.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->vref.p, vref.data(), sizeof(float) * vref.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->vref64.p, vref64.data(), sizeof(double) * vref64.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->slow2.p, slow2.data(), sizeof(float) * slow2.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->sel.p, sel.data(), sel.size(), cudaMemcpyHostToDevice, st));
    if (p.nmy == 1) {  // selection rows and weights padded to 16 bytes (asynchronous table copies)
        const size_t nsp = (size_t)(nmx + 15) / 16 * 16, nwp = (size_t)(nmx + 3) / 4 * 4;
        std::vector<uint8_t> selp(nz * nsp, 0x7f);
        std::vector<float> wlp(nz * nwp, 0.f);
        for (int iz = 0; iz < nz; iz++) {
            memcpy(&selp[iz * nsp], &sel[(size_t)iz * nmx], nmx);
            memcpy(&wlp[iz * nwp], &wl[(size_t)iz * nmx], sizeof(float) * nmx);
        }
        CK(cudaMemcpyAsync(c->selbp.p, selp.data(), selp.size(), cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(c->wlinp.p, wlp.data(), sizeof(float) * wlp.size(), cudaMemcpyHostToDevice, st));
        CK(cudaStreamSynchronize(st));  // selp and wlp are locals
    }
    CK(cudaMemcpyAsync(c->wlin.p, wl.data(), sizeof(float) * wl.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->taper.p, taper.data(), sizeof(float) * nmx, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->tapery.p, tapery.data(), sizeof(float) * tapery.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->twy.p, twy.data(), sizeof(float2) * twy.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->zflag.p, zf.data(), nz, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->twid.p, tw.data(), sizeof(float2) * tw.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->wtab.p, wtab.data(), sizeof(float2) * nf, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->scale_recv.p, srec.data(), sizeof(float) * srec.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->scale_src.p, ssrc.data(), sizeof(float) * ssrc.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->wav.p, wav, sizeof(float) * p.nt, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->ssyn_ref.p, syn_ref.data(), sizeof(float) * syn_ref.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->ssyn_exact.p, syn_exact.data(), sizeof(float) * syn_exact.size(), cudaMemcpyHostToDevice, st));
    const int64_t zero = 0;
    CK(cudaMemcpyAsync(c->wav_base.p, &zero, sizeof(int64_t), cudaMemcpyHostToDevice, st));
    // wavelet spectrum over the band (wem.c:112-119 with the 1/sqrtf(ntfft) of wem.c:231)
    if (nwf > 0) {
        SpectraArgs sa{};
        sa.d = P<float>(c->wav);
        sa.ntr = 1;
        sa.nt = std::min(p.nt, nf);  // padt = 1 and an odd nt: f_op transforms nt - 1 samples
        sa.ntfft = nf;
        sa.ifmin = ifmin;
        sa.nwf = nwf;
        sa.out_base = P<int64_t>(c->wav_base);
        sa.out_fstride = 1;
        sa.wtab = P<float2>(c->wtab);
        sa.scale = P<float>(c->scale_src);
        sa.out = P<float2>(c->srcw);
        if (launch_spectra(sa, st)) return fail(WEM_ERR_CUDA, "spectra launch: %s", cudaGetErrorString(cudaGetLastError()));
    }
    CK(cudaStreamSynchronize(st));  // the host vectors above go out of scope

    c->p = p;
    c->ntfft = ntfft;
    c->nw = nw;
    c->nf = nf;
    c->ifmin = ifmin;
    c->ifmax = ifmax;
    c->nwf = nwf;
    c->nkx = nkx;
    c->nky = nky;
    c->nfft = nfft;
    c->blu = blu;
    c->dw = dw;
    c->dkx = 2 * 3.141592653589793 / ((float)nkx) / p.dmx;
    c->dkx64 = 2 * 3.141592653589793 / ((double)nkx * (double)p.dmx);
    c->dky = 2 * 3.141592653589793 / ((float)nky) / p.dmy;
    c->prepared = true;
    c->prep_gen++;
    {
        const char *e = getenv("WEM_PAIRED");
        c->paired_env = !(e && !strcmp(e, "0"));
        c->paired = c->paired_env;
        const char *pt = getenv("WEM_PHASE_TABLES");
        c->use_ptab = !(pt && !strcmp(pt, "0"));
        const char *tm = getenv("WEM_TMA");
        c->tma_env = !(tm && !strcmp(tm, "0"));
        c->use_tma = c->tma_env;
    }
    c->last_nshot = -1;
    return WEM_OK;
}

// Upload per-shot metadata when it changed: source cells and per-trace output offsets.
static int set_shots(wem_ctx *c, int nshot, const float *sx, const float *sy, const int64_t *toff,
                     const int32_t *tcell, int64_t *ntr_out)
{
    const wem_params &p = c->p;
    if (nshot < 1 || !sx || !toff || !tcell) return fail(WEM_ERR_ARG, "migrate: bad shot arguments");
    if (toff[0] != 0) return fail(WEM_ERR_ARG, "trace_offset[0] must be 0");
    std::vector<int> igx(nshot);
    for (int s = 0; s < nshot; s++) {
        if (toff[s + 1] < toff[s]) return fail(WEM_ERR_ARG, "trace_offset not monotone at shot %d", s);
        // wem.c:112-113: the cast binds to (sx - omx), then a float division, then truncation
        const int gx = (int)(sx[s] - p.omx) / p.dmx;
        const float syv = sy ? sy[s] : 0.f;
        const int gy = (int)(syv - p.omy) / p.dmy;
        if (gx < 0 || gx >= p.nmx || gy < 0 || gy >= p.nmy)
            return fail(WEM_ERR_ARG, "shot %d: source (%g, %g) falls outside the grid (igx=%d, igy=%d)", s, sx[s], syv, gx, gy);
        igx[s] = gx * p.nmy + gy;  // source cell (= igx in 2-D)
    }
    const int64_t ntr = toff[nshot];
    std::vector<int64_t> base(ntr > 0 ? ntr : 1);
    for (int s = 0; s < nshot; s++)
        for (int64_t i = toff[s]; i < toff[s + 1]; i++) {
            const int cell = tcell[i];
            if (cell < 0 || cell >= p.nmx * p.nmy) return fail(WEM_ERR_ARG, "trace %lld: cell %d outside the grid", (long long)i, cell);
            base[i] = ((int64_t)s * c->nwf) * ((int64_t)p.nmx * p.nmy) + cell;
        }
    *ntr_out = ntr;
    const bool same = c->last_nshot == nshot && c->h_igx == igx && c->h_tbase.size() == (size_t)ntr &&
                      (ntr == 0 || memcmp(c->h_tbase.data(), base.data(), sizeof(int64_t) * ntr) == 0);
    if (same) return WEM_OK;
    int rc;
    if ((rc = ensure(c->igx, sizeof(int) * nshot)) || (rc = ensure(c->tbase, sizeof(int64_t) * base.size()))) return rc;
    CK(cudaMemcpyAsync(c->igx.p, igx.data(), sizeof(int) * nshot, cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(c->tbase.p, base.data(), sizeof(int64_t) * base.size(), cudaMemcpyHostToDevice, c->st));
    CK(cudaStreamSynchronize(c->st));
    c->h_igx = igx;
    c->h_tbase.assign(base.begin(), base.begin() + ntr);
    c->last_nshot = nshot;
    return WEM_OK;
}

// ---------------------------------------------------------------- launch autotuner
// The 2-D depth kernel has choices whose best setting depends on nkx, nref, nmx, the
// velocity model and the device: the CTA shape -- "wide" (512 threads; S shots of an item
// share one set of per-depth phase tables) or "narrow" (256 threads, more CTAs per SM where
// the shared memory allows) --, in the PSPI nearest-lower mode (FP32) the paired inverse
// transforms or one transform per reference, and how the precomputed tables reach shared
// memory (bulk copies on the TMA engine or per-thread cp.async). The first migration of a
// geometry times the candidates on a slice of its own work (one wave of items over the
// first 48 depth steps, with that slice's precomputed tables, after a warm-up launch):
// shape x transforms first, then the table copies for the winner. The process keeps the
// choice per geometry. WEM_CTA_SHAPE=wide|narrow, WEM_PAIRED=0 and WEM_TMA=0 pin a choice;
// WEM_AUTOTUNE=0 takes the wide shape, the paired transforms and bulk copies wherever they
// apply.
struct TuneEntry {
    int device, nkx, pspi, interp, nmx, nref, prec, paired_ok, tma_ok, shape_env;
    int wide, paired, tma;
};

static int tcmode(const wem_ctx *c) { return c->p.precision == WEM_PREC_SPLIT16 ? 1 : 0; }

// the form of the 2-D depth kernel for a CTA shape: split16 when asked for; in the PSPI
// nearest-lower mode the paired inverse transforms when their shared memory fits; FP32
static int mig_form(const wem_ctx *c, int wide)
{
    const wem_params &p = c->p;
    if (c->blu) return MIG_FORM_BLU;
    if (tcmode(c)) return MIG_FORM_SPLIT16;
    if (c->paired && p.pspi && p.interp == WEM_INTERP_REF) {
        int S, th;
        size_t smem;
        if (!migrate_config(c->nfft, wide, p.pspi, p.interp, p.nmx, p.nref, &S, &th, &smem, MIG_FORM_PAIRED) &&
            (int)smem <= c->max_smem)
            return MIG_FORM_PAIRED;
    }
    if (p.pspi && c->use_ptab && c->nfft >= 1024) {
        // reference counts whose phase tables do not fit in shared memory beside the rows:
        // the tables are read from the precomputed ones in device memory
        int S, th;
        size_t smem;
        if (migrate_config(c->nfft, wide, p.pspi, p.interp, p.nmx, p.nref, &S, &th, &smem, MIG_FORM_FP32) ||
            (int)smem > c->max_smem)
            return MIG_FORM_GT;
    }
    return MIG_FORM_FP32;
}
static std::mutex g_tune_mu;
static std::vector<TuneEntry> g_tune;

static MigArgs mig_args(wem_ctx *c, int nshot, int ngroups)
{
    const wem_params &p = c->p;
    MigArgs a{};
    a.nmx = p.nmx;
    a.nz = p.nz;
    a.nref = p.pspi ? p.nref : 1;
    a.nwf = c->nwf;
    a.ifmin = c->ifmin;
    a.nshot = nshot;
    a.ngroups = ngroups;
    a.dw = c->dw;
    a.dz = p.dz;
    a.dkx = c->dkx;
    a.inv_n = 1.0f / (float)c->nkx;
    a.recv = P<float2>(c->recv);
    a.srcw = P<float2>(c->srcw);
    a.igx = P<int>(c->igx);
    a.vref = P<float>(c->vref);
    a.slow2 = P<float>(c->slow2);
    a.po = P<float>(c->po);
    a.pd = P<float>(c->pd);
    a.selb = P<uint8_t>(c->sel);
    a.wlin = P<float>(c->wlin);
    a.taper = P<float>(c->taper);
    a.zflag = P<uint8_t>(c->zflag);
    a.twid = P<float2>(c->twid);
    a.slots = P<float2>(c->slots);
    a.tcw = P<uint4>(c->tcw);
    a.err = P<int>(c->tcerr);
    a.refmask = P<unsigned long long>(c->refmask);
    a.cxmask = P<unsigned long long>(c->refmask) + c->p.nz;
    a.wpos = P<int>(c->wposb);
    a.wdot = P<float2>(c->twid) + c->wdot_off;
    a.selbp = P<uint8_t>(c->selbp);
    a.wlinp = P<float>(c->wlinp);
    a.ptab = nullptr;
    a.nlog = c->nkx;
    if (c->blu) {
        a.chirp = P<float2>(c->twid) + c->chirp_off;
        a.bfft = P<float2>(c->twid) + c->bfft_off;
    }
    a.vref64 = P<double>(c->vref64);
    a.dkx64 = c->dkx64;
    a.tma = c->use_tma ? 1 : 0;
    return a;
}

static int ph_half_of(const wem_ctx *c);
static int ph_stride_of(const wem_ctx *c);
static bool alloc_phase_tables(wem_ctx *c);

// shots*frequencies per ms of one launch setting (c->paired, c->use_tma, `wide`) on a slice
// of the survey; 0 when it does not fit. c->recv must hold nshot*nwf rows (their contents do
// not matter for timing). With precomputed tables the slice's tables are built first, so the
// trial runs the path the migration takes.
static int trial_rate(wem_ctx *c, int nshot, int wide, double *rate)
{
    const wem_params &p = c->p;
    *rate = 0.0;
    int S, threads, bps = 0;
    size_t smem;
    const int form = mig_form(c, wide);
    if (migrate_config(c->nfft, wide, p.pspi, p.interp, p.nmx, p.nref, &S, &threads, &smem, form) ||
        (int)smem > c->max_smem)
        return WEM_OK;
    if (migrate_max_grid(c->nfft, wide, p.pspi, p.interp, p.nmx, p.nref, &bps, form) || bps < 1) {
        cudaGetLastError();
        return WEM_OK;
    }
    const int cap = c->nsm * bps;
    const int ngroups = (nshot + S - 1) / S;
    const int ngroups_t = std::min(ngroups, cap);
    const bool tables = alloc_phase_tables(c);
    if (form == MIG_FORM_GT && !tables) return WEM_OK;  // that form reads the precomputed tables
    const int nwf_t = std::max(1, std::min(tables ? c->ptab_nc : c->nwf, cap / ngroups_t));
    const int items = ngroups_t * nwf_t;  // <= cap: one wave
    int rc;
    MigArgs a = mig_args(c, nshot, ngroups_t);
    a.nwf = nwf_t;  // frequency rows iwi < nwf_t <= nwf stay inside recv
    a.nz = std::min(p.nz, 48);
    if ((rc = ensure(c->slots, sizeof(float2) * (size_t)items * a.nz * p.nmx))) return rc;
    a.slots = P<float2>(c->slots);
    if (tables) {  // the slice's tables, laid out for a.nwf x a.nz
        a.ptab = P<float2>(c->ptab);
        if (launch_phase_tables(ph_half_of(c), ph_stride_of(c), a, P<float2>(c->ptab), c->st, tcmode(c)))
            return fail(WEM_ERR_CUDA, "phase-table launch (tuning): %s", cudaGetErrorString(cudaGetLastError()));
    }
    CK(cudaMemsetAsync(c->tcerr.p, 0, sizeof(int), c->st));
    if (launch_migrate(c->nfft, wide, p.pspi, p.interp, a, items, c->st, form))
        return fail(WEM_ERR_CUDA, "migrate launch (tuning): %s", cudaGetErrorString(cudaGetLastError()));
    CK(cudaEventRecord(c->ev0, c->st));
    if (launch_migrate(c->nfft, wide, p.pspi, p.interp, a, items, c->st, form))
        return fail(WEM_ERR_CUDA, "migrate launch (tuning): %s", cudaGetErrorString(cudaGetLastError()));
    CK(cudaEventRecord(c->ev1, c->st));
    CK(cudaEventSynchronize(c->ev1));
    int terr = 0;
    CK(cudaMemcpy(&terr, c->tcerr.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (terr) return fail(WEM_ERR_TIMEOUT, "a bounded wait of the depth kernel ran out (tuning)");
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    const int shots = std::min(nshot, ngroups_t * S);
    *rate = ms > 0.f ? (double)shots * nwf_t / ms : 0.0;
    return WEM_OK;
}

// Sets *wide, c->paired and c->use_tma for this migration (see the autotuner note above).
static int choose_launch(wem_ctx *c, int nshot, int *wide)
{
    const wem_params &p = c->p;
    const char *e = getenv("WEM_CTA_SHAPE");
    const int shape_env = e && !strcmp(e, "narrow") ? 1 : (e && !strcmp(e, "wide") ? 2 : 0);
    const bool paired_ok = c->paired_env && p.pspi && p.interp == WEM_INTERP_REF && !tcmode(c) && !c->blu;
    const bool tma_ok = c->tma_env && p.pspi && c->use_ptab;
    c->paired = paired_ok;
    c->use_tma = tma_ok;
    // fits(w, 0): the shape runs with the phase tables in shared memory; fits(w, 1): in any form
    auto fits = [&](int w, bool any) {
        int S, th;
        size_t smem;
        const int form = mig_form(c, w);
        if (form == MIG_FORM_GT && !any) return false;
        return !migrate_config(c->nfft, w, p.pspi, p.interp, p.nmx, p.nref, &S, &th, &smem, form) &&
               (int)smem <= c->max_smem;
    };
    const bool wide_fits = fits(1, true);
    c->last_tuned = 0;
    // untuned: the wide shape, unless only the narrow one keeps the tables in shared memory
    *wide = shape_env == 1 ? 0 : (wide_fits && (fits(1, false) || !fits(0, false)) ? 1 : 0);
    const char *t = getenv("WEM_AUTOTUNE");
    if ((t && !strcmp(t, "0")) || c->nwf < 1) return WEM_OK;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        for (const TuneEntry &te : g_tune)
            if (te.device == c->device && te.nkx == c->nkx && te.pspi == p.pspi && te.interp == p.interp &&
                te.nmx == p.nmx && te.nref == p.nref && te.prec == p.precision && te.paired_ok == (int)paired_ok &&
                te.tma_ok == (int)tma_ok && te.shape_env == shape_env) {
                *wide = te.wide;
                c->paired = te.paired != 0;
                c->use_tma = te.tma != 0;
                return WEM_OK;
            }
    }
    int rc;
    if ((rc = ensure(c->recv, sizeof(float2) * (size_t)nshot * std::max(c->nwf, 1) * p.nmx))) return rc;
    // shape x transforms
    double best = -1.0;
    int bw = *wide, bp = c->paired ? 1 : 0;
    for (int w = 1; w >= 0; w--) {
        if ((shape_env == 1 && w) || (shape_env == 2 && !w && wide_fits)) continue;
        for (int pr = paired_ok ? 1 : 0; pr >= 0; pr--) {
            c->paired = pr != 0;
            double r = 0.0;
            if ((rc = trial_rate(c, nshot, w, &r))) return rc;
            if (r > best) {
                best = r;
                bw = w;
                bp = pr;
            }
        }
    }
    *wide = bw;
    c->paired = bp != 0;
    // table copies
    if (tma_ok) {
        double r_bulk = 0.0, r_async = 0.0;
        c->use_tma = true;
        if ((rc = trial_rate(c, nshot, bw, &r_bulk))) return rc;
        c->use_tma = false;
        if ((rc = trial_rate(c, nshot, bw, &r_async))) return rc;
        c->use_tma = r_bulk >= r_async;
    }
    c->last_tuned = 1;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune.push_back({ c->device, c->nkx, p.pspi, p.interp, p.nmx, p.nref, p.precision, (int)paired_ok, (int)tma_ok,
                       shape_env, *wide, (int)c->paired, (int)c->use_tma });
    return WEM_OK;
}

// the paired-plane plan of the 3-D passes when it was built and pass B's shared memory
// (with the columns' spectra) fits the device
static const int *plan3_for(wem_ctx *c, Mig3dArgs a)
{
    if (!c->plan3_ok) return nullptr;
    a.plan = P<int>(c->plan3);
    size_t smem = 0;
    if (m3d_cols_smem(c->nkx, c->p.pspi, a, &smem) || (int)smem > c->max_smem) return nullptr;
    return P<int>(c->plan3);
}

// 3-D migration: spectra -> per depth step the three plane passes of wem_3d.cu for
// every (shot, frequency) of a batch -> image chunks -> image.
static int run_migrate3d(wem_ctx *c, int nshot, int64_t ntr, const float *d_dev, float *m_dev)
{
    const wem_params &p = c->p;
    cudaStream_t st = c->st;
    const int nmx = p.nmx, nmy = p.nmy, nz = p.nz, n = nmx * nmy;
    const int nref = p.pspi ? p.nref : 1;
    const int nitems = nshot * c->nwf;
    const int chunk = std::max(32, (nitems + 15) / 16);
    const int nchunk = (nitems + chunk - 1) / chunk;
    // items per batch: whole chunks, within half of the free device memory
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b));
    const size_t per_item = sizeof(float2) * ((size_t)2 * n + (size_t)2 * nmx * c->nky * (1 + nref));
    const size_t parts_b = sizeof(float2) * (size_t)nchunk * nz * n;
    const size_t recv_b = sizeof(float2) * (size_t)nshot * c->nwf * n;
    if (parts_b + recv_b + per_item * chunk > free_b)
        return fail(WEM_ERR_NOMEM, "3-D survey needs %zu MB of device memory at least", (parts_b + recv_b + per_item * chunk) >> 20);
    long long fit = (long long)((free_b - parts_b - recv_b) / 2 / per_item);
    int batch = (int)std::min<long long>(nitems, std::max<long long>(chunk, fit / chunk * chunk));
    int rc;
    if ((rc = ensure(c->recv, recv_b)) || (rc = ensure(c->m3_parts, parts_b)) ||
        (rc = ensure(c->m3_U, sizeof(float2) * (size_t)batch * 2 * n)) ||
        (rc = ensure(c->m3_Y, sizeof(float2) * (size_t)batch * 2 * nmx * c->nky)) ||
        (rc = ensure(c->m3_C, sizeof(float2) * (size_t)batch * 2 * nref * nmx * c->nky)) ||
        (rc = ensure(c->dsum3, sizeof(float2) * (size_t)batch * 2 * WHOLE_MAX * c->nky)) ||
        (rc = ensure(c->m3_items, sizeof(int) * 2 * (size_t)nitems)))
        return rc;
    std::vector<int> items(2 * (size_t)nitems);
    for (int it = 0; it < nitems; it++) { items[it] = it % c->nwf; items[nitems + it] = it / c->nwf; }
    CK(cudaMemcpyAsync(c->m3_items.p, items.data(), sizeof(int) * items.size(), cudaMemcpyHostToDevice, st));
    int kernels = 0;
    CK(cudaEventRecord(c->ev0, st));
    CK(cudaMemsetAsync(c->recv.p, 0, recv_b, st));
    CK(cudaMemsetAsync(c->m3_parts.p, 0, parts_b, st));
    CK(cudaEventRecord(c->evk[0], st));
    if (c->nwf > 0 && ntr > 0) {
        SpectraArgs sa{};
        sa.d = d_dev; sa.ntr = (int)ntr; sa.nt = std::min(p.nt, c->nf); sa.ld = p.nt; sa.ntfft = c->nf;
        sa.ifmin = c->ifmin; sa.nwf = c->nwf;
        sa.out_base = P<int64_t>(c->tbase); sa.out_fstride = n; sa.wtab = P<float2>(c->wtab);
        sa.scale = P<float>(c->scale_recv); sa.out = P<float2>(c->recv);
        if (launch_spectra(sa, st)) return fail(WEM_ERR_CUDA, "spectra launch: %s", cudaGetErrorString(cudaGetLastError()));
        kernels++;
    }
    CK(cudaEventRecord(c->evk[1], st));
    for (int b0 = 0; b0 < nitems; b0 += batch) {
        const int nb = std::min(batch, nitems - b0);
        Mig3dArgs a{};
        a.nmx = nmx; a.nmy = nmy; a.nkx = c->nkx; a.nky = c->nky; a.nz = nz; a.nref = nref; a.nwf = c->nwf;
        a.ifmin = c->ifmin; a.nitems = nb; a.chunk = chunk;
        a.dw = c->dw; a.dz = p.dz; a.dkx = c->dkx; a.dky = c->dky; a.inv_n = 1.0f / ((float)c->nkx * c->nky);
        a.vref = P<float>(c->vref); a.slow2 = P<float>(c->slow2); a.po = P<float>(c->po); a.pd = P<float>(c->pd); a.wlin = P<float>(c->wlin);
        a.taper = P<float>(c->taper); a.tapery = P<float>(c->tapery); a.selb = P<uint8_t>(c->sel);
        a.zflag = P<uint8_t>(c->zflag); a.twx = P<float2>(c->twid); a.twy = P<float2>(c->twy);
        a.item_iwi = P<int>(c->m3_items) + b0; a.item_shot = P<int>(c->m3_items) + nitems + b0;
        a.src_cell = P<int>(c->igx); a.srcw = P<float2>(c->srcw); a.recv = P<float2>(c->recv);
        a.U = P<float2>(c->m3_U); a.Y = P<float2>(c->m3_Y); a.C = P<float2>(c->m3_C);
        // batches start on chunk boundaries, so the chunk index of local item i is (b0+i)/chunk
        a.img_parts = P<float2>(c->m3_parts) + (size_t)(b0 / chunk) * nz * n;
        a.plan = plan3_for(c, a);
        if (a.plan) {
            a.wpos = P<int>(c->wposb);
            a.dsum = P<float2>(c->dsum3);
        }
        if (m3d_launch_init(a, st)) return fail(WEM_ERR_CUDA, "3-D init launch: %s", cudaGetErrorString(cudaGetLastError()));
        kernels++;
        for (int iz = 0; iz < nz; iz++) {
            a.iz = iz;
            if (m3d_launch_step(c->nkx, c->nky, p.pspi, p.interp, a, c->nsm, st))
                return fail(WEM_ERR_CUDA, "3-D depth step launch: %s", cudaGetErrorString(cudaGetLastError()));
            kernels += 3;
        }
    }
    CK(cudaEventRecord(c->evk[2], st));
    if (launch_image_reduce(P<float2>(c->m3_parts), nchunk, nz, n, m_dev, st))
        return fail(WEM_ERR_CUDA, "reduce launch: %s", cudaGetErrorString(cudaGetLastError()));
    kernels++;
    CK(cudaEventRecord(c->evk[3], st));
    CK(cudaEventRecord(c->ev1, st));
    c->last_kernels = kernels;
    return WEM_OK;
}

// entries of a precomputed phase table (|k| = 0 .. nkx/2) and their stride (float2) in c->ptab:
// the layout the depth kernels' shared memory takes (ph_stride in wem_step.cuh)
static int ph_half_of(const wem_ctx *c) { return c->nkx / 2 + 1; }
static int ph_stride_of(const wem_ctx *c) { return c->blu ? c->nfft / 4 + 2 : c->nkx / 2 + 2; }

// The 2-D PSPI kernels read the phase tables of every (frequency, depth) from an array that
// wem_phase_tables_kernel fills first. The whole band's tables when they fit (at most 32 GiB
// and half the free device memory, counting the array already held); otherwise the band is
// cut into equal sub-bands whose tables fit, and each sub-band is one table launch followed by
// the depth kernel on that sub-band's items (WEM_PTAB_CHUNK=n caps a sub-band at n
// frequencies). Only where not even one frequency's tables fit does each CTA build its own.
// Sets c->ptab_nc (frequencies per sub-band; 0: no precomputed tables); true when c->ptab
// holds them.
static bool alloc_phase_tables(wem_ctx *c)
{
    const wem_params &p = c->p;
    c->ptab_nc = 0;
    if (!c->use_ptab || c->nwf < 1 || !p.pspi || p.nmy > 1) return false;
    const size_t per_f = sizeof(float2) * (size_t)p.nz * p.nref * (size_t)ph_stride_of(c);
    int cap = c->nwf;
    if (const char *e = getenv("WEM_PTAB_CHUNK")) {
        const int v = atoi(e);
        if (v > 0 && v < cap) cap = v;
    }
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    const size_t budget = std::min<size_t>(32ull << 30, (fr + c->ptab.n) / 2);
    const long long fit = (long long)(budget / per_f);
    if (fit < 1) return false;
    int nc = (int)std::min<long long>(cap, fit);
    const int nchunk = (c->nwf + nc - 1) / nc;
    nc = (c->nwf + nchunk - 1) / nchunk;  // equal sub-bands
    if (c->ptab.n < per_f * nc && ensure(c->ptab, per_f * nc) != WEM_OK) {
        cudaGetLastError();
        return false;
    }
    c->ptab_nc = nc;
    return true;
}

// The depth kernel's arguments for the sub-band [f0, f0 + nf) of the frequency band: the
// band offsets of the wavelet spectrum and the receiver rows, the row stride of the full band.
static MigArgs band_args(MigArgs a, const wem_ctx *c, int f0, int nf)
{
    a.ifmin = c->ifmin + f0;
    a.nwf = nf;
    a.recv_nwf = c->nwf;
    a.srcw += f0;
    if (a.recv) a.recv += (size_t)f0 * c->p.nmx;
    return a;
}

// record an event on c->st; inside a stream capture as a graph node (so that the
// per-kernel times stay readable after every replay)
static cudaError_t rec(cudaEvent_t ev, cudaStream_t st, bool capture)
{
    return capture ? cudaEventRecordWithFlags(ev, st, cudaEventRecordExternal) : cudaEventRecord(ev, st);
}

// the launch sequence of a 2-D migration: zero the spectra and accumulators -> trace
// spectra -> depth recursion -> image reduction, with events between the kernels
static int enqueue_migrate(wem_ctx *c, int nshot, int64_t ntr, const float *d_dev, float *m_dev, int wide, int grid,
                           int ngroups, size_t recv_elems, bool capture)
{
    const wem_params &p = c->p;
    cudaStream_t st = c->st;
    const int nmx = p.nmx, nz = p.nz;
    int kernels = 0;
    CK(rec(c->ev0, st, capture));
    CK(cudaMemsetAsync(c->recv.p, 0, sizeof(float2) * recv_elems, st));
    CK(cudaMemsetAsync(c->slots.p, 0, sizeof(float2) * (size_t)grid * nz * nmx, st));
    CK(cudaMemsetAsync(c->tcerr.p, 0, sizeof(int), st));  // the depth kernel's timeout word
    CK(rec(c->evk[0], st, capture));
    if (c->nwf > 0 && ntr > 0) {
        SpectraArgs sa{};
        sa.d = d_dev;
        sa.ntr = (int)ntr;
        sa.nt = std::min(p.nt, c->nf);  // the samples f_op transforms (wem.c:490-493)
        sa.ld = p.nt;
        sa.ntfft = c->nf;
        sa.ifmin = c->ifmin;
        sa.nwf = c->nwf;
        sa.out_base = P<int64_t>(c->tbase);
        sa.out_fstride = nmx;
        sa.wtab = P<float2>(c->wtab);
        sa.scale = P<float>(c->scale_recv);
        sa.out = P<float2>(c->recv);
        if (launch_spectra(sa, st)) return fail(WEM_ERR_CUDA, "spectra launch: %s", cudaGetErrorString(cudaGetLastError()));
        kernels++;
    }
    CK(rec(c->evk[1], st, capture));
    // the band at once, or sub-band by sub-band when only a part of its tables fits
    const int nc = c->ptab_ok ? c->ptab_nc : c->nwf;
    for (int f0 = 0; f0 < c->nwf; f0 += nc) {
        const int nf = std::min(nc, c->nwf - f0);
        MigArgs a = band_args(mig_args(c, nshot, ngroups), c, f0, nf);
        if (c->ptab_ok) {
            a.ptab = P<float2>(c->ptab);
            if (launch_phase_tables(ph_half_of(c), ph_stride_of(c), a, P<float2>(c->ptab), st, tcmode(c)))
                return fail(WEM_ERR_CUDA, "phase-table launch: %s", cudaGetErrorString(cudaGetLastError()));
            kernels++;
        }
        const int g = (int)std::min<long long>(grid, (long long)ngroups * nf);
        if (launch_migrate(c->nfft, wide, p.pspi, p.interp, a, g, st, mig_form(c, wide)))
            return fail(WEM_ERR_CUDA, "migrate launch: %s", cudaGetErrorString(cudaGetLastError()));
        kernels++;
    }
    CK(rec(c->evk[2], st, capture));
    if (launch_image_reduce(P<float2>(c->slots), grid, nz, nmx, m_dev, st))
        return fail(WEM_ERR_CUDA, "reduce launch: %s", cudaGetErrorString(cudaGetLastError()));
    kernels++;
    CK(rec(c->evk[3], st, capture));
    CK(rec(c->ev1, st, capture));
    c->last_kernels = kernels;
    return WEM_OK;
}

// GPU part of a migration: spectra -> depth recursion -> image. Stream-ordered on c->st.
// The whole sequence is captured once as a CUDA graph and replayed by later calls with
// the same shots, buffers and tables (WEM_GRAPH=0 launches it directly every time).
static int run_migrate(wem_ctx *c, int nshot, int64_t ntr, const float *d_dev, float *m_dev)
{
    const wem_params &p = c->p;
    if (p.nmy > 1) return run_migrate3d(c, nshot, ntr, d_dev, m_dev);
    cudaStream_t st = c->st;
    const int nmx = p.nmx, nz = p.nz;
    int S, threads, bps = 0, wide = 0;
    size_t smem;
    int rc;
    if ((rc = choose_launch(c, nshot, &wide))) return rc;
    const int form = mig_form(c, wide);
    if (migrate_config(c->nfft, wide, p.pspi, p.interp, nmx, p.nref, &S, &threads, &smem, form))
        return fail(WEM_ERR_SIZE, "no kernel for nkx=%d", c->nkx);
    if ((int)smem > c->max_smem)
        return fail(WEM_ERR_SIZE, "nref=%d needs %zu B of shared memory per CTA (device limit %d B)", p.nref, smem,
                    c->max_smem);
    if (migrate_max_grid(c->nfft, wide, p.pspi, p.interp, nmx, p.nref, &bps, form) || bps < 1)
        return fail(WEM_ERR_CUDA, "kernel does not fit on the device (smem %zu B, %d threads): %s", smem, threads,
                    cudaGetErrorString(cudaGetLastError()));
    const int ngroups = (nshot + S - 1) / S;
    const long long nitems = (long long)ngroups * c->nwf;
    int grid = (int)((long long)c->nsm * bps < nitems ? (long long)c->nsm * bps : nitems);
    if (grid < 1) grid = 1;
    const size_t recv_elems = (size_t)nshot * (c->nwf > 0 ? c->nwf : 1) * nmx;
    if ((rc = ensure(c->recv, sizeof(float2) * recv_elems)) ||
        (rc = ensure(c->slots, sizeof(float2) * (size_t)grid * nz * nmx)))
        return rc;
    c->ptab_ok = alloc_phase_tables(c);
    if (form == MIG_FORM_GT && !c->ptab_ok)
        return fail(WEM_ERR_SIZE, "nref=%d: the phase tables fit neither in shared memory (%zu B per CTA, device "
                    "limit %d B) nor in device memory", p.nref, smem, c->max_smem);
    c->last_form = form;
    c->last_tma = c->ptab_ok && c->use_tma && p.pspi ? 1 : 0;
    c->last_threads = threads;
    c->last_S = S;
    c->last_grid = grid;
    c->last_replayed = 0;
    if (!c->use_graph) return enqueue_migrate(c, nshot, ntr, d_dev, m_dev, wide, grid, ngroups, recv_elems, false);

    const wem_ctx::GraphKey key{ nshot, wide, grid, ntr, d_dev, m_dev, g_alloc_gen.load(), c->prep_gen };
    if (c->gexec && key == c->gkey) {
        CK(cudaGraphLaunch(c->gexec, st));
        c->last_replayed = 1;
        return WEM_OK;
    }
    if (c->gexec) {
        cudaGraphExecDestroy(c->gexec);
        c->gexec = nullptr;
    }
    CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    rc = enqueue_migrate(c, nshot, ntr, d_dev, m_dev, wide, grid, ngroups, recv_elems, true);
    cudaGraph_t g = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(st, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return rc;
    }
    cudaGraphExec_t ex = nullptr;
    if (ee != cudaSuccess || !g || cudaGraphInstantiate(&ex, g, 0) != cudaSuccess) {
        // this driver cannot capture the sequence: launch directly from now on
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        c->use_graph = false;
        return enqueue_migrate(c, nshot, ntr, d_dev, m_dev, wide, grid, ngroups, recv_elems, false);
    }
    cudaGraphDestroy(g);
    c->gexec = ex;
    c->gkey = key;
    CK(cudaGraphLaunch(ex, st));
    return WEM_OK;
}

extern "C" int wem_migrate_device(wem_ctx *c, int nshot, const float *sx, const float *sy, const int64_t *toff,
                                  const int32_t *tcell, const float *d_dev, float *m_dev, int sync)
{
    if (!c || !c->prepared) return fail(WEM_ERR_ARG, "wem_migrate_device: context not prepared (call wem_prepare)");
    if (nshot < 1 || !toff) return fail(WEM_ERR_ARG, "wem_migrate_device: need nshot >= 1 and trace offsets");
    if (!m_dev || (!d_dev && toff[nshot] > 0)) return fail(WEM_ERR_ARG, "wem_migrate_device: null buffer");
    CK(cudaSetDevice(c->device));
    int64_t ntr = 0;
    int rc = set_shots(c, nshot, sx, sy, toff, tcell, &ntr);
    if (rc) return rc;
    if ((rc = run_migrate(c, nshot, ntr, d_dev, m_dev))) return rc;
    if (sync) {
        CK(cudaStreamSynchronize(c->st));
        if ((rc = collect_times(c))) return rc;
    }
    return WEM_OK;
}

// Host -> device copy on c->st. Pinned (or managed) sources go straight to the copy engine.
// A pageable source of more than a few MB goes through two pinned 16 MiB slots: the host
// copies chunk k into one slot while the copy engine moves chunk k - 1 out of the other, so
// the transfer runs at the copy engine's pinned rate instead of the driver's pageable path.
static int copy_h2d(wem_ctx *c, void *dst, const void *src, size_t bytes)
{
    constexpr size_t SLOT = 16u << 20;
    cudaPointerAttributes at{};
    const bool pinned = cudaPointerGetAttributes(&at, src) == cudaSuccess &&
                        (at.type == cudaMemoryTypeHost || at.type == cudaMemoryTypeManaged);
    cudaGetLastError();
    if (pinned || bytes <= 2 * SLOT) {
        CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->st));
        return WEM_OK;
    }
    for (int i = 0; i < 2; i++) {
        if (!c->stage[i]) CK(cudaHostAlloc(&c->stage[i], SLOT, cudaHostAllocDefault));
        if (!c->stage_ev[i]) CK(cudaEventCreateWithFlags(&c->stage_ev[i], cudaEventDisableTiming));
    }
    int k = 0;
    for (size_t off = 0; off < bytes; off += SLOT, k ^= 1) {
        const size_t n = std::min(SLOT, bytes - off);
        CK(cudaEventSynchronize(c->stage_ev[k]));  // the slot's previous chunk has left
        memcpy(c->stage[k], (const char *)src + off, n);
        CK(cudaMemcpyAsync((char *)dst + off, c->stage[k], n, cudaMemcpyHostToDevice, c->st));
        CK(cudaEventRecord(c->stage_ev[k], c->st));
    }
    return WEM_OK;
}

// Device -> host copy on c->st that has completed when it returns (the stream is synchronised).
// A pageable destination of more than a few MB comes through the two pinned slots: the copy
// engine fills one while the host empties the other.
static int copy_d2h_sync(wem_ctx *c, void *dst, const void *src, size_t bytes)
{
    constexpr size_t SLOT = 16u << 20;
    cudaPointerAttributes at{};
    const bool pinned = cudaPointerGetAttributes(&at, dst) == cudaSuccess &&
                        (at.type == cudaMemoryTypeHost || at.type == cudaMemoryTypeManaged);
    cudaGetLastError();
    if (pinned || bytes <= 2 * SLOT) {
        CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->st));
        CK(cudaStreamSynchronize(c->st));
        return WEM_OK;
    }
    for (int i = 0; i < 2; i++) {
        if (!c->stage[i]) CK(cudaHostAlloc(&c->stage[i], SLOT, cudaHostAllocDefault));
        if (!c->stage_ev[i]) CK(cudaEventCreateWithFlags(&c->stage_ev[i], cudaEventDisableTiming));
    }
    const size_t nchunk = (bytes + SLOT - 1) / SLOT;
    auto issue = [&](size_t k) -> cudaError_t {
        const size_t off = k * SLOT, n = std::min(SLOT, bytes - off);
        cudaError_t e = cudaMemcpyAsync(c->stage[k & 1], (const char *)src + off, n, cudaMemcpyDeviceToHost, c->st);
        return e != cudaSuccess ? e : cudaEventRecord(c->stage_ev[k & 1], c->st);
    };
    CK(issue(0));
    for (size_t k = 0; k < nchunk; k++) {
        CK(cudaEventSynchronize(c->stage_ev[k & 1]));  // chunk k is in its slot
        if (k + 1 < nchunk) CK(issue(k + 1));           // the other slot was emptied in step k - 1
        const size_t off = k * SLOT, n = std::min(SLOT, bytes - off);
        memcpy((char *)dst + off, c->stage[k & 1], n);
    }
    return WEM_OK;
}

extern "C" int wem_migrate(wem_ctx *c, int nshot, const float *sx, const float *sy, const int64_t *toff,
                           const int32_t *tcell, const float *d, float *m)
{
    if (!c || !c->prepared) return fail(WEM_ERR_ARG, "wem_migrate: context not prepared (call wem_prepare)");
    if (nshot < 1 || !toff) return fail(WEM_ERR_ARG, "wem_migrate: need nshot >= 1 and trace offsets");
    if (!m || (!d && toff[nshot] > 0)) return fail(WEM_ERR_ARG, "wem_migrate: null buffer");
    CK(cudaSetDevice(c->device));
    const wem_params &p = c->p;
    int64_t ntr = 0;
    int rc = set_shots(c, nshot, sx, sy, toff, tcell, &ntr);
    if (rc) return rc;
    const size_t dbytes = sizeof(float) * (size_t)ntr * p.nt;
    const size_t mbytes = sizeof(float) * (size_t)p.nmx * p.nmy * p.nz;
    if ((rc = ensure(c->data, dbytes)) || (rc = ensure(c->image, mbytes))) return rc;
    if (dbytes && (rc = copy_h2d(c, c->data.p, d, dbytes))) return rc;
    if ((rc = run_migrate(c, nshot, ntr, P<float>(c->data), P<float>(c->image)))) return rc;
    CK(cudaMemcpyAsync(m, c->image.p, mbytes, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    return collect_times(c);
}


// ------------------------------------------------------------------ derivative convolutions
// The angle computation differentiates its volumes along one axis at a time:
// IDFT(m(k) i k DFT(u)) * scale with m the whole axis (mode 1, scale 1/L) or its left /
// right half (modes 2, 3, scale 1; wem.c:900-945). Along the axis this is a circular
// convolution with w(j) = scale sum_k m(k) i k e^{+2 pi i k j / L}; k is the float
// wavenumber of the reference (axis_k), w is summed in double.
static void deriv_kernel_host(int L, float dk, int mode, float scale, std::vector<double> &wr, std::vector<double> &wi)
{
    std::vector<double> kx(L);
    for (int k = 0; k < L; k++) {
        const float kf = k <= L / 2 ? dk * (float)k : -(dk * (float)L - dk * (float)k);
        const bool on = mode == 1 || (mode == 2 && k > L / 2) || (mode == 3 && k <= L / 2);
        kx[k] = on ? (double)kf : 0.0;
    }
    std::vector<double> cs(L), sn(L);  // e^{2 pi i m / L}
    for (int m = 0; m < L; m++) {
        const double ph = 6.283185307179586476925286766559 * (double)m / L;
        cs[m] = cos(ph);
        sn[m] = sin(ph);
    }
    wr.assign(L, 0.0);
    wi.assign(L, 0.0);
    for (int j = 0; j < L; j++) {
        double re = 0.0, im = 0.0;
        for (int k = 0; k < L; k++) {
            if (kx[k] == 0.0) continue;
            const int m = (int)(((long long)k * j) % L);
            // i k e^{i ph} = k (-sin ph + i cos ph), ph = 2 pi k j / L
            re -= kx[k] * sn[m];
            im += kx[k] * cs[m];
        }
        wr[j] = re * scale;
        wi[j] = im * scale;
    }
}

// The derivative kernels of `modes` (nout of them) along an axis of L samples as transfer
// functions of the M-point rows of launch_angles_conv (M = angles_conv_length(L)):
// H_o = FFT_M(g_o) / M, g_o = w_o at j and at M - j for w_o(-j) = w_o(L - j), in double; H
// holds [nout][M] and tw the row FFT's twiddles.
static int deriv_conv_tables(wem_ctx *c, DevBuf &H, DevBuf &tw, int L, float dk, const int *modes, int nout)
{
    const int M = angles_conv_length(L);
    if (!M) return fail(WEM_ERR_SIZE, "wem_angles: an axis of %d samples (the derivatives take at most 2048)", L);
    std::vector<float2> h((size_t)nout * M), t(twiddle_table_size(M) + 1);
    std::vector<double> wr, wi;
    for (int o = 0; o < nout; o++) {
        deriv_kernel_host(L, dk, modes[o], modes[o] == 1 ? 1.f / (float)L : 1.f, wr, wi);
        std::vector<double> gr(M, 0.0), gi(M, 0.0);
        for (int j = 0; j < L; j++) {
            gr[j] = wr[j];
            gi[j] = wi[j];
            if (j > 0) {
                gr[M - j] = wr[L - j];
                gi[M - j] = wi[L - j];
            }
        }
        fft_pow2_double(gr, gi, -1);
        for (int q = 0; q < M; q++) h[(size_t)o * M + q] = make_float2((float)(gr[q] / M), (float)(gi[q] / M));
    }
    twiddle_table_host(M, t.data());
    int rc;
    if ((rc = ensure(H, sizeof(float2) * h.size())) || (rc = ensure(tw, sizeof(float2) * t.size()))) return rc;
    CK(cudaMemcpyAsync(H.p, h.data(), sizeof(float2) * h.size(), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(tw.p, t.data(), sizeof(float2) * t.size(), cudaMemcpyHostToDevice, c->st));
    CK(cudaStreamSynchronize(c->st));  // h and t are locals
    return WEM_OK;
}

// out[o] = derivative o of u along an axis of L samples (tables of deriv_conv_tables):
// cols == 1 lines of L contiguous samples; cols > 1 column c of planes [L][cols]
static int deriv_conv(wem_ctx *c, const DevBuf &H, const DevBuf &tw, const float2 *u, float2 *const *out, int nout,
                      int L, int cols, long long nlines)
{
    AngleConvArgs a{};
    a.L = L;
    a.cols = cols;
    a.nout = nout;
    a.nlines = nlines;
    a.tw = P<float2>(const_cast<DevBuf &>(tw));
    a.H = P<float2>(const_cast<DevBuf &>(H));
    a.u = u;
    for (int o = 0; o < nout; o++) a.out[o] = out[o];
    if (launch_angles_conv(a, c->nsm, c->st))
        return fail(WEM_ERR_CUDA, "angles: derivative launch (L=%d): %s", L, cudaGetErrorString(cudaGetLastError()));
    return WEM_OK;
}

// ---------------------------------------------------------------- incidence angles
// u_x (whole axis), u_left, u_right: the derivative modes of deriv_kernel_host
static const int kDerivModes[3] = { 1, 2, 3 };

// 3-D (nmy > 1), compute_angles with both lateral axes: per shot and batch of frequencies
// the source is continued down with the plane passes of wem_3d.cu (mode 3, ssop_source's
// split-step step on the unpadded plane, every depth kept), then one-axis transforms
// give u_x, u_y, u_z and the left/right parts along x and y of every depth volume, and
// wem_angles_accum3_kernel adds the batch to the running sums. nmx and nmy must be powers
// of two in [64, 1024] (the plane FFTs of wem_3d.cu).
static int angles3d(wem_ctx *c, const wem_params &p, const float *vel, const float *wav, int nshot, const float *sx,
                    const float *sy, float *angx, float *angy)
{
    const int nmx = p.nmx, nmy = p.nmy, nz = p.nz, n = nmx * nmy;
    if (!m3d_supported(nmx, nmy))
        return fail(WEM_ERR_SIZE, "wem_angles: 3-D needs nmx = %d and nmy = %d to be powers of two in [64, 1024]", nmx,
                    nmy);
    if (!(p.dmy > 0)) return fail(WEM_ERR_ARG, "wem_angles: 3-D needs dmy > 0");
    CK(cudaSetDevice(c->device));
    cudaStream_t st = c->st;
    wem_params q = p;
    q.padt = 1;
    int ntfft, nw, ifmin, ifmax;
    float dw;
    freq_grid(q, &ntfft, &nw, &ifmin, &ifmax, &dw);
    const int nwf = ifmax - ifmin;
    const size_t nn = (size_t)n * nz;
    if (nwf < 1) {
        memset(angx, 0, sizeof(float) * nn * nshot);
        if (angy) memset(angy, 0, sizeof(float) * nn * nshot);
        return WEM_OK;
    }
    // slowness split of compute_angles (wem.c:609-618), depth-major; taper; depth flags
    std::vector<float> po(nz), pd(nn);
    std::vector<uint8_t> zf(nz);
    for (int iz = 0; iz < nz; iz++) {
        float s = 0.;
        for (int ix = 0; ix < n; ix++) s += vel[(size_t)ix * nz + iz];
        s /= (float)nmx * nmy;
        s = 1. / s;
        po[iz] = s;
        for (int ix = 0; ix < n; ix++) pd[(size_t)iz * n + ix] = 1.0 / vel[(size_t)ix * nz + iz] - po[iz];
        const float z = p.oz + p.dz * iz;
        zf[iz] = z >= p.sz ? Z_SRC : 0;
    }
    const std::vector<float> tx = taper_of(nmx), ty = taper_of(nmy);
    std::vector<float2> fx(twiddle_table_size(nmx)), fy(twiddle_table_size(nmy));
    twiddle_table_host(nmx, fx.data());
    twiddle_table_host(nmy, fy.data());
    auto dft_table = [](int L) {
        std::vector<float2> w(L);
        for (int k = 0; k < L; k++) {
            const double a = -6.283185307179586476925286766559 * k / L;
            w[k] = make_float2((float)cos(a), (float)sin(a));
        }
        return w;
    };
    const int lop = (nw - 1) * 2;
    const std::vector<float2> wt = dft_table(lop);
    const float dkx = 2 * 3.141592653589793 / ((float)nmx) / p.dmx;
    const float dky = 2 * 3.141592653589793 / ((float)nmy) / p.dmy;
    const float dkz = 2 * 3.141592653589793 / ((float)nz) / p.dz;
    std::vector<float> sc(nwf, 1.f / sqrtf((float)ntfft));
    // frequencies per batch: 9 depth volumes each, within half of the free memory
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b));
    const size_t per_f = sizeof(float2) * ((size_t)8 * nn + (size_t)6 * n);
    const int batch = (int)std::max<long long>(1, std::min<long long>(nwf, (long long)(free_b / 2 / per_f)));
    const size_t vol = sizeof(float2) * (size_t)batch * nn;
    DevBuf bpo, bpd, btx, bty, bfx, bfy, bwt, bsc, bsrc, bbase, bwav, bzf, bitems, bcell, bU, bY, bC, bS,
        bSX, bLX, bRX, bSY, bLY, bRY, bSZ, bsum, bang;
    DevBuf bHx, bHy, bHz, bTx, bTy, bTz;  // derivative transfer functions and row twiddles of the three axes
    auto release = [&]() {
        DevBuf *bs[] = { &bpo, &bpd, &btx, &bty, &bfx, &bfy, &bwt, &bsc, &bsrc, &bbase, &bwav, &bzf,
                         &bitems, &bcell, &bU, &bY, &bC, &bS, &bSX, &bLX, &bRX, &bSY, &bLY, &bRY, &bSZ, &bsum,
                         &bang, &bHx, &bHy, &bHz, &bTx, &bTy, &bTz };
        for (DevBuf *b : bs)
            if (b->p) cudaFree(b->p);
    };
    int rc;
    if ((rc = ensure(bpo, sizeof(float) * nz)) || (rc = ensure(bpd, sizeof(float) * nn)) ||
        (rc = ensure(btx, sizeof(float) * nmx)) || (rc = ensure(bty, sizeof(float) * nmy)) ||
        (rc = ensure(bfx, sizeof(float2) * fx.size())) || (rc = ensure(bfy, sizeof(float2) * fy.size())) ||
        (rc = ensure(bwt, sizeof(float2) * lop)) ||
        (rc = ensure(bsc, sizeof(float) * nwf)) || (rc = ensure(bsrc, sizeof(float2) * nwf)) ||
        (rc = ensure(bbase, sizeof(int64_t))) || (rc = ensure(bwav, sizeof(float) * p.nt)) || (rc = ensure(bzf, nz)) ||
        (rc = ensure(bitems, sizeof(int) * 2 * (size_t)nwf)) || (rc = ensure(bcell, sizeof(int))) ||
        (rc = ensure(bU, sizeof(float2) * (size_t)batch * 2 * n)) || (rc = ensure(bY, sizeof(float2) * (size_t)batch * 2 * n)) ||
        (rc = ensure(bC, sizeof(float2) * (size_t)batch * 2 * n)) || (rc = ensure(bS, vol)) ||
        (rc = ensure(bSX, vol)) || (rc = ensure(bLX, vol)) || (rc = ensure(bRX, vol)) || (rc = ensure(bSY, vol)) ||
        (rc = ensure(bLY, vol)) || (rc = ensure(bRY, vol)) || (rc = ensure(bSZ, vol)) ||
        (rc = ensure(bsum, sizeof(float) * 4 * nn)) || (rc = ensure(bang, sizeof(float) * 2 * nn)) ||
        (rc = deriv_conv_tables(c, bHx, bTx, nmx, dkx, kDerivModes, 3)) ||
        (rc = deriv_conv_tables(c, bHy, bTy, nmy, dky, kDerivModes, 3)) ||
        (rc = deriv_conv_tables(c, bHz, bTz, nz, dkz, kDerivModes, 1))) {
        release();
        return rc;
    }
#define CKR(call)                                                                                                 \
    do {                                                                                                          \
        cudaError_t e_ = (call);                                                                                  \
        if (e_ != cudaSuccess) {                                                                                  \
            release();                                                                                            \
            return fail(WEM_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__);     \
        }                                                                                                         \
    } while (0)
#define LCHK(expr, what)                                                                                          \
    do {                                                                                                          \
        if (expr) {                                                                                               \
            release();                                                                                            \
            return fail(WEM_ERR_CUDA, "angles: %s launch: %s", what, cudaGetErrorString(cudaGetLastError()));    \
        }                                                                                                         \
    } while (0)
    std::vector<int> items(2 * (size_t)nwf, 0);  // [iwi][shot = 0]
    for (int f = 0; f < nwf; f++) items[f] = f;
    const int64_t zero = 0;
    CKR(cudaMemcpyAsync(bpo.p, po.data(), sizeof(float) * nz, cudaMemcpyHostToDevice, st));
    CKR(cudaMemcpyAsync(bpd.p, pd.data(), sizeof(float) * nn, cudaMemcpyHostToDevice, st));
    CKR(cudaMemcpyAsync(btx.p, tx.data(), sizeof(float) * nmx, cudaMemcpyHostToDevice, st));
    CKR(cudaMemcpyAsync(bty.p, ty.data(), sizeof(float) * nmy, cudaMemcpyHostToDevice, st));
    CKR(cudaMemcpyAsync(bfx.p, fx.data(), sizeof(float2) * fx.size(), cudaMemcpyHostToDevice, st));
    CKR(cudaMemcpyAsync(bfy.p, fy.data(), sizeof(float2) * fy.size(), cudaMemcpyHostToDevice, st));
    CKR(cudaMemcpyAsync(bwt.p, wt.data(), sizeof(float2) * lop, cudaMemcpyHostToDevice, st));
    CKR(cudaMemcpyAsync(bsc.p, sc.data(), sizeof(float) * nwf, cudaMemcpyHostToDevice, st));
    CKR(cudaMemcpyAsync(bbase.p, &zero, sizeof(int64_t), cudaMemcpyHostToDevice, st));
    CKR(cudaMemcpyAsync(bwav.p, wav, sizeof(float) * p.nt, cudaMemcpyHostToDevice, st));
    CKR(cudaMemcpyAsync(bzf.p, zf.data(), nz, cudaMemcpyHostToDevice, st));
    CKR(cudaMemcpyAsync(bitems.p, items.data(), sizeof(int) * items.size(), cudaMemcpyHostToDevice, st));
    SpectraArgs sa{};
    sa.d = P<float>(bwav); sa.ntr = 1; sa.nt = p.nt < lop ? p.nt : lop; sa.ntfft = lop; sa.ifmin = ifmin; sa.nwf = nwf;
    sa.out_base = P<int64_t>(bbase); sa.out_fstride = 1; sa.wtab = P<float2>(bwt); sa.scale = P<float>(bsc);
    sa.out = P<float2>(bsrc);
    LCHK(launch_spectra(sa, st), "spectra");
    int kernels = 1;
    CKR(cudaEventRecord(c->ev0, st));
    for (int s = 0; s < nshot; s++) {
        const float ys = sy ? sy[s] : 0.f;
        const int igx = (int)((float)(int)(sx[s] - p.omx) / p.dmx);  // wem.c:654-655
        const int igy = (int)((float)(int)(ys - p.omy) / p.dmy);
        if (igx < 0 || igx >= nmx || igy < 0 || igy >= nmy) {
            release();
            return fail(WEM_ERR_ARG, "wem_angles: shot %d at (%g, %g) is outside the grid", s, (double)sx[s], (double)ys);
        }
        const int cell = igx * nmy + igy;
        CKR(cudaMemcpyAsync(bcell.p, &cell, sizeof(int), cudaMemcpyHostToDevice, st));
        CKR(cudaMemsetAsync(bsum.p, 0, sizeof(float) * 4 * nn, st));
        for (int b0 = 0; b0 < nwf; b0 += batch) {
            const int nb = std::min(batch, nwf - b0);
            Mig3dArgs a{};
            a.nmx = nmx; a.nmy = nmy; a.nkx = nmx; a.nky = nmy; a.nz = nz; a.nref = 1; a.nwf = nwf;
            a.ifmin = ifmin; a.nitems = nb; a.chunk = 32; a.dw = dw; a.dz = p.dz; a.dkx = dkx; a.dky = dky;
            a.inv_n = 1.0f / ((float)nmx * nmy);
            a.po = P<float>(bpo); a.pd = P<float>(bpd); a.taper = P<float>(btx); a.tapery = P<float>(bty);
            a.zflag = P<uint8_t>(bzf); a.twx = P<float2>(bfx); a.twy = P<float2>(bfy);
            a.item_iwi = P<int>(bitems) + b0; a.item_shot = P<int>(bitems) + nwf;  // shot 0 for every item
            a.src_cell = P<int>(bcell); a.srcw = P<float2>(bsrc);
            a.U = P<float2>(bU); a.Y = P<float2>(bY); a.C = P<float2>(bC); a.smig = P<float2>(bS);
            a.mode = 3; a.pspi = 0;
            LCHK(m3d_launch_init(a, st), "3-D init");
            for (int iz = 0; iz < nz; iz++) {
                a.iz = iz;
                LCHK(m3d_launch_step(nmx, nmy, 0, 0, a, c->nsm, st), "3-D source step");
            }
            kernels += 1 + 3 * nz;
            // derivatives of the depth volumes [f][z][x][y] (wem.c:900-992): x along the columns
            // of the [x][y] planes, y along their rows, z along the columns of the [z][x y]
            // volumes of each frequency
            const long long nbl = nb;
            const float2 *vs = P<float2>(bS);
            float2 *ox[3] = { P<float2>(bSX), P<float2>(bLX), P<float2>(bRX) };
            float2 *oy[3] = { P<float2>(bSY), P<float2>(bLY), P<float2>(bRY) };
            float2 *oz[1] = { P<float2>(bSZ) };
            if ((rc = deriv_conv(c, bHx, bTx, vs, ox, 3, nmx, nmy, nbl * nz * nmy)) ||
                (rc = deriv_conv(c, bHy, bTy, vs, oy, 3, nmy, 1, nbl * nz * nmx)) ||
                (rc = deriv_conv(c, bHz, bTz, vs, oz, 1, nz, n, nbl * n))) {
                release();
                return rc;
            }
            AngleAccum3Args ac{};
            ac.n = n; ac.nz = nz; ac.nwf = nb; ac.nw = nw; ac.nfreq_div = ifmax - ifmin + 1;
            ac.last = b0 + nb >= nwf;
            ac.u = P<float2>(bS); ac.ux = P<float2>(bSX); ac.uy = P<float2>(bSY); ac.uz = P<float2>(bSZ);
            ac.lx = P<float2>(bLX); ac.rx = P<float2>(bRX); ac.ly = P<float2>(bLY); ac.ry = P<float2>(bRY);
            ac.sum = P<float>(bsum); ac.angx = P<float>(bang); ac.angy = P<float>(bang) + nn;
            LCHK(launch_angles_accum3(ac, st), "accumulation");
            kernels += 4;
        }
        CKR(cudaMemcpyAsync(angx + (size_t)s * nn, bang.p, sizeof(float) * nn, cudaMemcpyDeviceToHost, st));
        if (angy) CKR(cudaMemcpyAsync(angy + (size_t)s * nn, P<float>(bang) + nn, sizeof(float) * nn, cudaMemcpyDeviceToHost, st));
        CKR(cudaStreamSynchronize(st));
    }
    CKR(cudaEventRecord(c->ev1, st));
    CKR(cudaStreamSynchronize(st));
#undef CKR
#undef LCHK
    release();
    cudaEventElapsedTime(&c->last_ms, c->ev0, c->ev1);
    c->last_kernels = kernels;
    return WEM_OK;
}

// compute_angles (wem.c:566-684) for each shot: the band [fmin, fmax] of the unpadded
// time axis (ntfft = nt), no spatial padding; any grid length (direct transforms).
extern "C" int wem_angles(wem_ctx *c, const wem_params *pp, const float *vel, const float *wav, int nshot,
                          const float *sx, const float *sy, float *angx, float *angy)
{
    if (!c || !pp || !vel || !wav) return fail(WEM_ERR_ARG, "wem_angles: null argument");
    if (nshot < 1 || !sx || !angx) return fail(WEM_ERR_ARG, "wem_angles: need nshot >= 1, sx and angx");
    const wem_params &p = *pp;
    if (p.nt < 2 || p.nmx < 1 || p.nz < 1 || !(p.dt > 0) || !(p.dmx > 0) || !(p.dz > 0))
        return fail(WEM_ERR_ARG, "wem_angles: invalid grid (nt=%d nmx=%d nz=%d)", p.nt, p.nmx, p.nz);
    if (p.nmy != 1) return angles3d(c, p, vel, wav, nshot, sx, sy, angx, angy);
    const int nmx = p.nmx, nz = p.nz;
    if (nmx > 2048 || nz > 2048)
        return fail(WEM_ERR_SIZE, "wem_angles: nmx = %d and nz = %d must be at most 2048 (the derivatives' rows)", nmx, nz);
    CK(cudaSetDevice(c->device));
    cudaStream_t st = c->st;
    // slowness split of compute_angles (wem.c:609-618), depth-major on the device
    std::vector<float> po(nz), pd((size_t)nz * nmx);
    for (int iz = 0; iz < nz; iz++) {
        float s = 0.;
        for (int ix = 0; ix < nmx; ix++) s += vel[(size_t)ix * nz + iz];
        s /= (float)nmx * p.nmy;
        s = 1. / s;
        po[iz] = s;
        for (int ix = 0; ix < nmx; ix++) pd[(size_t)iz * nmx + ix] = 1.0 / vel[(size_t)ix * nz + iz] - po[iz];
    }
    const std::vector<float> taper = taper_of(nmx);
    wem_params q = p;
    q.padt = 1;  // compute_angles does not pad the time axis (wem.c:589)
    int ntfft, nw, ifmin, ifmax;
    float dw;
    freq_grid(q, &ntfft, &nw, &ifmin, &ifmax, &dw);
    const int nwf = ifmax - ifmin;
    const size_t n = (size_t)nmx * nz;
    if (nwf < 1) {
        memset(angx, 0, sizeof(float) * n * nshot);
        if (angy) memset(angy, 0, sizeof(float) * n * nshot);
        return WEM_OK;
    }
    const float dkx = 2 * 3.141592653589793 / ((float)nmx) / p.dmx;
    const float dkz = 2 * 3.141592653589793 / ((float)nz) / p.dz;
    // source spectrum: f_op of the wavelet on (nw - 1) * 2 samples, / sqrtf(ntfft)
    const int lop = (nw - 1) * 2;
    std::vector<float2> wt(lop), twx(nmx);
    for (int k = 0; k < lop; k++) {
        const double a = -6.283185307179586476925286766559 * k / lop;
        wt[k] = make_float2((float)cos(a), (float)sin(a));
    }
    for (int k = 0; k < nmx; k++) {
        const double a = -6.283185307179586476925286766559 * k / nmx;
        twx[k] = make_float2((float)cos(a), (float)sin(a));
    }
    std::vector<float> sc(nwf, 1.f / sqrtf((float)ntfft));
    // power-of-two widths: the row FFT's per-pass twiddles instead of the direct table
    const bool fftx = angles_fft_supported(nmx);
    std::vector<float2> twf(fftx ? twiddle_table_size(nmx) : 0);
    if (fftx) twiddle_table_host(nmx, twf.data());
    const int64_t zero = 0;
    // shots per batch: all their source volumes and derivatives (5 each) within half the free memory
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b));
    const size_t per_shot = sizeof(float2) * (size_t)5 * nwf * n + sizeof(float) * 2 * n;
    const int nbatch = (int)std::max<long long>(1, std::min<long long>(nshot, (long long)(free_b / 2 / per_shot)));
    const size_t plane = sizeof(float2) * (size_t)nbatch * nwf * n;
    DevBuf bwt, btwx, bsc, bsrc, bbase, bpo, bpd, btap, bwav, btwf;
    DevBuf bHz, bTz, bHx, bTx;  // derivative transfer functions and row twiddles (z; x where x has no row FFT)
    DevBuf bigx;                // the batch's source cells
    // the volumes stay with the context for the next call: u, u_x, u_left, u_right, u_z, the
    // angles
    DevBuf &bU = c->ang_vol[0], &bX = c->ang_vol[1], &bL = c->ang_vol[2], &bR = c->ang_vol[3],
           &bZ = c->ang_vol[4], &bang = c->ang_vol[6];
    auto release = [&]() {
        DevBuf *bs[] = { &bwt, &btwx, &bsc, &bsrc, &bbase, &bpo, &bpd, &btap, &bwav, &btwf,
                         &bHz, &bTz, &bHx, &bTx, &bigx };
        for (DevBuf *b : bs)
            if (b->p) cudaFree(b->p);
    };
    int rc;
    if ((rc = ensure(bwt, sizeof(float2) * lop)) || (rc = ensure(btwx, sizeof(float2) * nmx)) ||
        (rc = ensure(bsc, sizeof(float) * nwf)) ||
        (rc = ensure(bsrc, sizeof(float2) * nwf)) || (rc = ensure(bbase, sizeof(int64_t))) || (rc = ensure(bU, plane)) ||
        (rc = ensure(bX, plane)) || (rc = ensure(bL, plane)) || (rc = ensure(bR, plane)) ||
        (rc = ensure(bZ, plane)) || (rc = ensure(bang, sizeof(float) * 2 * n * nbatch)) ||
        (rc = ensure(bigx, sizeof(int) * nbatch)) ||
        (rc = ensure(bpo, sizeof(float) * nz)) || (rc = ensure(bpd, sizeof(float) * n)) ||
        (rc = ensure(btap, sizeof(float) * nmx)) || (rc = ensure(bwav, sizeof(float) * p.nt)) ||
        (rc = ensure(btwf, sizeof(float2) * (twf.size() + 1)))) {
        release();
        return rc;
    }
#define CKR(call)                                                                                                 \
    do {                                                                                                          \
        cudaError_t e_ = (call);                                                                                  \
        if (e_ != cudaSuccess) {                                                                                  \
            release();                                                                                            \
            return fail(WEM_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__);     \
        }                                                                                                         \
    } while (0)
    CKR(cudaMemcpyAsync(bwt.p, wt.data(), sizeof(float2) * lop, cudaMemcpyHostToDevice, st));
    CKR(cudaMemcpyAsync(btwx.p, twx.data(), sizeof(float2) * nmx, cudaMemcpyHostToDevice, st));
    CKR(cudaMemcpyAsync(bsc.p, sc.data(), sizeof(float) * nwf, cudaMemcpyHostToDevice, st));
    CKR(cudaMemcpyAsync(bbase.p, &zero, sizeof(int64_t), cudaMemcpyHostToDevice, st));
    CKR(cudaMemcpyAsync(bpo.p, po.data(), sizeof(float) * nz, cudaMemcpyHostToDevice, st));
    CKR(cudaMemcpyAsync(bpd.p, pd.data(), sizeof(float) * n, cudaMemcpyHostToDevice, st));
    CKR(cudaMemcpyAsync(btap.p, taper.data(), sizeof(float) * nmx, cudaMemcpyHostToDevice, st));
    CKR(cudaMemcpyAsync(bwav.p, wav, sizeof(float) * p.nt, cudaMemcpyHostToDevice, st));
    if (fftx) CKR(cudaMemcpyAsync(btwf.p, twf.data(), sizeof(float2) * twf.size(), cudaMemcpyHostToDevice, st));
    if ((rc = deriv_conv_tables(c, bHz, bTz, nz, dkz, kDerivModes, 1)) ||
        (!fftx && (rc = deriv_conv_tables(c, bHx, bTx, nmx, dkx, kDerivModes, 3)))) {
        release();
        return rc;
    }
    SpectraArgs sa{};
    sa.d = P<float>(bwav);
    sa.ntr = 1;
    sa.nt = p.nt < lop ? p.nt : lop;
    sa.ntfft = lop;
    sa.ifmin = ifmin;
    sa.nwf = nwf;
    sa.out_base = P<int64_t>(bbase);
    sa.out_fstride = 1;
    sa.wtab = P<float2>(bwt);
    sa.scale = P<float>(bsc);
    sa.out = P<float2>(bsrc);
    if (launch_spectra(sa, st)) {
        release();
        return fail(WEM_ERR_CUDA, "angles: spectra launch: %s", cudaGetErrorString(cudaGetLastError()));
    }
    int kernels = 1;
    CK(cudaEventRecord(c->ev0, st));
    std::vector<int> igxs(nshot);
    for (int s = 0; s < nshot; s++) {
        igxs[s] = (int)((float)(int)(sx[s] - p.omx) / p.dmx);  // (int) (sx - omx)/dmx, wem.c:654
        if (igxs[s] < 0 || igxs[s] >= nmx) {
            release();
            return fail(WEM_ERR_ARG, "wem_angles: shot %d at sx=%g is outside the grid", s, (double)sx[s]);
        }
    }
    const size_t vol = (size_t)nwf * n;  // one shot's volume, samples
    for (int s0 = 0; s0 < nshot; s0 += nbatch) {
        const int nb = std::min(nbatch, nshot - s0);
        CKR(cudaMemcpyAsync(bigx.p, igxs.data() + s0, sizeof(int) * nb, cudaMemcpyHostToDevice, st));
        AngleArgs a{};
        a.nmx = nmx; a.nz = nz; a.nwf = nwf; a.ifmin = ifmin; a.igx = 0; a.nshot = nb; a.igxs = P<int>(bigx);
        a.dw = dw; a.dz = p.dz; a.oz = p.oz; a.sz = p.sz; a.dkx = dkx; a.inv_sqrt_n = 1.f / sqrtf((float)nmx);
        a.po = P<float>(bpo); a.pd = P<float>(bpd); a.taper = P<float>(btap); a.srcw = P<float2>(bsrc);
        a.twx = P<float2>(btwx); a.u = P<float2>(bU);
        AngleXArgs xf{};
        xf.nlines = (long long)nb * nwf * nz; xf.dkx = dkx; xf.twx = P<float2>(btwf); xf.u = P<float2>(bU);
        xf.ux = P<float2>(bX); xf.ul = P<float2>(bL); xf.ur = P<float2>(bR);
        if (fftx) {
            AngleArgs af = a;
            af.twx = P<float2>(btwf);
            if (launch_angles_fft(af, xf, 0, st)) {
                release();
                return fail(WEM_ERR_CUDA, "angles: extrapolation launch: %s", cudaGetErrorString(cudaGetLastError()));
            }
        } else if (launch_angles_extrap(a, st)) {
            release();
            return fail(WEM_ERR_CUDA, "angles: extrapolation launch: %s", cudaGetErrorString(cudaGetLastError()));
        }
        // derivatives of all the batch's volumes: u_x, u_left, u_right (wem.c:900-945) along x --
        // the row FFT for power-of-two widths, else circular convolutions on the rows -- and u_z
        // along z (the columns of every [z][x] plane)
        if (fftx) {
            if (launch_angles_fft(a, xf, 1, st)) {
                release();
                return fail(WEM_ERR_CUDA, "angles: x-derivative launch: %s", cudaGetErrorString(cudaGetLastError()));
            }
        } else {
            float2 *ox[3] = { P<float2>(bX), P<float2>(bL), P<float2>(bR) };
            if ((rc = deriv_conv(c, bHx, bTx, P<float2>(bU), ox, 3, nmx, 1, (long long)nb * nwf * nz))) {
                release();
                return rc;
            }
        }
        {
            float2 *oz[1] = { P<float2>(bZ) };
            if ((rc = deriv_conv(c, bHz, bTz, P<float2>(bU), oz, 1, nz, nmx, (long long)nb * nwf * nmx))) {
                release();
                return rc;
            }
        }
        for (int j = 0; j < nb; j++) {
            AngleAccumArgs ac{};
            ac.nmx = nmx; ac.nz = nz; ac.nwf = nwf; ac.nw = nw; ac.nfreq_div = ifmax - ifmin + 1;
            ac.u = P<float2>(bU) + j * vol; ac.ux = P<float2>(bX) + j * vol; ac.uz = P<float2>(bZ) + j * vol;
            ac.uzp = nullptr;
            ac.ul = P<float2>(bL) + j * vol; ac.ur = P<float2>(bR) + j * vol;
            ac.angx = P<float>(bang) + (size_t)j * 2 * n; ac.angy = P<float>(bang) + (size_t)j * 2 * n + n;
            if (launch_angles_accum(ac, st)) {
                release();
                return fail(WEM_ERR_CUDA, "angles: accumulation launch: %s", cudaGetErrorString(cudaGetLastError()));
            }
        }
        kernels += 3 + nb;
        for (int j = 0; j < nb; j++) {
            const int s = s0 + j;
            CKR(cudaMemcpyAsync(angx + (size_t)s * n, P<float>(bang) + (size_t)j * 2 * n, sizeof(float) * n,
                                cudaMemcpyDeviceToHost, st));
            if (angy)
                CKR(cudaMemcpyAsync(angy + (size_t)s * n, P<float>(bang) + (size_t)j * 2 * n + n, sizeof(float) * n,
                                    cudaMemcpyDeviceToHost, st));
        }
        CKR(cudaStreamSynchronize(st));  // bang is reused by the next batch
    }
    CKR(cudaEventRecord(c->ev1, st));
    CKR(cudaStreamSynchronize(st));
#undef CKR
    release();
    cudaEventElapsedTime(&c->last_ms, c->ev0, c->ev1);
    c->last_kernels = kernels;
    return WEM_OK;
}

extern "C" int wem_migrate_survey(wem_ctx *c, const wem_params *p, const float *vel, const float *wav, int nshot,
                                  const float *sx, const float *sy, const int64_t *toff, const int32_t *tcell,
                                  const float *d, float *m)
{
    int rc = wem_prepare(c, p, vel, wav);
    if (rc) return rc;
    return wem_migrate(c, nshot, sx, sy, toff, tcell, d, m);
}

// GPU part of a modelling: image transpose -> Born recursion -> synthesis. On c->st.
// 3-D modelling with the reference's operator (wem.c:252-281): per batch of items, the
// source continued down with every depth kept (pass C writes smig), then the receiver
// continued up from the bottom with m * smig injected before each step (pass A), then
// the surface planes collected; the synthesis is the 2-D path's.
static int run_model3d(wem_ctx *c, int nshot, int64_t ntr, const float *m_dev, float *d_dev, int exact)
{
    const wem_params &p = c->p;
    cudaStream_t st = c->st;
    const int nmx = p.nmx, nmy = p.nmy, nz = p.nz, n = nmx * nmy;
    const int nref = p.pspi ? p.nref : 1;
    const int nitems = nshot * c->nwf;
    const size_t dg_elems = (size_t)nshot * (c->nwf > 0 ? c->nwf : 1) * n;
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b));
    const size_t per_item = sizeof(float2) * ((size_t)2 * n + (size_t)2 * nmx * c->nky * (1 + nref) + (size_t)nz * n);
    const size_t fixed = sizeof(float2) * dg_elems + sizeof(float) * (size_t)nz * n;
    if (fixed + per_item > free_b)
        return fail(WEM_ERR_NOMEM, "3-D modelling needs %zu MB of device memory at least", (fixed + per_item) >> 20);
    int batch = (int)std::min<long long>(nitems, std::max<long long>(1, (long long)((free_b - fixed) / 2 / per_item)));
    int rc;
    if ((rc = ensure(c->recv, sizeof(float2) * dg_elems)) || (rc = ensure(c->mimg, sizeof(float) * (size_t)nz * n)) ||
        (rc = ensure(c->m3_U, sizeof(float2) * (size_t)batch * 2 * n)) ||
        (rc = ensure(c->m3_Y, sizeof(float2) * (size_t)batch * 2 * nmx * c->nky)) ||
        (rc = ensure(c->m3_C, sizeof(float2) * (size_t)batch * 2 * nref * nmx * c->nky)) ||
        (rc = ensure(c->dsum3, sizeof(float2) * (size_t)batch * 2 * WHOLE_MAX * c->nky)) ||
        (rc = ensure(c->smig, sizeof(float2) * (size_t)batch * nz * n)) ||
        (rc = ensure(c->m3_items, sizeof(int) * 2 * (size_t)std::max(nitems, 1))))
        return rc;
    std::vector<int> items(2 * (size_t)std::max(nitems, 1));
    for (int it = 0; it < nitems; it++) { items[it] = it % c->nwf; items[nitems + it] = it / c->nwf; }
    if (nitems > 0) CK(cudaMemcpyAsync(c->m3_items.p, items.data(), sizeof(int) * 2 * nitems, cudaMemcpyHostToDevice, st));
    int kernels = 0;
    CK(cudaEventRecord(c->ev0, st));
    CK(cudaMemsetAsync(c->recv.p, 0, sizeof(float2) * dg_elems, st));
    if (launch_transpose(m_dev, n, nz, P<float>(c->mimg), st))
        return fail(WEM_ERR_CUDA, "transpose launch: %s", cudaGetErrorString(cudaGetLastError()));
    kernels++;
    CK(cudaEventRecord(c->evk[0], st));
    CK(cudaEventRecord(c->evk[1], st));
    const float inv_sqt = (float)(1.0 / (double)sqrtf((float)c->ntfft));
    for (int b0 = 0; b0 < nitems; b0 += batch) {
        const int nb = std::min(batch, nitems - b0);
        Mig3dArgs a{};
        a.nmx = nmx; a.nmy = nmy; a.nkx = c->nkx; a.nky = c->nky; a.nz = nz; a.nref = nref; a.nwf = c->nwf;
        a.ifmin = c->ifmin; a.nitems = nb; a.chunk = 32;  // pass C runs 32 items per job
        a.dw = c->dw; a.dz = p.dz; a.dkx = c->dkx; a.dky = c->dky; a.inv_n = 1.0f / ((float)c->nkx * c->nky);
        a.vref = P<float>(c->vref); a.slow2 = P<float>(c->slow2); a.po = P<float>(c->po); a.pd = P<float>(c->pd);
        a.wlin = P<float>(c->wlin); a.taper = P<float>(c->taper); a.tapery = P<float>(c->tapery);
        a.selb = P<uint8_t>(c->sel); a.zflag = P<uint8_t>(c->zflag); a.twx = P<float2>(c->twid); a.twy = P<float2>(c->twy);
        a.item_iwi = P<int>(c->m3_items) + b0; a.item_shot = P<int>(c->m3_items) + nitems + b0;
        a.src_cell = P<int>(c->igx); a.srcw = P<float2>(c->srcw); a.recv = nullptr;
        a.U = P<float2>(c->m3_U); a.Y = P<float2>(c->m3_Y); a.C = P<float2>(c->m3_C); a.img_parts = nullptr;
        a.pspi = p.pspi; a.smig = P<float2>(c->smig); a.mimg = P<float>(c->mimg);
        a.refmask = P<unsigned long long>(c->refmask);
        a.plan = plan3_for(c, a);
        if (a.plan) {
            a.wpos = P<int>(c->wposb);
            a.dsum = P<float2>(c->dsum3);
        }
        a.mode = 1;
        if (m3d_launch_init(a, st)) return fail(WEM_ERR_CUDA, "3-D init launch: %s", cudaGetErrorString(cudaGetLastError()));
        kernels++;
        for (int iz = 0; iz < nz; iz++) {  // source down (wem.c:255-265)
            a.iz = iz;
            if (m3d_launch_step(c->nkx, c->nky, p.pspi, p.interp, a, c->nsm, st))
                return fail(WEM_ERR_CUDA, "3-D modelling step launch: %s", cudaGetErrorString(cudaGetLastError()));
            kernels += 3;
        }
        // receiver up (wem.c:266-276): the reference's operator, or with exact = 1 the exact
        // adjoint of the migration step (PSPI; for split-step the reference's operator is it)
        a.mode = exact && p.pspi ? 4 : 2;
        for (int iz = nz - 1; iz >= 0; iz--) {
            a.iz = iz;
            if (m3d_launch_step(c->nkx, c->nky, p.pspi, p.interp, a, c->nsm, st))
                return fail(WEM_ERR_CUDA, "3-D modelling step launch: %s", cudaGetErrorString(cudaGetLastError()));
            kernels += 3;
        }
        if (m3d_launch_collect(a, P<float2>(c->recv), inv_sqt, st))
            return fail(WEM_ERR_CUDA, "3-D collect launch: %s", cudaGetErrorString(cudaGetLastError()));
        kernels++;
    }
    CK(cudaEventRecord(c->evk[2], st));
    if (ntr > 0) {
        SynthArgs sy{};
        sy.dg = P<float2>(c->recv);
        sy.nwf = c->nwf; sy.ifmin = c->ifmin; sy.nt = p.nt; sy.nf = c->nf; sy.ntr = (int)ntr;
        sy.in_base = P<int64_t>(c->tbase); sy.in_fstride = n; sy.wtab = P<float2>(c->wtab);
        sy.scale = P<float>(c->ssyn_ref);
        sy.out = d_dev;
        if (launch_synth(sy, st)) return fail(WEM_ERR_CUDA, "synthesis launch: %s", cudaGetErrorString(cudaGetLastError()));
        kernels++;
    }
    CK(cudaEventRecord(c->evk[3], st));
    CK(cudaEventRecord(c->ev1, st));
    c->last_kernels = kernels;
    return WEM_OK;
}

static int run_model(wem_ctx *c, int nshot, int64_t ntr, const float *m_dev, float *d_dev, int exact)
{
    const wem_params &p = c->p;
    if (p.nmy > 1) return run_model3d(c, nshot, ntr, m_dev, d_dev, exact);
    cudaStream_t st = c->st;
    const int nmx = p.nmx, nz = p.nz;
    int S, threads, bps = 0;
    size_t smem;
    if (model_config(c->nfft, p.pspi, nmx, p.nref, &S, &threads, &smem, c->blu))
        return fail(WEM_ERR_SIZE, "no kernel for nkx=%d", c->nkx);
    if ((int)smem > c->max_smem)
        return fail(WEM_ERR_SIZE, "nref=%d needs %zu B of shared memory per CTA (device limit %d B)", p.nref, smem,
                    c->max_smem);
    if (model_max_grid(c->nfft, p.pspi, p.interp, exact, nmx, p.nref, &bps, c->blu) || bps < 1)
        return fail(WEM_ERR_CUDA, "modelling kernel does not fit on the device: %s", cudaGetErrorString(cudaGetLastError()));
    const int ngroups = (nshot + S - 1) / S;
    const long long nitems = (long long)ngroups * c->nwf;
    int grid = (int)((long long)c->nsm * bps < nitems ? (long long)c->nsm * bps : nitems);
    if (grid < 1) grid = 1;
    int rc;
    const size_t dg_elems = (size_t)nshot * (c->nwf > 0 ? c->nwf : 1) * nmx;
    if ((rc = ensure(c->recv, sizeof(float2) * dg_elems)) ||
        (rc = ensure(c->smig, sizeof(float2) * (size_t)grid * S * nz * nmx)) ||
        (rc = ensure(c->mimg, sizeof(float) * (size_t)nz * nmx)))
        return rc;
    int kernels = 0;
    CK(cudaEventRecord(c->ev0, st));
    CK(cudaMemsetAsync(c->tcerr.p, 0, sizeof(int), st));  // no timeout word from an earlier migration
    CK(cudaMemsetAsync(c->recv.p, 0, sizeof(float2) * dg_elems, st));
    if (launch_transpose(m_dev, nmx, nz, P<float>(c->mimg), st))
        return fail(WEM_ERR_CUDA, "transpose launch: %s", cudaGetErrorString(cudaGetLastError()));
    kernels++;
    CK(cudaEventRecord(c->evk[0], st));
    CK(cudaEventRecord(c->evk[1], st));
    if (c->nwf > 0) {
        MigArgs a{};
        a.nmx = nmx; a.nz = nz; a.nref = p.pspi ? p.nref : 1; a.nwf = c->nwf; a.ifmin = c->ifmin;
        a.nshot = nshot; a.ngroups = ngroups; a.dw = c->dw; a.dz = p.dz; a.dkx = c->dkx;
        a.inv_n = 1.0f / (float)c->nkx;
        a.recv = nullptr; a.srcw = P<float2>(c->srcw); a.igx = P<int>(c->igx); a.vref = P<float>(c->vref); a.slow2 = P<float>(c->slow2);
        a.po = P<float>(c->po); a.pd = P<float>(c->pd); a.selb = P<uint8_t>(c->sel); a.wlin = P<float>(c->wlin);
        a.taper = P<float>(c->taper); a.zflag = P<uint8_t>(c->zflag); a.twid = P<float2>(c->twid); a.slots = nullptr;
        a.refmask = P<unsigned long long>(c->refmask);
        a.selbp = P<uint8_t>(c->selbp);
        a.wlinp = P<float>(c->wlinp);
        a.nlog = c->nkx;
        if (c->blu) {
            a.chirp = P<float2>(c->twid) + c->chirp_off;
            a.bfft = P<float2>(c->twid) + c->bfft_off;
        }
        BornArgs b{};
        b.img = P<float>(c->mimg);
        b.smig = P<float2>(c->smig);
        b.inv_sqt = (float)(1.0 / (double)sqrtf((float)c->ntfft));
        // the band at once, or sub-band by sub-band when only a part of its tables fits
        const bool tables = alloc_phase_tables(c);
        const int nc = tables ? c->ptab_nc : c->nwf;
        for (int f0 = 0; f0 < c->nwf; f0 += nc) {
            const int nf = std::min(nc, c->nwf - f0);
            MigArgs ab = band_args(a, c, f0, nf);
            b.dg = P<float2>(c->recv) + (size_t)f0 * nmx;
            if (tables) {
                ab.ptab = P<float2>(c->ptab);
                if (launch_phase_tables(ph_half_of(c), ph_stride_of(c), ab, P<float2>(c->ptab), st))
                    return fail(WEM_ERR_CUDA, "phase-table launch: %s", cudaGetErrorString(cudaGetLastError()));
                kernels++;
            }
            const int g = (int)std::min<long long>(grid, (long long)ngroups * nf);
            if (launch_model(c->nfft, p.pspi, p.interp, exact, ab, b, g, st, c->blu))
                return fail(WEM_ERR_CUDA, "modelling launch: %s", cudaGetErrorString(cudaGetLastError()));
            kernels++;
        }
    }
    CK(cudaEventRecord(c->evk[2], st));
    if (ntr > 0) {
        SynthArgs sy{};
        sy.dg = P<float2>(c->recv);
        sy.nwf = c->nwf; sy.ifmin = c->ifmin; sy.nt = p.nt; sy.nf = c->nf; sy.ntr = (int)ntr;
        sy.in_base = P<int64_t>(c->tbase); sy.in_fstride = nmx; sy.wtab = P<float2>(c->wtab);
        sy.scale = exact ? P<float>(c->ssyn_exact) : P<float>(c->ssyn_ref);
        sy.out = d_dev;
        if (launch_synth(sy, st)) return fail(WEM_ERR_CUDA, "synthesis launch: %s", cudaGetErrorString(cudaGetLastError()));
        kernels++;
    }
    CK(cudaEventRecord(c->evk[3], st));
    CK(cudaEventRecord(c->ev1, st));
    c->last_kernels = kernels;
    return WEM_OK;
}

extern "C" int wem_model_device(wem_ctx *c, int nshot, const float *sx, const float *sy, const int64_t *toff,
                                const int32_t *tcell, const float *m_dev, float *d_dev, int exact, int sync)
{
    if (!c || !c->prepared) return fail(WEM_ERR_ARG, "wem_model_device: context not prepared (call wem_prepare)");
    if (nshot < 1 || !toff) return fail(WEM_ERR_ARG, "wem_model_device: need nshot >= 1 and trace offsets");
    if (!m_dev || (!d_dev && toff[nshot] > 0)) return fail(WEM_ERR_ARG, "wem_model_device: null buffer");
    CK(cudaSetDevice(c->device));
    int64_t ntr = 0;
    int rc = set_shots(c, nshot, sx, sy, toff, tcell, &ntr);
    if (rc) return rc;
    if ((rc = run_model(c, nshot, ntr, m_dev, d_dev, exact ? 1 : 0))) return rc;
    if (sync) {
        CK(cudaStreamSynchronize(c->st));
        if ((rc = collect_times(c))) return rc;
    }
    return WEM_OK;
}

extern "C" int wem_model(wem_ctx *c, int nshot, const float *sx, const float *sy, const int64_t *toff,
                         const int32_t *tcell, const float *m, float *d, int exact)
{
    if (!c || !c->prepared) return fail(WEM_ERR_ARG, "wem_model: context not prepared (call wem_prepare)");
    if (nshot < 1 || !toff) return fail(WEM_ERR_ARG, "wem_model: need nshot >= 1 and trace offsets");
    if (!m || (!d && toff[nshot] > 0)) return fail(WEM_ERR_ARG, "wem_model: null buffer");
    CK(cudaSetDevice(c->device));
    const wem_params &p = c->p;
    int64_t ntr = 0;
    int rc = set_shots(c, nshot, sx, sy, toff, tcell, &ntr);
    if (rc) return rc;
    const size_t dbytes = sizeof(float) * (size_t)ntr * p.nt;
    const size_t mbytes = sizeof(float) * (size_t)p.nmx * p.nmy * p.nz;
    if ((rc = ensure(c->data, dbytes)) || (rc = ensure(c->image, mbytes))) return rc;
    CK(cudaMemcpyAsync(c->image.p, m, mbytes, cudaMemcpyHostToDevice, c->st));
    if ((rc = run_model(c, nshot, ntr, P<float>(c->image), P<float>(c->data), exact ? 1 : 0))) return rc;
    if (dbytes) {
        if ((rc = copy_d2h_sync(c, d, c->data.p, dbytes))) return rc;
    } else {
        CK(cudaStreamSynchronize(c->st));
    }
    return collect_times(c);
}

// ---------------------------------------------------------------- wem() drop-in
static std::mutex g_default_mu;
static wem_ctx *g_default = nullptr;

static int default_ctx(wem_ctx **out)
{
    std::lock_guard<std::mutex> lk(g_default_mu);
    if (!g_default) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
        int rc = wem_ctx_create(&g_default, dev);
        if (rc) return rc;
    }
    *out = g_default;
    return WEM_OK;
}

extern "C" int wem(float **d, float **m, float **wav, int nt, float ot, float dt, int nmx, float omx, float dmx, int nmy,
                   float omy, float dmy, float sx, float sy, int nz, float oz, float dz, float gz, float sz, float **vel,
                   int nref, float fmin, float fmax, int padt, int padx, bool adj, bool pspi, bool verbose)
{
    if (!d || !m || !wav || !vel || !wav[0]) return fail(WEM_ERR_ARG, "wem: null argument");
    if (nt < 1 || nmx < 1 || nmy < 1 || nz < 1) return fail(WEM_ERR_ARG, "wem: invalid sizes");
    wem_ctx *c;
    int rc = default_ctx(&c);
    if (rc) return rc;
    wem_params p{};
    p.nt = nt; p.ot = ot; p.dt = dt;
    p.nmx = nmx; p.omx = omx; p.dmx = dmx;
    p.nmy = nmy; p.omy = omy; p.dmy = dmy;
    p.nz = nz; p.oz = oz; p.dz = dz; p.gz = gz; p.sz = sz;
    p.nref = nref; p.fmin = fmin; p.fmax = fmax; p.padt = padt; p.padx = padx;
    p.pspi = pspi ? 1 : 0;
    p.interp = WEM_INTERP_REF;
    p.precision = WEM_PREC_FP32;
    p.verbose = verbose ? 1 : 0;
    const int n = nmx * nmy;
    std::vector<float> v((size_t)n * nz), dd((size_t)n * nt), mm((size_t)n * nz);
    for (int ix = 0; ix < n; ix++) {
        if (!vel[ix] || !d[ix] || !m[ix]) return fail(WEM_ERR_ARG, "wem: null row %d", ix);
        memcpy(&v[(size_t)ix * nz], vel[ix], sizeof(float) * nz);
        if (adj) memcpy(&dd[(size_t)ix * nt], d[ix], sizeof(float) * nt);
        else memcpy(&mm[(size_t)ix * nz], m[ix], sizeof(float) * nz);
    }
    if ((rc = wem_prepare(c, &p, v.data(), wav[0]))) return rc;
    std::vector<int64_t> off = { 0, (int64_t)n };
    std::vector<int32_t> cell(n);
    for (int i = 0; i < n; i++) cell[i] = i;
    if (adj) {
        // migration: d -> m, m overwritten (wem.c:73-74)
        if ((rc = wem_migrate(c, 1, &sx, &sy, off.data(), cell.data(), dd.data(), mm.data()))) return rc;
        for (int ix = 0; ix < n; ix++) memcpy(m[ix], &mm[(size_t)ix * nz], sizeof(float) * nz);
    } else {
        // modelling with the reference's operator: m -> d, d overwritten (wem.c:76-77)
        if ((rc = wem_model(c, 1, &sx, &sy, off.data(), cell.data(), mm.data(), dd.data(), 0))) return rc;
        for (int ix = 0; ix < n; ix++) memcpy(d[ix], &dd[(size_t)ix * nt], sizeof(float) * nt);
    }
    if (verbose) fprintf(stderr, "wem: %d frequencies x %d depth steps on the GPU in %.3f ms\n", c->nwf, nz, c->last_ms);
    return WEM_OK;
}
