// wem_noalloc.cu -- wem_migrate_noalloc: shot-profile migration that allocates nothing.
//
// Who needs it: callers that must not call cudaMalloc/cudaFree once they are running
// -- for example a host application that hands every byte of device memory to its
// own pool at start-up, or a processing loop with a fixed memory budget that must
// not stall on the allocator or fail halfway through a survey. They pass their own
// device buffers for the inputs and the output; everything the migration needs
// besides those (the per-velocity tables, the trace spectra, the image
// accumulator) lives in one file-scope device array of fixed size, g_wem_scratch.
// CUDA loads a module's device memory when the module is first used on a device
// (lazy loading, the default since CUDA 12.2), so the array -- and the code of the
// kernels this path launches -- takes its device memory at the first call on each
// device, and keeps it until the process exits. A caller that is about to give all
// free device memory to its own pool therefore makes one small call first (or runs
// with CUDA_MODULE_LOADING=EAGER, which loads everything when the context is made).
//
// The path is the same computation as wem_migrate (wem.c:3-204 semantics) with two
// differences: the tables are derived on the GPU from the caller's velocity instead
// of on the host, and the image is accumulated with atomic float additions into one
// depth-major image instead of per-CTA compensated accumulators, so the low bits of
// the result depend on the order in which the CTAs finish.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "../../include/shotwem_gb300.h"
#include "wem_fft.cuh"
#include "wem_internal.h"
#include "wem_step.cuh"

namespace gbwem {
int set_error(int code, const char *msg);  // wem_api.cu: records wem_last_error()
}

using namespace gbwem;

// Size of the scratch array. What fits (checked on every call): see noalloc_layout.
#define WEM_NOALLOC_SCRATCH_BYTES (24u << 20)

static __device__ __align__(256) unsigned char g_wem_scratch[WEM_NOALLOC_SCRATCH_BYTES];

namespace {

struct Layout {
    size_t po, pd, vref, slow2, sel, wlin, taper, zflag, twid, wtab, srec, ssrc, srcw, igx, tbase, wbase, recv, img, total;
};

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

Layout noalloc_layout(int nmx, int nz, int nref, int ntw, int nf, int nwf, int nshot)
{
    Layout L{};
    size_t o = 0;
    auto take = [&](size_t bytes) { const size_t at = o; o = align256(o + bytes); return at; };
    L.po = take(sizeof(float) * nz);
    L.pd = take(sizeof(float) * (size_t)nz * nmx);
    L.vref = take(sizeof(float) * (size_t)nz * nref);
    L.slow2 = take(sizeof(float) * (size_t)nz * nref);
    L.sel = take((size_t)nz * nmx);
    L.wlin = take(sizeof(float) * (size_t)nz * nmx);
    L.taper = take(sizeof(float) * nmx);
    L.zflag = take((size_t)nz);
    L.twid = take(sizeof(float2) * (size_t)ntw);
    L.wtab = take(sizeof(float2) * (size_t)nf);
    L.srec = take(sizeof(float) * (size_t)nwf);
    L.ssrc = take(sizeof(float) * (size_t)nwf);
    L.srcw = take(sizeof(float2) * (size_t)nwf);
    L.igx = take(sizeof(int) * (size_t)nshot);
    L.tbase = take(sizeof(int64_t) * (size_t)nshot * nmx);
    L.wbase = take(sizeof(int64_t));
    L.recv = take(sizeof(float2) * (size_t)nshot * nwf * nmx);
    L.img = take(sizeof(float) * (size_t)nz * nmx);
    L.total = o;
    return L;
}

// The device address of g_wem_scratch on the current device. A host-side reference to
// g_wem_scratch names a host shadow, not device memory, so the address must come from
// cudaGetSymbolAddress with the device current. It is looked up on every call (a cheap
// query once the module is loaded): after a cudaDeviceReset the module is loaded again
// and the array may sit at another address.
int scratch_for_current_device(void **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_error(WEM_ERR_CUDA, cudaGetErrorString(e));
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_wem_scratch);
    if (e != cudaSuccess || !p) return set_error(WEM_ERR_CUDA, "cudaGetSymbolAddress(g_wem_scratch) failed");
    *out = p;
    return WEM_OK;
}

struct TableArgs {
    const float *vel;  // [nmx][nz] (the reference's layout)
    int nmx, nz, nref, ntw, nkx, nf, nwf, ifmin, ntfft, nshot, lmx;
    float oz, dz, sz, gz, dw;
    float *po, *pd, *vref, *slow2, *wlin, *taper, *srec, *ssrc;
    uint8_t *sel;
    uint8_t *zflag;
    float2 *twid, *wtab;
    int *igx;
    int64_t *tbase, *wbase;
    int igx_val[64];
};

// The host setup of wem_prepare (wem.c:28-70 and the grids of wem.c:79-89) on the
// GPU: block iz < nz builds depth iz; the extra blocks fill the depth-independent
// tables. The integer decisions and their float arithmetic (po, pd, the reference
// velocities, the selection bytes and the linear weights) follow the host's operation
// order exactly. The taper (device expf) and the FFT and DFT twiddles (device sincos in
// double) can differ from the host tables by one unit in the last place.
__global__ void __launch_bounds__(256) noalloc_tables_kernel(const TableArgs a)
{
    __shared__ float s_po, s_vmin, s_vmax;
    const int b = blockIdx.x, tid = threadIdx.x;
    if (b < a.nz) {
        const int iz = b;
        if (tid == 0) {
            float s = 0.f;
            for (int ix = 0; ix < a.nmx; ix++) s = __fadd_rn(s, a.vel[(size_t)ix * a.nz + iz]);
            s = __fdiv_rn(s, (float)a.nmx);
            s = __double2float_rn(__ddiv_rn(1.0, (double)s));
            float vmin = a.vel[iz], vmax = a.vel[(size_t)(a.nmx - 1) * a.nz + iz];
            for (int ix = 0; ix < a.nmx; ix++) {
                const float v = a.vel[(size_t)ix * a.nz + iz];
                vmin = v < vmin ? v : vmin;
                vmax = v > vmax ? v : vmax;
            }
            s_po = s;
            s_vmin = vmin;
            s_vmax = vmax;
            a.po[iz] = s;
            const float z = __fadd_rn(a.oz, __fmul_rn(a.dz, (float)iz));
            a.zflag[iz] = (uint8_t)((z >= a.sz ? Z_SRC : 0) | (z >= a.gz ? Z_REC : 0));
        }
        __syncthreads();
        const float po = s_po, vmin = s_vmin, vmax = s_vmax;
        const int nr = a.nref;
        for (int r = tid; r < nr; r += blockDim.x) {
            const float vr =
                nr > 1 ? __fadd_rn(vmin, __fdiv_rn(__fmul_rn((float)r, __fsub_rn(vmax, vmin)), __fsub_rn((float)nr, 1.f)))
                       : vmin;
            a.vref[(size_t)iz * nr + r] = vr;
            a.slow2[(size_t)iz * nr + r] = __fdiv_rn(1.f, __fmul_rn(vr, vr));
        }
        for (int ix = tid; ix < a.nmx; ix += blockDim.x) {
            const float v = a.vel[(size_t)ix * a.nz + iz];
            a.pd[(size_t)iz * a.nmx + ix] = __double2float_rn(__dsub_rn(__ddiv_rn(1.0, (double)v), (double)po));
            int i1 = 0, i2 = 0;
            if (vmax > __fadd_rn(vmin, 10.f)) {
                int ir = __float2int_rz(__fdiv_rn(__fmul_rn((float)(nr - 1), __fsub_rn(v, vmin)), __fsub_rn(vmax, vmin)));
                if (ir < 0) ir = 0;
                i1 = ir;
                i2 = ir + 1;
                if (ir > nr - 2) { i1 = nr - 1; i2 = nr - 1; }
            }
            const float vr1 = nr > 1 ? __fadd_rn(vmin, __fdiv_rn(__fmul_rn((float)i1, __fsub_rn(vmax, vmin)), __fsub_rn((float)nr, 1.f))) : vmin;
            const float vr2 = nr > 1 ? __fadd_rn(vmin, __fdiv_rn(__fmul_rn((float)i2, __fsub_rn(vmax, vmin)), __fsub_rn((float)nr, 1.f))) : vmin;
            uint8_t word = (uint8_t)i1;  // where it interpolates, i2 = i1 + 1
            float wl = 0.f;
            if (__fsub_rn(vr2, vr1) > 10.f) {
                word |= SEL_INTERP;
                wl = __fdiv_rn(__fsub_rn(v, vr1), __fsub_rn(vr2, vr1));
            }
            a.sel[(size_t)iz * a.nmx + ix] = word;
            a.wlin[(size_t)iz * a.nmx + ix] = wl;
        }
        return;
    }
    // depth-independent tables, one grid-stride pass over the extra blocks
    const int nb = gridDim.x - a.nz;
    const int i0 = (b - a.nz) * blockDim.x + tid, step = nb * blockDim.x;
    for (int x = i0; x < a.nmx; x += step) {
        // boundary taper of wem.c:546-564, 2-D
        float tmx = 1.f;
        if (x < a.lmx) {
            const float q = __double2float_rn(0.015 * (double)((float)a.lmx - (float)x));
            tmx = expf(-__fmul_rn(q, q));
        } else if (x > a.nmx - a.lmx) {
            const float q = __double2float_rn(0.015 * (double)((float)x - (float)a.nmx + (float)a.lmx));
            tmx = expf(-__fmul_rn(q, q));
        }
        a.taper[x] = tmx;
    }
    // per-pass FFT twiddles (the layout of twiddle_table_host)
    for (int e = i0; e < a.ntw; e += step) {
        int log2n = 0;
        while ((1 << log2n) < a.nkx) log2n++;
        const int npass = (log2n + 3) / 4;
        int ns = 1, off = 0;
        for (int p = 0; p < npass; p++) {
            const int R = (p < log2n / 4) ? 16 : (1 << (log2n % 4));
            if (p > 0) {
                const int cnt = ns * (R - 1);
                if (e < off + cnt) {
                    const int k = (e - off) / (R - 1), r = (e - off) % (R - 1) + 1;
                    const double ang = -6.283185307179586476925286766559 * (double)((long long)r * k) / ((double)ns * R);
                    double sn, cs;
                    sincos(ang, &sn, &cs);
                    a.twid[e] = make_float2((float)cs, (float)sn);
                    break;
                }
                off += cnt;
            }
            ns *= R;
        }
    }
    for (int k = i0; k < a.nf; k += step) {
        double sn, cs;
        sincos(-6.283185307179586476925286766559 * (double)k / (double)a.nf, &sn, &cs);
        a.wtab[k] = make_float2((float)cs, (float)sn);
    }
    const float sq = __fsqrt_rn((float)a.ntfft);
    for (int i = i0; i < a.nwf; i += step) {
        const float w = __fmul_rn((float)(a.ifmin + i), a.dw);
        a.srec[i] = __double2float_rn((double)__fmul_rn(w, w) / (double)sq);
        a.ssrc[i] = __double2float_rn(1.0 / (double)sq);
    }
    for (int s = i0; s < a.nshot; s += step) a.igx[s] = a.igx_val[s];
    for (int t = i0; t < a.nshot * a.nmx; t += step)
        a.tbase[t] = ((int64_t)(t / a.nmx) * a.nwf) * a.nmx + (t % a.nmx);
    if (i0 == 0) a.wbase[0] = 0;
}

// wem_migrate_kernel's recursion with the image added atomically into img[iz][x].
template <int N, bool PSPI, int INTERP, int S>
__global__ void __launch_bounds__(2 * S * (N / 16)) wem_migrate_atomic_kernel(const MigArgs a, float *img)
{
    using SH = MigShape<N>;
    constexpr int T = SH::T, PADN = SH::PADN;
    constexpr int NT = 2 * S * T;
    extern __shared__ float4 smem_raw[];
    const Smem<N, PSPI> sm(smem_raw, a.nref, a.nmx, 2 * S);
    const int tid = threadIdx.x;
    const int team = tid / T, t = tid - team * T;
    const bool is_src = team < S;
    const int sg = is_src ? team : team - S;
    float2 *xbuf = sm.x + (size_t)team * PADN;
    float2 *sacc = sm.acc + (size_t)team * sm.acc_stride;
    const unsigned sync = team_sync_handle<N>(tid);
    for (int i = tid; i < SH::TW; i += NT) sm.tw[i] = a.twid[i];
    const int nitems = a.ngroups * a.nwf;
    const int nmx = a.nmx;
    for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
        const int g = item % a.ngroups;
        const int iwi = item / a.ngroups;
        const int shot = g * S + sg;
        const bool shot_ok = shot < a.nshot;
        const int iw = a.ifmin + iwi;
        const float w = __fmul_rn((float)iw, a.dw);
        const float w2 = __fmul_rn(w, w);
        const float factor = iw == 0 ? 1.f : 2.f;
        float2 v[16];
        const int igx = shot_ok ? a.igx[shot] : -1;
        const float2 sw = a.srcw[iwi];
        const float2 *rrow = a.recv + ((size_t)(shot_ok ? shot : 0) * a.nwf + iwi) * nmx;
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const int x = t + T * m;
            float2 u = make_float2(0.f, 0.f);
            if (x < nmx && shot_ok) u = is_src ? (x == igx ? sw : u) : rrow[x];
            v[m] = u;
        }
        for (int iz = 0; iz < a.nz; iz++) {
            __syncthreads();
            build_tables<N, PSPI, INTERP>(a, sm, w, w2, iz, tid, NT);
            __syncthreads();
            const uint8_t zf = a.zflag[iz];
            if (is_src ? (zf & Z_SRC) : (zf & Z_REC)) step_mig<N, PSPI, INTERP>(v, is_src, a, sm, xbuf, sacc, t, sync);
            if (zf & Z_REC) {
                if (is_src) {
#pragma unroll
                    for (int m = 0; m < 16; m++) {
                        const int x = t + T * m;
                        if (x < nmx) xbuf[x] = v[m];
                    }
                }
                __syncthreads();
                if (!is_src) {
                    const float2 *us = sm.x + (size_t)sg * PADN;
                    float *cv = reinterpret_cast<float *>(xbuf);
#pragma unroll
                    for (int m = 0; m < 16; m++) {
                        const int x = t + T * m;
                        if (x < nmx) {
                            const float2 s_ = us[x];
                            cv[x] = factor * (v[m].x * s_.x + v[m].y * s_.y);
                        }
                    }
                }
                __syncthreads();
                for (int x = tid; x < nmx; x += NT) {
                    float c = 0.f;
#pragma unroll
                    for (int s_ = 0; s_ < S; s_++) c += reinterpret_cast<const float *>(sm.x + (size_t)(S + s_) * PADN)[x];
                    atomicAdd(&img[(size_t)iz * nmx + x], c);
                }
            }
        }
    }
}

template <int N> struct NaDispatch {
    static constexpr int T = N / 16;
    static constexpr int S = (2 * T >= 256) ? 1 : (256 / (2 * T) > 8 ? 8 : 256 / (2 * T));
};

template <int N, bool PSPI, int INTERP>
int launch_atomic(const MigArgs &a, float *img, int nsm, cudaStream_t st)
{
    using SH = MigShape<N>;
    constexpr int S = NaDispatch<N>::S;
    const int threads = 2 * S * SH::T;
    const size_t smem = mig_smem_bytes<N>(PSPI, a.nref, a.nmx, 2 * S);
    auto k = wem_migrate_atomic_kernel<N, PSPI, INTERP, S>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return -1;
    int bps = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k, threads, smem) != cudaSuccess || bps < 1) return -1;
    MigArgs b = a;
    b.ngroups = (a.nshot + S - 1) / S;
    const long long items = (long long)b.ngroups * a.nwf;
    const int grid = (int)((long long)nsm * bps < items ? (long long)nsm * bps : items);
    k<<<grid > 0 ? grid : 1, threads, smem, st>>>(b, img);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <int N>
int launch_atomic_sel(int pspi, int interp, const MigArgs &a, float *img, int nsm, cudaStream_t st)
{
    if (!pspi) return launch_atomic<N, false, 0>(a, img, nsm, st);
    if (interp == 0) return launch_atomic<N, true, 0>(a, img, nsm, st);
    return launch_atomic<N, true, 1>(a, img, nsm, st);
}

}  // namespace

// Limits of the no-allocation path (everything must fit g_wem_scratch as well).
#define NA_MAX_NMX 1024
#define NA_MAX_NZ 1024
#define NA_MAX_NREF 16
#define NA_MAX_SHOTS 64

extern "C" WEM_API int wem_migrate_noalloc(const wem_params *pp, const float *vel_dev, const float *wav_dev, int nshot,
                                           const float *sx, const float *sy, const float *d_dev, float *m_dev,
                                           void *stream)
{
    if (!pp || !vel_dev || !wav_dev || !sx || !d_dev || !m_dev)
        return set_error(WEM_ERR_ARG, "wem_migrate_noalloc: null argument");
    const wem_params p = *pp;
    if (p.nt < 2 || p.nmx < 2 || p.nz < 1 || p.padt < 1 || p.padx < 1 || !(p.dt > 0) || !(p.dmx > 0) || nshot < 1)
        return set_error(WEM_ERR_ARG, "wem_migrate_noalloc: invalid grid or shot count");
    if (p.nmy != 1 || p.precision != WEM_PREC_FP32 || (p.interp != WEM_INTERP_REF && p.interp != WEM_INTERP_LINEAR))
        return set_error(WEM_ERR_SIZE, "wem_migrate_noalloc: 2-D, FP32 only");
    if (p.pspi && (p.nref < 2 || p.nref > NA_MAX_NREF))
        return set_error(WEM_ERR_ARG, "wem_migrate_noalloc: PSPI needs 2 <= nref <= 16");
    const int nkx = p.padx * p.nmx;
    if (nkx != 256 && nkx != 512 && nkx != 1024 && nkx != 2048)
        return set_error(WEM_ERR_SIZE, "wem_migrate_noalloc: padx*nmx must be 256, 512, 1024 or 2048");
    if (p.nmx > NA_MAX_NMX || p.nz > NA_MAX_NZ || nshot > NA_MAX_SHOTS)
        return set_error(WEM_ERR_SIZE, "wem_migrate_noalloc: nmx <= 1024, nz <= 1024 and nshot <= 64 at most");
    // frequency grid with the reference's float expressions (wem.c:79-89, 486-487)
    const int ntfft = (int)2 * p.padt * ((float)p.nt) / 2;
    const int nw = (int)ntfft / 2 + 1;
    int ifmax, ifmin;
    if (p.fmax * p.dt * ntfft + 1 < nw) ifmax = (int)p.fmax * p.dt * ntfft + 1;
    else ifmax = nw;
    if (p.fmin * p.dt * ntfft + 1 < ifmax) ifmin = (int)p.fmin * p.dt * ntfft;
    else ifmin = 0;
    const int nwf = ifmax - ifmin, nf = (nw - 1) * 2;
    if (nf < 2) return set_error(WEM_ERR_ARG, "wem_migrate_noalloc: trace too short");
    const float dw = 2 * 3.141592653589793 / ((float)ntfft) / p.dt;
    const float dkx = 2 * 3.141592653589793 / ((float)nkx) / p.dmx;
    const int ntw = twiddle_table_size(nkx);
    const int nref = p.pspi ? p.nref : 1;
    TableArgs ta{};
    for (int s = 0; s < nshot; s++) {
        const int gx = (int)(sx[s] - p.omx) / p.dmx;
        const int gy = (int)((sy ? sy[s] : 0.f) - p.omy) / p.dmy;
        if (gx < 0 || gx >= p.nmx || gy != 0)
            return set_error(WEM_ERR_ARG, "wem_migrate_noalloc: a source falls outside the grid");
        ta.igx_val[s] = gx;
    }
    const Layout L = noalloc_layout(p.nmx, p.nz, nref, ntw, nf, nwf, nshot);
    if (L.total > WEM_NOALLOC_SCRATCH_BYTES)
        return set_error(WEM_ERR_SIZE, "wem_migrate_noalloc: survey too large for the 24 MiB scratch array "
                                       "(tables ~12*nz*nmx B + spectra 8*nshot*nfreq*nmx B + image 4*nz*nmx B)");
    void *base = nullptr;
    int rc = scratch_for_current_device(&base);
    if (rc) return rc;
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return set_error(WEM_ERR_CUDA, "cudaDeviceGetAttribute failed");
    cudaStream_t st = (cudaStream_t)stream;
    unsigned char *sb = (unsigned char *)base;
#define NA(T, f) reinterpret_cast<T *>(sb + L.f)
    // what must start at zero: the spectra (cells without data) and the image
    if (cudaMemsetAsync(NA(float2, recv), 0, sizeof(float2) * (size_t)nshot * nwf * p.nmx, st) != cudaSuccess ||
        cudaMemsetAsync(NA(float, img), 0, sizeof(float) * (size_t)p.nz * p.nmx, st) != cudaSuccess)
        return set_error(WEM_ERR_CUDA, "cudaMemsetAsync on the scratch array failed");
    ta.vel = vel_dev;
    ta.nmx = p.nmx; ta.nz = p.nz; ta.nref = nref; ta.ntw = ntw; ta.nkx = nkx; ta.nf = nf; ta.nwf = nwf;
    ta.ifmin = ifmin; ta.ntfft = ntfft; ta.nshot = nshot; ta.lmx = p.nmx > 100 ? 30 : 0;
    ta.oz = p.oz; ta.dz = p.dz; ta.sz = p.sz; ta.gz = p.gz; ta.dw = dw;
    ta.po = NA(float, po); ta.pd = NA(float, pd); ta.vref = NA(float, vref); ta.slow2 = NA(float, slow2); ta.wlin = NA(float, wlin);
    ta.taper = NA(float, taper); ta.srec = NA(float, srec); ta.ssrc = NA(float, ssrc);
    ta.sel = NA(uint8_t, sel); ta.zflag = NA(uint8_t, zflag); ta.twid = NA(float2, twid); ta.wtab = NA(float2, wtab);
    ta.igx = NA(int, igx); ta.tbase = NA(int64_t, tbase); ta.wbase = NA(int64_t, wbase);
    noalloc_tables_kernel<<<p.nz + 64, 256, 0, st>>>(ta);
    if (cudaGetLastError() != cudaSuccess) return set_error(WEM_ERR_CUDA, "table kernel launch failed");
    if (nwf > 0) {
        SpectraArgs sa{};
        sa.d = wav_dev; sa.ntr = 1; sa.nt = p.nt < nf ? p.nt : nf; sa.ld = p.nt; sa.ntfft = nf; sa.ifmin = ifmin;
        sa.nwf = nwf;
        sa.out_base = NA(int64_t, wbase); sa.out_fstride = 1; sa.wtab = NA(float2, wtab);
        sa.scale = NA(float, ssrc); sa.out = NA(float2, srcw);
        if (launch_spectra(sa, st)) return set_error(WEM_ERR_CUDA, "wavelet spectrum launch failed");
        sa.d = d_dev; sa.ntr = nshot * p.nmx; sa.out_base = NA(int64_t, tbase); sa.out_fstride = p.nmx;
        sa.scale = NA(float, srec); sa.out = NA(float2, recv);
        if (launch_spectra(sa, st)) return set_error(WEM_ERR_CUDA, "trace spectra launch failed");
        MigArgs a{};
        a.nmx = p.nmx; a.nz = p.nz; a.nref = nref; a.nwf = nwf; a.ifmin = ifmin; a.nshot = nshot;
        a.dw = dw; a.dz = p.dz; a.dkx = dkx; a.inv_n = 1.0f / (float)nkx;
        a.recv = NA(float2, recv); a.srcw = NA(float2, srcw); a.igx = NA(int, igx); a.vref = NA(float, vref);
        a.slow2 = NA(float, slow2);
        a.po = NA(float, po); a.pd = NA(float, pd); a.selb = NA(uint8_t, sel); a.wlin = NA(float, wlin);
        a.taper = NA(float, taper); a.zflag = NA(uint8_t, zflag); a.twid = NA(float2, twid); a.slots = nullptr;
        int r2 = -1;
        switch (nkx) {
        case 256: r2 = launch_atomic_sel<256>(p.pspi, p.interp, a, NA(float, img), nsm, st); break;
        case 512: r2 = launch_atomic_sel<512>(p.pspi, p.interp, a, NA(float, img), nsm, st); break;
        case 1024: r2 = launch_atomic_sel<1024>(p.pspi, p.interp, a, NA(float, img), nsm, st); break;
        case 2048: r2 = launch_atomic_sel<2048>(p.pspi, p.interp, a, NA(float, img), nsm, st); break;
        }
        if (r2) return set_error(WEM_ERR_CUDA, "migration kernel launch failed");
    }
    if (launch_transpose(NA(float, img), p.nz, p.nmx, m_dev, st)) return set_error(WEM_ERR_CUDA, "transpose launch failed");
#undef NA
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return set_error(WEM_ERR_CUDA, cudaGetErrorString(e));
    return WEM_OK;
}
