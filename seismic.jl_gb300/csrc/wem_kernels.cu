// wem_kernels.cu -- device kernels of the shot-profile wave-equation migration.
//
//   wem_migrate_kernel  the hot path: for every (group of S shots, frequency) work
//                       item, the whole depth recursion of extrap1f (wem.c:206-250)
//                       with the PSPI (wem.c:380-471) or split-step (wem.c:289-378)
//                       operator and the cross-correlation imaging condition
//                       (wem.c:243-247), fused. Each wavefield row lives in the
//                       registers of a team of N/16 threads for the whole recursion;
//                       the phase tables of a depth step are built once per CTA in
//                       shared memory and shared by all its rows (source rows use
//                       their complex conjugates: -dz, wem.c:237 vs 241).
//   wem_spectra_kernel  t -> omega transform of traces restricted to the processed
//                       band (f_op adj, wem.c:480-499, and the w^2 weighting of
//                       wem.c:122-133), as a tiled direct DFT.
//   wem_image_reduce    deterministic compensated sum of the per-CTA image
//                       accumulators, written in the reference's m[ix][iz] layout.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <math.h>

#include "wem_fft.cuh"
#include "wem_internal.h"

namespace gbwem {

// ------------------------------------------------------------------ phase tables
// Table entry kk in [0, N/2] holds exp(i sqrt(s) dz)/N (propagating) or
// exp(-0.2 sqrt(-s) |dz|)/N (evanescent), s = w^2 slow^2 - kx^2, with the FP32
// operation order of wem.c:341-343 / 434-436 (no contraction). Negative
// wavenumbers share the entry of |kx|; the source row (-dz) uses the conjugate,
// which is exactly what the reference gets from sqrtf(s)*(-dz).
__device__ __forceinline__ float2 phase_entry(float w2, float slow2, float kx, float dz, float inv_n)
{
    const float s = __fsub_rn(__fmul_rn(w2, slow2), __fmul_rn(kx, kx));
    float2 P;
    if (s >= 0.f) {
        const float th = __fmul_rn(__fsqrt_rn(s), dz);
        float sn, cs;
        sincosf(th, &sn, &cs);
        P = make_float2(cs, sn);
    } else {
        const float e = expf(-__fmul_rn(__fmul_rn(0.2f, __fsqrt_rn(-s)), fabsf(dz)));
        P = make_float2(e, 0.f);
    }
    return make_float2(P.x * inv_n, P.y * inv_n);
}

__device__ __forceinline__ void kahan_add(float2 *slot, float v)
{
    float2 s = *slot;
    const float y = __fsub_rn(v, s.y);
    const float t = __fadd_rn(s.x, y);
    s.y = __fsub_rn(__fsub_rn(t, s.x), y);
    s.x = t;
    *slot = s;
}

// ------------------------------------------------------------------ migration
template <int N> struct MigShape {
    static constexpr int T = N / 16;           // threads per row team
    static constexpr int HALF = N / 2 + 1;     // phase-table entries per reference
    static constexpr int PADN = pad16(N);      // exchange buffer length (float2)
    static constexpr int TW = fft_tw_size<N>();
    static constexpr int TWP = (TW + 1) & ~1;  // keep 16-byte alignment of what follows
};

// shared-memory footprint (bytes) of one CTA
__host__ __device__ constexpr size_t mig_smem_bytes(int TWP, int HALF, int PADN, int nph, int ncorr, int teams)
{
    return sizeof(float2) * ((size_t)TWP + (size_t)nph * HALF + (size_t)((ncorr + 1) & ~1) + (size_t)teams * PADN);
}

template <int N, bool PSPI, int INTERP, int S>
__global__ void __launch_bounds__(2 * S * (N / 16)) wem_migrate_kernel(const MigArgs a)
{
    using SH = MigShape<N>;
    constexpr int T = SH::T, HALF = SH::HALF, PADN = SH::PADN;
    constexpr int NT = 2 * S * T;
    extern __shared__ float4 smem_raw[];
    float2 *s_tw = reinterpret_cast<float2 *>(smem_raw);
    float2 *s_ph = s_tw + SH::TWP;
    const int nph = PSPI ? a.nref : 1;
    float2 *s_corr = s_ph + (size_t)nph * HALF;           // split-step correction, [nmx]
    const int ncorr = PSPI ? 0 : ((a.nmx + 1) & ~1);
    float2 *s_x = s_corr + ncorr;                          // 2S exchange buffers

    const int tid = threadIdx.x;
    const int team = tid / T, t = tid - team * T;
    const bool is_src = team < S;
    const int sg = is_src ? team : team - S;               // shot within the group
    float2 *xbuf = s_x + (size_t)team * PADN;
    const int bar = 1 + team;

    for (int i = tid; i < SH::TW; i += NT) s_tw[i] = a.twid[i];

    float2 *slot = a.slots + (size_t)blockIdx.x * a.nz * a.nmx;
    const int nitems = a.ngroups * a.nwf;
    const int nmx = a.nmx;

    for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
        const int g = item % a.ngroups;
        const int iwi = item / a.ngroups;
        const int shot = g * S + sg;
        const bool shot_ok = shot < a.nshot;
        const int iw = a.ifmin + iwi;
        const float w = __fmul_rn((float)iw, a.dw);        // w = iw*dw, wem.c:228
        const float w2 = __fmul_rn(w, w);
        const float factor = iw == 0 ? 1.f : 2.f;          // wem.c:226-227

        // initial rows (wem.c:230-233): source spike at igx, receiver spectra
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
            __syncthreads();  // the previous step no longer reads s_ph / s_corr / s_x
            if (PSPI) {
                const float *vr = a.vref + (size_t)iz * a.nref;
                for (int e = tid; e < a.nref * HALF; e += NT) {
                    const int r = e / HALF, kk = e - r * HALF;
                    const float v_ = vr[r];
                    const float slow2 = __fdiv_rn(1.0f, __fmul_rn(v_, v_));
                    s_ph[e] = phase_entry(w2, slow2, __fmul_rn(a.dkx, (float)kk), a.dz, a.inv_n);
                }
            } else {
                const float po = a.po[iz];
                const float slow2 = __fmul_rn(po, po);
                for (int e = tid; e < HALF; e += NT)
                    s_ph[e] = phase_entry(w2, slow2, __fmul_rn(a.dkx, (float)e), a.dz, a.inv_n);
                // split-step correction exp(i w pd dz) times the taper (wem.c:353-359)
                const float *pd = a.pd + (size_t)iz * nmx;
                for (int x = tid; x < nmx; x += NT) {
                    const float th = __fmul_rn(__fmul_rn(w, pd[x]), a.dz);
                    float sn, cs;
                    sincosf(th, &sn, &cs);
                    const float tp = a.taper[x];
                    s_corr[x] = make_float2(cs * tp, sn * tp);
                }
            }
            __syncthreads();

            const uint8_t zf = a.zflag[iz];
            const bool active = is_src ? (zf & Z_SRC) : (zf & Z_REC);

            // ---- one depth step of this team's row (all teams run it; inactive
            //      rows discard the result so that barriers stay uniform)
            float2 sp[16];
#pragma unroll
            for (int m = 0; m < 16; m++) sp[m] = v[m];
            fft_row<N, -1>(sp, xbuf, s_tw, t, bar);

            float2 acc[16];
            if (PSPI) {
                uint32_t sel[16];
                float wl[16];
                const uint32_t *selr = a.sel + (size_t)iz * nmx;
                const float *wlr = a.wlin + (size_t)iz * nmx;
#pragma unroll
                for (int m = 0; m < 16; m++) {
                    const int x = t + T * m;
                    acc[m] = make_float2(0.f, 0.f);
                    sel[m] = x < nmx ? selr[x] : 0xffffu;   // never matches a reference
                    wl[m] = (INTERP == 1 && x < nmx) ? wlr[x] : 0.f;
                }
                for (int r = 0; r < a.nref; r++) {
                    const float2 *ph = s_ph + (size_t)r * HALF;
                    float2 u[16];
#pragma unroll
                    for (int m = 0; m < 16; m++) {
                        const int k = t + T * m;
                        const int kk = k <= N / 2 ? k : N - k;
                        const float2 P = ph[kk];
                        u[m] = is_src ? cmulc(sp[m], P) : cmul(sp[m], P);
                    }
                    fft_row<N, +1>(u, xbuf, s_tw, t, bar);
#pragma unroll
                    for (int m = 0; m < 16; m++) {
                        const uint32_t s_ = sel[m];
                        const int i1 = s_ & 0xff, i2 = (s_ >> 8) & 0xff;
                        const bool interp = (s_ & SEL_INTERP) != 0;
                        if (INTERP == 0) {
                            // wem.c:454-459 with linear_interp's float return (wem.c:477)
                            if (r == i1) acc[m] = interp ? make_float2(u[m].x, 0.f) : u[m];
                        } else {
                            if (!interp) {
                                if (r == i1) acc[m] = u[m];
                            } else {
                                if (r == i1) { acc[m].x += u[m].x * (1.f - wl[m]); acc[m].y += u[m].y * (1.f - wl[m]); }
                                if (r == i2) { acc[m].x += u[m].x * wl[m]; acc[m].y += u[m].y * wl[m]; }
                            }
                        }
                    }
                }
            } else {
#pragma unroll
                for (int m = 0; m < 16; m++) {
                    const int k = t + T * m;
                    const int kk = k <= N / 2 ? k : N - k;
                    const float2 P = s_ph[kk];
                    acc[m] = is_src ? cmulc(sp[m], P) : cmul(sp[m], P);
                }
                fft_row<N, +1>(acc, xbuf, s_tw, t, bar);
#pragma unroll
                for (int m = 0; m < 16; m++) {
                    const int x = t + T * m;
                    if (x < nmx) {
                        const float2 c = s_corr[x];
                        acc[m] = is_src ? cmulc(acc[m], c) : cmul(acc[m], c);
                    } else {
                        acc[m] = make_float2(0.f, 0.f);
                    }
                }
            }
            if (active) {
#pragma unroll
                for (int m = 0; m < 16; m++) {
                    const int x = t + T * m;
                    v[m] = x < nmx ? acc[m] : make_float2(0.f, 0.f);
                }
            }

            // ---- imaging condition (wem.c:243-247), summed over the group's shots
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
                    const float2 *us = s_x + (size_t)sg * PADN;
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
                float2 *srow = slot + (size_t)iz * nmx;
                for (int x = tid; x < nmx; x += NT) {
                    float c = 0.f;
#pragma unroll
                    for (int s_ = 0; s_ < S; s_++) c += reinterpret_cast<const float *>(s_x + (size_t)(S + s_) * PADN)[x];
                    kahan_add(&srow[x], c);
                }
            }
        }
    }
}

// ------------------------------------------------------------------ spectra
// out[out_base[tr] + iwi*fstride] = scale[iwi] * sum_t d[tr][t] e^{-2 pi i (ifmin+iwi) t / ntfft}
// Tile: 32 traces x 64 frequencies per CTA of 256 threads, samples staged 32 at a time.
__global__ void __launch_bounds__(256) wem_spectra_kernel(const SpectraArgs a)
{
    constexpr int TR = 32, FQ = 64, KC = 32;
    __shared__ float s_d[TR][KC + 1];
    __shared__ float2 s_w[KC][FQ];
    const int tid = threadIdx.x;
    const int tr0 = blockIdx.x * TR, f0 = blockIdx.y * FQ;
    const int tx = tid & 15, ty = tid >> 4;  // 16 x 16: 4 freqs x 2 traces each
    float2 acc[2][4];
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = make_float2(0.f, 0.f);

    for (int k0 = 0; k0 < a.nt; k0 += KC) {
        __syncthreads();
        for (int e = tid; e < TR * KC; e += 256) {
            const int i = e / KC, k = e - i * KC;
            const int tr = tr0 + i, ts = k0 + k;
            s_d[i][k] = (tr < a.ntr && ts < a.nt) ? a.d[(size_t)tr * a.nt + ts] : 0.f;
        }
        for (int e = tid; e < KC * FQ; e += 256) {
            const int k = e / FQ, f = e - k * FQ;
            const int iw = a.ifmin + f0 + f, ts = k0 + k;
            float2 wv = make_float2(0.f, 0.f);
            if (f0 + f < a.nwf && ts < a.nt) wv = a.wtab[(int)(((long long)iw * ts) % a.ntfft)];
            s_w[k][f] = wv;
        }
        __syncthreads();
#pragma unroll 8
        for (int k = 0; k < KC; k++) {
            const float d0 = s_d[ty * 2][k], d1 = s_d[ty * 2 + 1][k];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const float2 wv = s_w[k][tx * 4 + j];
                acc[0][j].x = fmaf(d0, wv.x, acc[0][j].x);
                acc[0][j].y = fmaf(d0, wv.y, acc[0][j].y);
                acc[1][j].x = fmaf(d1, wv.x, acc[1][j].x);
                acc[1][j].y = fmaf(d1, wv.y, acc[1][j].y);
            }
        }
    }
#pragma unroll
    for (int i = 0; i < 2; i++) {
        const int tr = tr0 + ty * 2 + i;
        if (tr >= a.ntr) continue;
        const int64_t base = a.out_base[tr];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int f = f0 + tx * 4 + j;
            if (f < a.nwf) {
                const float sc = a.scale[f];
                a.out[base + (int64_t)f * a.out_fstride] = make_float2(acc[i][j].x * sc, acc[i][j].y * sc);
            }
        }
    }
}

// ------------------------------------------------------------------ image reduce
// m[x][iz] = sum over slots of (sum - compensation), compensated, fixed order;
// 32x32 tiles so that both the [iz][x] reads and the [x][iz] writes coalesce.
__global__ void __launch_bounds__(256) wem_image_reduce_kernel(const float2 *slots, int nslots, int nz, int nmx,
                                                               float *m)
{
    __shared__ float tile[32][33];
    const int x0 = blockIdx.x * 32, z0 = blockIdx.y * 32;
    const int lx = threadIdx.x & 31, ly = threadIdx.x >> 5;  // 32 x 8
    const size_t plane = (size_t)nz * nmx;
    for (int j = ly; j < 32; j += 8) {
        const int iz = z0 + j, x = x0 + lx;
        float s = 0.f, c = 0.f;
        if (iz < nz && x < nmx) {
            const float2 *p = slots + (size_t)iz * nmx + x;
            for (int q = 0; q < nslots; q++) {
                const float2 e = p[(size_t)q * plane];
                const float val = __fsub_rn(e.x, e.y);
                const float y = __fsub_rn(val, c);
                const float tt = __fadd_rn(s, y);
                c = __fsub_rn(__fsub_rn(tt, s), y);
                s = tt;
            }
        }
        tile[j][lx] = s;
    }
    __syncthreads();
    for (int j = ly; j < 32; j += 8) {
        const int x = x0 + j, iz = z0 + lx;
        if (x < nmx && iz < nz) m[(size_t)x * nz + iz] = tile[lx][j];
    }
}

// ------------------------------------------------------------------ host side
int twiddle_table_size(int nkx)
{
    switch (nkx) {
    case 32: return fft_tw_size<32>();
    case 64: return fft_tw_size<64>();
    case 128: return fft_tw_size<128>();
    case 256: return fft_tw_size<256>();
    case 512: return fft_tw_size<512>();
    case 1024: return fft_tw_size<1024>();
    case 2048: return fft_tw_size<2048>();
    case 4096: return fft_tw_size<4096>();
    default: return -1;
    }
}

// per-pass tables [j mod Ns][r-1] of W_{Ns R}^{r (j mod Ns)} = e^{-2 pi i r k/(Ns R)}, double -> float
void twiddle_table_host(int nkx, float2 *out)
{
    int log2n = 0;
    while ((1 << log2n) < nkx) log2n++;
    const int npass = (log2n + 3) / 4;
    int ns = 1, off = 0;
    for (int p = 0; p < npass; p++) {
        const int R = (p < log2n / 4) ? 16 : (1 << (log2n % 4));
        if (p > 0)
            for (int k = 0; k < ns; k++)
                for (int r = 1; r < R; r++) {
                    const long long e = (long long)r * k;
                    const double ang = -6.283185307179586476925286766559 * (double)e / ((double)ns * R);
                    out[off++] = make_float2((float)cos(ang), (float)sin(ang));
                }
        ns *= R;
    }
}

template <int N> struct Dispatch {
    static constexpr int T = N / 16;
    // shots per CTA: the CTA holds 2S rows; aim at 256 threads
    static constexpr int S = (2 * T >= 256) ? 1 : (256 / (2 * T) > 8 ? 8 : 256 / (2 * T));
};

template <int N, bool PSPI, int INTERP>
static int launch_n(const MigArgs &a, int grid, size_t smem, cudaStream_t st)
{
    constexpr int S = Dispatch<N>::S;
    auto k = wem_migrate_kernel<N, PSPI, INTERP, S>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return -1;
    k<<<grid, 2 * S * (N / 16), smem, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <int N>
static int launch_sel(int pspi, int interp, const MigArgs &a, int grid, size_t smem, cudaStream_t st)
{
    if (!pspi) return launch_n<N, false, 0>(a, grid, smem, st);
    if (interp == 0) return launch_n<N, true, 0>(a, grid, smem, st);
    return launch_n<N, true, 1>(a, grid, smem, st);
}

template <int N>
static void config_n(int pspi, int nmx, int nref, int *S, int *threads, size_t *smem)
{
    using SH = MigShape<N>;
    *S = Dispatch<N>::S;
    *threads = 2 * Dispatch<N>::S * SH::T;
    *smem = mig_smem_bytes(SH::TWP, SH::HALF, SH::PADN, pspi ? nref : 1, pspi ? 0 : nmx, 2 * Dispatch<N>::S);
}

int migrate_config(int nkx, int pspi, int nmx, int nref, int *S, int *threads, size_t *smem)
{
    switch (nkx) {
    case 32: config_n<32>(pspi, nmx, nref, S, threads, smem); return 0;
    case 64: config_n<64>(pspi, nmx, nref, S, threads, smem); return 0;
    case 128: config_n<128>(pspi, nmx, nref, S, threads, smem); return 0;
    case 256: config_n<256>(pspi, nmx, nref, S, threads, smem); return 0;
    case 512: config_n<512>(pspi, nmx, nref, S, threads, smem); return 0;
    case 1024: config_n<1024>(pspi, nmx, nref, S, threads, smem); return 0;
    case 2048: config_n<2048>(pspi, nmx, nref, S, threads, smem); return 0;
    case 4096: config_n<4096>(pspi, nmx, nref, S, threads, smem); return 0;
    default: return -1;
    }
}

template <int N, bool PSPI, int INTERP>
static int occ_n(int threads, size_t smem, int *bps)
{
    constexpr int S = Dispatch<N>::S;
    auto k = wem_migrate_kernel<N, PSPI, INTERP, S>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return -1;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, k, threads, smem) == cudaSuccess ? 0 : -1;
}

template <int N>
static int occ_sel(int pspi, int interp, int threads, size_t smem, int *bps)
{
    if (!pspi) return occ_n<N, false, 0>(threads, smem, bps);
    if (interp == 0) return occ_n<N, true, 0>(threads, smem, bps);
    return occ_n<N, true, 1>(threads, smem, bps);
}

int migrate_max_grid(int nkx, int pspi, int interp, int S, int threads, size_t smem, int *bps)
{
    (void)S;
    switch (nkx) {
    case 32: return occ_sel<32>(pspi, interp, threads, smem, bps);
    case 64: return occ_sel<64>(pspi, interp, threads, smem, bps);
    case 128: return occ_sel<128>(pspi, interp, threads, smem, bps);
    case 256: return occ_sel<256>(pspi, interp, threads, smem, bps);
    case 512: return occ_sel<512>(pspi, interp, threads, smem, bps);
    case 1024: return occ_sel<1024>(pspi, interp, threads, smem, bps);
    case 2048: return occ_sel<2048>(pspi, interp, threads, smem, bps);
    case 4096: return occ_sel<4096>(pspi, interp, threads, smem, bps);
    default: return -1;
    }
}

int launch_migrate(int nkx, int pspi, int interp, int S, const MigArgs &a, int grid, cudaStream_t st)
{
    int s_, th;
    size_t smem;
    if (migrate_config(nkx, pspi, a.nmx, a.nref, &s_, &th, &smem)) return -1;
    (void)S;
    switch (nkx) {
    case 32: return launch_sel<32>(pspi, interp, a, grid, smem, st);
    case 64: return launch_sel<64>(pspi, interp, a, grid, smem, st);
    case 128: return launch_sel<128>(pspi, interp, a, grid, smem, st);
    case 256: return launch_sel<256>(pspi, interp, a, grid, smem, st);
    case 512: return launch_sel<512>(pspi, interp, a, grid, smem, st);
    case 1024: return launch_sel<1024>(pspi, interp, a, grid, smem, st);
    case 2048: return launch_sel<2048>(pspi, interp, a, grid, smem, st);
    case 4096: return launch_sel<4096>(pspi, interp, a, grid, smem, st);
    default: return -1;
    }
}

int launch_spectra(const SpectraArgs &a, cudaStream_t st)
{
    if (a.ntr <= 0 || a.nwf <= 0) return 0;
    dim3 grid((a.ntr + 31) / 32, (a.nwf + 63) / 64);
    wem_spectra_kernel<<<grid, 256, 0, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_image_reduce(const float2 *slots, int nslots, int nz, int nmx, float *m, cudaStream_t st)
{
    dim3 grid((nmx + 31) / 32, (nz + 31) / 32);
    wem_image_reduce_kernel<<<grid, 256, 0, st>>>(slots, nslots, nz, nmx, m);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace gbwem
