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
#include "wem_step.cuh"

namespace gbwem {

// ------------------------------------------------------------------ migration
template <int N, bool PSPI, int INTERP, int S>
__global__ void __launch_bounds__(2 * S * (N / 16)) wem_migrate_kernel(const MigArgs a)
{
    using SH = MigShape<N>;
    constexpr int T = SH::T, PADN = SH::PADN;
    constexpr int NT = 2 * S * T;
    extern __shared__ float4 smem_raw[];
    const Smem<N, PSPI> sm(smem_raw, a.nref, a.nmx);

    const int tid = threadIdx.x;
    const int team = tid / T, t = tid - team * T;
    const bool is_src = team < S;
    const int sg = is_src ? team : team - S;               // shot within the group
    float2 *xbuf = sm.x + (size_t)team * PADN;
    const int bar = 1 + team;

    for (int i = tid; i < SH::TW; i += NT) sm.tw[i] = a.twid[i];

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
            __syncthreads();  // the previous step no longer reads the tables / exchange buffers
            build_tables<N, PSPI>(a, sm, w, w2, iz, tid, NT);
            __syncthreads();
            const uint8_t zf = a.zflag[iz];
            // all teams run the step (barriers stay uniform); inactive rows keep v
            step_mig<N, PSPI, INTERP>(v, is_src, is_src ? (zf & Z_SRC) : (zf & Z_REC), a, sm, xbuf, iz, t, bar);

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
                float2 *srow = slot + (size_t)iz * nmx;
                for (int x = tid; x < nmx; x += NT) {
                    float c = 0.f;
#pragma unroll
                    for (int s_ = 0; s_ < S; s_++) c += reinterpret_cast<const float *>(sm.x + (size_t)(S + s_) * PADN)[x];
                    kahan_add(&srow[x], c);
                }
            }
        }
    }
}

// ------------------------------------------------------------------ modelling (Born)
// One team per shot. Per (group of S shots, frequency): the source wavefield is
// continued down and kept at every depth in global scratch (smig, wem.c:253-265),
// then the receiver wavefield is continued up from the bottom with the image
// injected at each depth (wem.c:266-276); the surface row, divided by
// sqrt(ntfft) (wem.c:277-279), is the shot's spectrum at this frequency.
template <int N, bool PSPI, int INTERP, int S, bool EXACT>
__global__ void __launch_bounds__(S * (N / 16)) wem_model_kernel(const MigArgs a, const BornArgs b)
{
    using SH = MigShape<N>;
    constexpr int T = SH::T, PADN = SH::PADN;
    constexpr int NT = S * T;
    extern __shared__ float4 smem_raw[];
    const Smem<N, PSPI> sm(smem_raw, a.nref, a.nmx);
    const int tid = threadIdx.x;
    const int team = tid / T, t = tid - team * T;
    float2 *xbuf = sm.x + (size_t)team * PADN;
    const int bar = 1 + team;
    for (int i = tid; i < SH::TW; i += NT) sm.tw[i] = a.twid[i];

    const int nmx = a.nmx, nz = a.nz;
    float2 *smig = b.smig + ((size_t)blockIdx.x * S + team) * (size_t)nz * nmx;
    const int nitems = a.ngroups * a.nwf;
    for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
        const int g = item % a.ngroups;
        const int iwi = item / a.ngroups;
        const int shot = g * S + team;
        const bool shot_ok = shot < a.nshot;
        const int iw = a.ifmin + iwi;
        const float w = __fmul_rn((float)iw, a.dw);
        const float w2 = __fmul_rn(w, w);
        float2 v[16];
        const int igx = shot_ok ? a.igx[shot] : -1;
        const float2 sw = a.srcw[iwi];
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const int x = t + T * m;
            v[m] = (x < nmx && x == igx) ? sw : make_float2(0.f, 0.f);
        }
        // source, downward (wem.c:255-265)
        for (int iz = 0; iz < nz; iz++) {
            __syncthreads();
            build_tables<N, PSPI>(a, sm, w, w2, iz, tid, NT);
            __syncthreads();
            const bool act = (a.zflag[iz] & Z_SRC) != 0;
            step_mig<N, PSPI, INTERP>(v, true, act, a, sm, xbuf, iz, t, bar);
            float2 *row = smig + (size_t)iz * nmx;
#pragma unroll
            for (int m = 0; m < 16; m++) {
                const int x = t + T * m;
                if (x < nmx) row[x] = act ? v[m] : make_float2(0.f, 0.f);
            }
        }
        // receiver, upward with injection (wem.c:266-276)
#pragma unroll
        for (int m = 0; m < 16; m++) v[m] = make_float2(0.f, 0.f);
        for (int iz = nz - 1; iz >= 0; iz--) {
            __syncthreads();
            build_tables<N, PSPI>(a, sm, w, w2, iz, tid, NT);
            __syncthreads();
            const bool act = (a.zflag[iz] & Z_REC) != 0;
            if (act) {
                const float2 *row = smig + (size_t)iz * nmx;
                const float *mr = b.img + (size_t)iz * nmx;
#pragma unroll
                for (int m = 0; m < 16; m++) {
                    const int x = t + T * m;
                    if (x < nmx) {
                        const float mv = mr[x];
                        const float2 s_ = row[x];
                        v[m].x += mv * s_.x;
                        v[m].y += mv * s_.y;
                    }
                }
            }
            step_model<N, PSPI, INTERP, EXACT>(v, act, a, sm, xbuf, iz, t, bar);
        }
        if (shot_ok) {
            float2 *out = b.dg + ((size_t)shot * a.nwf + iwi) * nmx;
#pragma unroll
            for (int m = 0; m < 16; m++) {
                const int x = t + T * m;
                if (x < nmx) out[x] = make_float2(v[m].x * b.inv_sqt, v[m].y * b.inv_sqt);
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

// ------------------------------------------------------------------ synthesis
// out[tr][t] = sum_f Re(scale[f] * dg[in_base[tr] + f*fstride] * e^{+2 pi i (ifmin+f) t / nf}), t < nt:
// the half-spectrum inverse transform of f_op (wem.c:501-511) restricted to the
// processed band, after the w^2 weighting of wem.c:179-184.
// Tile: 32 traces x 64 samples per CTA of 256 threads, frequencies staged 32 at a time.
__global__ void __launch_bounds__(256) wem_synth_kernel(const SynthArgs a)
{
    constexpr int TR = 32, TS = 64, KC = 32;
    __shared__ float2 s_a[TR][KC + 1];
    __shared__ float2 s_w[KC][TS];
    const int tid = threadIdx.x;
    const int tr0 = blockIdx.x * TR, t0 = blockIdx.y * TS;
    const int tx = tid & 15, ty = tid >> 4;
    float acc[2][4];
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = 0.f;
    for (int f0 = 0; f0 < a.nwf; f0 += KC) {
        __syncthreads();
        for (int e = tid; e < TR * KC; e += 256) {
            const int i = e / KC, k = e - i * KC;
            const int tr = tr0 + i, f = f0 + k;
            float2 v = make_float2(0.f, 0.f);
            if (tr < a.ntr && f < a.nwf) {
                const float2 q = a.dg[a.in_base[tr] + (int64_t)f * a.in_fstride];
                const float sc = a.scale[f];
                v = make_float2(q.x * sc, q.y * sc);
            }
            s_a[i][k] = v;
        }
        for (int e = tid; e < KC * TS; e += 256) {
            const int k = e / TS, j = e - k * TS;
            const int iw = a.ifmin + f0 + k, ts = t0 + j;
            float2 wv = make_float2(0.f, 0.f);
            if (f0 + k < a.nwf && ts < a.nt) {
                const float2 q = a.wtab[(int)(((long long)iw * ts) % a.nf)];
                wv = make_float2(q.x, -q.y);  // e^{+i theta}
            }
            s_w[k][j] = wv;
        }
        __syncthreads();
#pragma unroll 8
        for (int k = 0; k < KC; k++) {
            const float2 a0 = s_a[ty * 2][k], a1 = s_a[ty * 2 + 1][k];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const float2 wv = s_w[k][tx * 4 + j];
                acc[0][j] = fmaf(a0.x, wv.x, fmaf(-a0.y, wv.y, acc[0][j]));
                acc[1][j] = fmaf(a1.x, wv.x, fmaf(-a1.y, wv.y, acc[1][j]));
            }
        }
    }
#pragma unroll
    for (int i = 0; i < 2; i++) {
        const int tr = tr0 + ty * 2 + i;
        if (tr >= a.ntr) continue;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int ts = t0 + tx * 4 + j;
            if (ts < a.nt) a.out[(size_t)tr * a.nt + ts] = acc[i][j];
        }
    }
}

// out[c][r] = in[r][c] (rows x cols), 32x32 tiles
__global__ void __launch_bounds__(256) wem_transpose_kernel(const float *in, int rows, int cols, float *out)
{
    __shared__ float tile[32][33];
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    const int lx = threadIdx.x & 31, ly = threadIdx.x >> 5;
    for (int j = ly; j < 32; j += 8) {
        const int r = r0 + j, c = c0 + lx;
        tile[j][lx] = (r < rows && c < cols) ? in[(size_t)r * cols + c] : 0.f;
    }
    __syncthreads();
    for (int j = ly; j < 32; j += 8) {
        const int c = c0 + j, r = r0 + lx;
        if (c < cols && r < rows) out[(size_t)c * rows + r] = tile[lx][j];
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

// ---------------------------------------------------------------- modelling launchers
template <int N> struct DispatchModel {
    static constexpr int T = N / 16;
    // one row team per shot; aim at 256 threads
    static constexpr int S = (T >= 256) ? 1 : (256 / T > 8 ? 8 : 256 / T);
};

template <int N>
static void model_config_n(int pspi, int nmx, int nref, int *S, int *threads, size_t *smem)
{
    using SH = MigShape<N>;
    *S = DispatchModel<N>::S;
    *threads = DispatchModel<N>::S * SH::T;
    *smem = mig_smem_bytes(SH::TWP, SH::HALF, SH::PADN, pspi ? nref : 1, pspi ? 0 : nmx, DispatchModel<N>::S);
}

int model_config(int nkx, int pspi, int nmx, int nref, int *S, int *threads, size_t *smem)
{
    switch (nkx) {
    case 32: model_config_n<32>(pspi, nmx, nref, S, threads, smem); return 0;
    case 64: model_config_n<64>(pspi, nmx, nref, S, threads, smem); return 0;
    case 128: model_config_n<128>(pspi, nmx, nref, S, threads, smem); return 0;
    case 256: model_config_n<256>(pspi, nmx, nref, S, threads, smem); return 0;
    case 512: model_config_n<512>(pspi, nmx, nref, S, threads, smem); return 0;
    case 1024: model_config_n<1024>(pspi, nmx, nref, S, threads, smem); return 0;
    case 2048: model_config_n<2048>(pspi, nmx, nref, S, threads, smem); return 0;
    case 4096: model_config_n<4096>(pspi, nmx, nref, S, threads, smem); return 0;
    default: return -1;
    }
}

template <int N, bool PSPI, int INTERP, bool EXACT>
static int model_n(const MigArgs *a, const BornArgs *b, int grid, size_t smem, cudaStream_t st, int threads, int *bps)
{
    constexpr int S = DispatchModel<N>::S;
    auto k = wem_model_kernel<N, PSPI, INTERP, S, EXACT>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return -1;
    if (bps) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, k, threads, smem) == cudaSuccess ? 0 : -1;
    k<<<grid, S * (N / 16), smem, st>>>(*a, *b);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <int N>
static int model_sel(int pspi, int interp, int exact, const MigArgs *a, const BornArgs *b, int grid, size_t smem,
                     cudaStream_t st, int threads, int *bps)
{
    if (!pspi) return model_n<N, false, 0, false>(a, b, grid, smem, st, threads, bps);
    if (exact) {
        if (interp == 0) return model_n<N, true, 0, true>(a, b, grid, smem, st, threads, bps);
        return model_n<N, true, 1, true>(a, b, grid, smem, st, threads, bps);
    }
    if (interp == 0) return model_n<N, true, 0, false>(a, b, grid, smem, st, threads, bps);
    return model_n<N, true, 1, false>(a, b, grid, smem, st, threads, bps);
}

static int model_dispatch(int nkx, int pspi, int interp, int exact, const MigArgs *a, const BornArgs *b, int grid,
                          size_t smem, cudaStream_t st, int threads, int *bps)
{
    switch (nkx) {
    case 32: return model_sel<32>(pspi, interp, exact, a, b, grid, smem, st, threads, bps);
    case 64: return model_sel<64>(pspi, interp, exact, a, b, grid, smem, st, threads, bps);
    case 128: return model_sel<128>(pspi, interp, exact, a, b, grid, smem, st, threads, bps);
    case 256: return model_sel<256>(pspi, interp, exact, a, b, grid, smem, st, threads, bps);
    case 512: return model_sel<512>(pspi, interp, exact, a, b, grid, smem, st, threads, bps);
    case 1024: return model_sel<1024>(pspi, interp, exact, a, b, grid, smem, st, threads, bps);
    case 2048: return model_sel<2048>(pspi, interp, exact, a, b, grid, smem, st, threads, bps);
    case 4096: return model_sel<4096>(pspi, interp, exact, a, b, grid, smem, st, threads, bps);
    default: return -1;
    }
}

int model_max_grid(int nkx, int pspi, int interp, int exact, int threads, size_t smem, int *bps)
{
    return model_dispatch(nkx, pspi, interp, exact, nullptr, nullptr, 0, smem, 0, threads, bps);
}

int launch_model(int nkx, int pspi, int interp, int exact, const MigArgs &a, const BornArgs &b, int grid, cudaStream_t st)
{
    int S, th;
    size_t smem;
    if (model_config(nkx, pspi, a.nmx, a.nref, &S, &th, &smem)) return -1;
    return model_dispatch(nkx, pspi, interp, exact, &a, &b, grid, smem, st, th, nullptr);
}

int launch_synth(const SynthArgs &a, cudaStream_t st)
{
    if (a.ntr <= 0 || a.nt <= 0) return 0;
    dim3 grid((a.ntr + 31) / 32, (a.nt + 63) / 64);
    wem_synth_kernel<<<grid, 256, 0, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_transpose(const float *in, int rows, int cols, float *out, cudaStream_t st)
{
    dim3 grid((cols + 31) / 32, (rows + 31) / 32);
    wem_transpose_kernel<<<grid, 256, 0, st>>>(in, rows, cols, out);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace gbwem
