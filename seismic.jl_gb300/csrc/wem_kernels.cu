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
#include <string.h>

#include "wem_kernels.cuh"

namespace gbwem {

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
            s_d[i][k] = (tr < a.ntr && ts < a.nt) ? a.d[(size_t)tr * (a.ld ? a.ld : a.nt) + ts] : 0.f;
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
// m[x][iz] = sum over slots of (sum - compensation), compensated, fixed order; one output
// per thread on tiles of 32 x by 8 z, so that the [iz][x] reads coalesce and enough loads are in
// flight (16 slots ahead per thread, the additions still in slot order), and the [x][iz] writes
// go through a transposed shared tile.
__global__ void __launch_bounds__(256) wem_image_reduce_kernel(const float2 *slots, int nslots, int nz, int nmx,
                                                               float *m)
{
    __shared__ float tile[8][33];
    const int x0 = blockIdx.x * 32, z0 = blockIdx.y * 8;
    const int lx = threadIdx.x & 31, ly = threadIdx.x >> 5;  // 32 x 8
    const size_t plane = (size_t)nz * nmx;
    const int iz = z0 + ly, x = x0 + lx;
    float s = 0.f, c = 0.f;
    if (iz < nz && x < nmx) {
        const float2 *p = slots + (size_t)iz * nmx + x;
#pragma unroll 16
        for (int q = 0; q < nslots; q++) {
            const float2 e = p[(size_t)q * plane];
            const float val = __fsub_rn(e.x, e.y);
            const float y = __fsub_rn(val, c);
            const float tt = __fadd_rn(s, y);
            c = __fsub_rn(__fsub_rn(tt, s), y);
            s = tt;
        }
    }
    tile[ly][lx] = s;
    __syncthreads();
    const int wx = x0 + (threadIdx.x >> 3), wz = z0 + (threadIdx.x & 7);
    if (wx < nmx && wz < nz) m[(size_t)wx * nz + wz] = tile[threadIdx.x & 7][threadIdx.x >> 3];
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

// ---------------------------------------------------------------- dispatch over the row length
#define WEM_SWITCH_N(nkx, CALL)            \
    switch (nkx) {                         \
    case 32: return CALL(32);              \
    case 64: return CALL(64);              \
    case 128: return CALL(128);            \
    case 256: return CALL(256);            \
    case 512: return CALL(512);            \
    case 1024: return CALL(1024);          \
    case 2048: return CALL(2048);          \
    case 4096: return CALL(4096);          \
    default: return -1;                    \
    }

// The phase tables of the paired form for every (frequency, depth): one CTA per (depth,
// frequency), entries as build_tables makes them (phase_entry, the same FP32 operations),
// references some point of the depth takes only. out: [nwf][nz][nref][phs].
// f64 = 1 (the split16 form): the entries in FP64 (phase_entry_fp64, as build_tables<F64>).
__global__ void __launch_bounds__(256) wem_phase_tables_kernel(const MigArgs a, int half, int phs, float2 *out, int f64)
{
    const int iz = blockIdx.x, iwi = blockIdx.y;
    const float w = __fmul_rn((float)(a.ifmin + iwi), a.dw);
    const float w2 = __fmul_rn(w, w);
    const unsigned long long used = ref_mask(a, iz);
    const float *sl = a.slow2 + (size_t)iz * a.nref;
    for (int r = 0; r < a.nref; r++) {
        if (!((used >> r) & 1ull)) continue;
        const float slow2 = sl[r];
        float2 *o = out + (((size_t)iwi * a.nz + iz) * a.nref + r) * phs;
        if (f64) {
            const double vr = a.vref64[(size_t)iz * a.nref + r], inv_n = 1.0 / (double)a.nlog;
            for (int kk = threadIdx.x; kk < half; kk += blockDim.x)
                o[kk] = phase_entry_fp64((double)w, vr, __dmul_rn((double)kk, a.dkx64), (double)a.dz, inv_n);
        } else {
            for (int kk = threadIdx.x; kk < half; kk += blockDim.x)
                o[kk] = phase_entry(w2, slow2, __fmul_rn(a.dkx, (float)kk), a.dz, a.inv_n);
        }
    }
}

// one bounded mbarrier wait that nothing completes (the waits of the tensor-core stages)
__global__ void wem_wait_probe_kernel(int *timed_out)
{
    __shared__ uint64_t mb;
    if (threadIdx.x == 0) {
        mbar_init(smem_u32(&mb), 1);
        mbar_init_fence();
        *timed_out = mbar_wait_bounded(smem_u32(&mb), 0) ? 0 : 1;
    }
}

int launch_wait_probe(int *timed_out, cudaStream_t st)
{
    wem_wait_probe_kernel<<<1, 32, 0, st>>>(timed_out);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// FP32 FMA throughput probe: 8 independent multiply-add chains per thread, 32 warps per
// SM, `iters` x 64 FMAs per thread. The result is stored only under a condition that the
// chains never meet, so that the compiler keeps every FMA.
__global__ void __launch_bounds__(512) wem_fma_probe_kernel(float *out, int iters)
{
    float a[8];
#pragma unroll
    for (int j = 0; j < 8; j++) a[j] = 1e-3f * (float)(threadIdx.x + j);
    const float b = 0.9999999f, c = 1e-7f;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < 8; u++)
#pragma unroll
            for (int j = 0; j < 8; j++) a[j] = fmaf(a[j], b, c);
    }
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < 8; j++) s += a[j];
    if (s == -1.f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

int launch_fma_probe(float *out, int iters, int grid, cudaStream_t st)
{
    wem_fma_probe_kernel<<<grid, 512, 0, st>>>(out, iters);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_phase_tables(int half, int phs, const MigArgs &a, float2 *out, cudaStream_t st, int f64)
{
    if (a.nz < 1 || a.nwf < 1) return 0;
    wem_phase_tables_kernel<<<dim3(a.nz, a.nwf), 256, 0, st>>>(a, half, phs, out, f64);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int migrate_config(int nkx, int wide, int pspi, int interp, int nmx, int nref, int *S, int *threads, size_t *smem,
                   int form)
{
#define CALL(N) mig_launch<N>(wide, pspi, interp, nref, nmx, nullptr, 0, 0, S, threads, smem, nullptr, form)
    WEM_SWITCH_N(nkx, CALL)
#undef CALL
}

int migrate_max_grid(int nkx, int wide, int pspi, int interp, int nmx, int nref, int *bps, int form)
{
    int S, th;
    size_t smem;
#define CALL(N) mig_launch<N>(wide, pspi, interp, nref, nmx, nullptr, 0, 0, &S, &th, &smem, bps, form)
    WEM_SWITCH_N(nkx, CALL)
#undef CALL
}

int launch_migrate(int nkx, int wide, int pspi, int interp, const MigArgs &a, int grid, cudaStream_t st, int form)
{
    int S, th;
    size_t smem;
#define CALL(N) mig_launch<N>(wide, pspi, interp, a.nref, a.nmx, &a, grid, st, &S, &th, &smem, nullptr, form)
    WEM_SWITCH_N(nkx, CALL)
#undef CALL
}

// IEEE binary16 bits of x, round to nearest even (|x| < 65504; subnormals kept)
static uint16_t half_bits(double x)
{
    const uint16_t sign = x < 0 ? 0x8000u : 0u;
    x = fabs(x);
    if (x == 0.0) return sign;
    int e;
    const double m = frexp(x, &e);  // x = m 2^e, m in [0.5, 1)
    if (e - 1 >= -14) {
        double q = nearbyint(ldexp(m, 11));  // 11 significant bits
        if (q == 2048.0) {
            q = 1024.0;
            e++;
        }
        return (uint16_t)(sign | ((e - 1 + 15) << 10) | ((int)q - 1024));
    }
    return (uint16_t)(sign | (int)nearbyint(ldexp(x, 24)));  // multiples of 2^-24 (1024 -> smallest normal)
}

static double half_value(uint16_t h)
{
    const int ex = (h >> 10) & 0x1f, mant = h & 0x3ff;
    const double v = ex == 0 ? ldexp((double)mant, -24) : ldexp(1024.0 + mant, ex - 25);
    return (h & 0x8000u) ? -v : v;
}

// The W operands of the split16 DFT stages as they sit in shared memory (layout of
// wem_tc.cuh): real form of the radix-16 and radix-8 DFT matrices for both signs,
// each split into fp16 hi = rn(w) and lo = rn(w - hi) from double precision values,
// stored K-major (row n = output component, K = input component) in 8x8 core matrices.
void tc_w_table_host(uint16_t *out)
{
    memset(out, 0, 10240);
    int off = 0;
    for (int R : { 16, 8 }) {
        const int K = 2 * R;  // fp16 per row, also the number of rows
        for (int dir = 0; dir < 2; dir++) {
            const double sgn = dir == 0 ? -1.0 : 1.0;
            uint16_t *hi = out + off / 2, *lo = out + (off + 2 * K * K) / 2;  // off in bytes
            for (int q = 0; q < R; q++)
                for (int r = 0; r < R; r++) {
                    const double ang = sgn * 6.283185307179586476925286766559 * (double)((r * q) % R) / R;
                    const double c = cos(ang), sn = sin(ang);
                    // W[k][n]: k = 2r + (0 re, 1 im) input, n = 2q + (0 re, 1 im) output
                    const double wv[2][2] = { { c, sn }, { -sn, c } };  // [k parity][n parity]
                    for (int kp = 0; kp < 2; kp++)
                        for (int np = 0; np < 2; np++) {
                            const int k = 2 * r + kp, n = 2 * q + np;
                            const int e = (n / 8) * (8 * K) + (k / 8) * 64 + (n % 8) * 8 + (k % 8);  // fp16 index
                            const uint16_t h = half_bits(wv[kp][np]);
                            hi[e] = h;
                            lo[e] = half_bits(wv[kp][np] - half_value(h));
                        }
                }
            off += 4 * K * K;  // hi and lo, K*K fp16 each
        }
    }
}

int model_config(int nkx, int pspi, int nmx, int nref, int *S, int *threads, size_t *smem, int blu)
{
#define CALL(N) model_launch<N>(pspi, 0, 0, nref, nmx, nullptr, nullptr, 0, 0, S, threads, smem, nullptr, blu)
    WEM_SWITCH_N(nkx, CALL)
#undef CALL
}

int model_max_grid(int nkx, int pspi, int interp, int exact, int nmx, int nref, int *bps, int blu)
{
    int S, th;
    size_t smem;
#define CALL(N) model_launch<N>(pspi, interp, exact, nref, nmx, nullptr, nullptr, 0, 0, &S, &th, &smem, bps, blu)
    WEM_SWITCH_N(nkx, CALL)
#undef CALL
}

int launch_model(int nkx, int pspi, int interp, int exact, const MigArgs &a, const BornArgs &b, int grid,
                 cudaStream_t st, int blu)
{
    int S, th;
    size_t smem;
#define CALL(N) model_launch<N>(pspi, interp, exact, a.nref, a.nmx, &a, &b, grid, st, &S, &th, &smem, nullptr, blu)
    WEM_SWITCH_N(nkx, CALL)
#undef CALL
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
    dim3 grid((nmx + 31) / 32, (nz + 7) / 8);
    wem_image_reduce_kernel<<<grid, 256, 0, st>>>(slots, nslots, nz, nmx, m);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
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
