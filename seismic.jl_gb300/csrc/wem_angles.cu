// wem_angles.cu -- source-side incidence angles on the GPU: the reference's
// compute_angles / extrapolate_source / ssop_source / calculate_derivatives
// (src/Imaging/c/wem.c:566-992), 2-D grids.
//
// Per frequency of the band (no time or space padding: ntfft = nt, nkx = nmx, nkz = nz):
//   1. wem_angles_extrap_kernel: the source wavefield continued down with the split-step
//      operator of ssop_source (taper, then exp(i w pd dz), FFT_x, phase with the mean
//      slowness, IFFT_x, wem.c:763-820), one CTA per frequency, the row in shared memory,
//      every depth stored: u[f][z][x].
//   2. the derivatives. The reference takes 3-D FFTs of u and inverse FFTs of i k_x A,
//      i k_z A, i k_x^left A, i k_x^right A (wem.c:822-985). The transform is separable
//      and each factor i k acts on one axis only, so IDFT3(i k_x DFT3(u)) =
//      IDFT_x(i k_x DFT_x(u)) exactly; along its axis that is a circular convolution, so
//      the host runtime (wem_api.cu, deriv_gemm) applies each derivative to all lines at
//      once as one complex GEMM against an L x L matrix built in FP64 (cuBLAS; the axes
//      have any length: nz is rarely a power of two).
//   When nmx is a power of two in [32, 2048] steps 1 and the x derivatives run on the
//   register-resident row FFT of wem_fft.cuh instead (wem_angles_extrap_fft_kernel,
//   wem_angles_xderiv_fft_kernel).
//   3. wem_angles_accum_kernel: per grid point, in frequency order,
//      ang += (180/pi) atan(|u_x| / (|u_z| + 1e-10)) and sign += +-|u| / nw, then
//      ang *= sign(sign) / (ifmax - ifmin + 1) (wem.c:675-676, 735-754).
// In 2-D the y terms vanish: u_y = 0 gives angy = 0 (the reference's value). 3-D grids
// (power-of-two nmx, nmy) continue the source with the plane passes of wem_3d.cu (mode 3)
// and take the x, y and z derivatives of every depth volume with the same GEMMs;
// wem_angles_accum3_kernel sums over batches of frequencies.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "wem_fft.cuh"
#include "wem_internal.h"
#include "wem_step.cuh"

namespace gbwem {

__device__ __forceinline__ float2 c_mul(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// wavenumber of index i on an axis of n samples: dk*i up to n/2, then -(dk*n - dk*i),
// in float without contraction (wem.c:802-803, 866-867, 905-906)
__device__ __forceinline__ float axis_k(int i, int n, float dk)
{
    return i <= n / 2 ? __fmul_rn(dk, (float)i) : -__fsub_rn(__fmul_rn(dk, (float)n), __fmul_rn(dk, (float)i));
}

// ------------------------------------------------------------------ 1. extrapolation
__global__ void __launch_bounds__(512) wem_angles_extrap_kernel(const AngleArgs a)
{
    extern __shared__ float2 sh[];
    const int nmx = a.nmx, tid = threadIdx.x, nth = blockDim.x;
    float2 *d = sh, *x = sh + nmx;
    const float2 *tw = sh + 2 * nmx;
    float2 *tws = sh + 2 * nmx;
    const int f = blockIdx.x, shot = blockIdx.y;  // one (frequency, shot of the batch) per CTA
    const int igx = a.igxs ? a.igxs[shot] : a.igx;
    const float w = __fmul_rn((float)(a.ifmin + f), a.dw);  // w = iw*dw
    const float dzs = -a.dz;                                 // extrapolate_source passes -dz
    for (int i = tid; i < nmx; i += nth) {
        tws[i] = a.twx[i];
        d[i] = i == igx ? a.srcw[f] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    for (int iz = 0; iz < a.nz; iz++) {
        float2 *urow = a.u + (((size_t)shot * a.nwf + f) * a.nz + iz) * nmx;
        const float z = __fadd_rn(a.oz, __fmul_rn(a.dz, (float)iz));
        if (!(z >= a.sz)) {  // CTA-uniform: nothing above the source
            for (int i = tid; i < nmx; i += nth) urow[i] = make_float2(0.f, 0.f);
            continue;
        }
        const float *pdr = a.pd + (size_t)iz * nmx;
        for (int i = tid; i < nmx; i += nth) {
            const float2 v = make_float2(d[i].x * a.taper[i], d[i].y * a.taper[i]);  // boundary_condition
            float sn, cs;
            sincosf(__fmul_rn(__fmul_rn(w, pdr[i]), dzs), &sn, &cs);              // cexpf(I*w*pd*dz)
            x[i] = c_mul(v, make_float2(cs, sn));
        }
        __syncthreads();
        const float po = a.po[iz];
        const float wp = __fmul_rn(__fmul_rn(w, w), __fmul_rn(po, po));
        for (int k = tid; k < nmx; k += nth) {  // forward DFT, phase shift
            float2 acc = make_float2(0.f, 0.f);
            int idx = 0;
            for (int j = 0; j < nmx; j++) {
                const float2 xv = x[j], wv = tw[idx];
                acc.x = fmaf(xv.x, wv.x, fmaf(-xv.y, wv.y, acc.x));
                acc.y = fmaf(xv.x, wv.y, fmaf(xv.y, wv.x, acc.y));
                idx += k;
                if (idx >= nmx) idx -= nmx;
            }
            const float kx = axis_k(k, nmx, a.dkx);
            const float s = __fsub_rn(__fsub_rn(wp, __fmul_rn(kx, kx)), 0.f);
            float2 L;
            if (s >= 0.f) {
                float sn, cs;
                sincosf(__fmul_rn(__fsqrt_rn(s), dzs), &sn, &cs);
                L = make_float2(cs, sn);
            } else {
                // cexpf(-0.2*sqrtf(fabs(s))*fabs(dz)): the argument is a double expression
                L = make_float2(expf((float)(-0.2 * (double)__fsqrt_rn(fabsf(s)) * (double)fabsf(dzs))), 0.f);
            }
            const float2 q = c_mul(acc, L);
            d[k] = make_float2(q.x * a.inv_sqrt_n, q.y * a.inv_sqrt_n);
        }
        __syncthreads();
        for (int i = tid; i < nmx; i += nth) {  // inverse DFT
            float2 acc = make_float2(0.f, 0.f);
            int idx = 0;
            for (int k = 0; k < nmx; k++) {
                const float2 dv = d[k], wv = tw[idx];  // conj(W^{ik})
                acc.x = fmaf(dv.x, wv.x, fmaf(dv.y, wv.y, acc.x));
                acc.y = fmaf(dv.y, wv.x, fmaf(-dv.x, wv.y, acc.y));
                idx += i;
                if (idx >= nmx) idx -= nmx;
            }
            const float2 v = make_float2(acc.x * a.inv_sqrt_n, acc.y * a.inv_sqrt_n);
            x[i] = v;
            urow[i] = v;
        }
        __syncthreads();
        float2 *t = d;  // the new row is in x
        d = x;
        x = t;
    }
}

// ------------------------------------------------------------------ 1'. FFT rows
// One team of N/16 threads per frequency: the same recursion with the row in registers.
template <int N>
__global__ void __launch_bounds__(N / 16 < 32 ? 32 : N / 16) wem_angles_extrap_fft_kernel(const AngleArgs a)
{
    constexpr int T = N / 16, TW = fft_tw_size<N>(), TWP = (TW + 1) & ~1;
    __shared__ float2 s_tw[TWP > 0 ? TWP : 2];
    __shared__ float2 s_x[pad16(N)];
    const int t = threadIdx.x;
    if (t >= T) return;  // T < 32: the rest of the warp idles
    const unsigned sync = team_sync_handle<N>(t);
    for (int i = t; i < TW; i += T) s_tw[i] = a.twx[i];
    team_sync<T>(sync);
    const int f = blockIdx.x, shot = blockIdx.y;  // one (frequency, shot of the batch) per CTA
    const int igx = a.igxs ? a.igxs[shot] : a.igx;
    const float w = __fmul_rn((float)(a.ifmin + f), a.dw);
    const float dzs = -a.dz;
    float2 v[16];
#pragma unroll
    for (int m = 0; m < 16; m++) v[m] = (t + T * m) == igx ? a.srcw[f] : make_float2(0.f, 0.f);
    for (int iz = 0; iz < a.nz; iz++) {
        float2 *urow = a.u + (((size_t)shot * a.nwf + f) * a.nz + iz) * N;
        const float z = __fadd_rn(a.oz, __fmul_rn(a.dz, (float)iz));
        if (!(z >= a.sz)) {
#pragma unroll
            for (int m = 0; m < 16; m++) urow[t + T * m] = make_float2(0.f, 0.f);
            continue;
        }
        const float *pdr = a.pd + (size_t)iz * N;
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const int x = t + T * m;
            const float tp = a.taper[x];
            float sn, cs;
            sincosf(__fmul_rn(__fmul_rn(w, pdr[x]), dzs), &sn, &cs);
            v[m] = c_mul(make_float2(v[m].x * tp, v[m].y * tp), make_float2(cs, sn));
        }
        fft_row<N, -1>(v, s_x, s_tw, t, sync);
        const float po = a.po[iz];
        const float wp = __fmul_rn(__fmul_rn(w, w), __fmul_rn(po, po));
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const int k = t + T * m;
            const float kx = axis_k(k, N, a.dkx);
            const float s = __fsub_rn(wp, __fmul_rn(kx, kx));
            float2 L;
            if (s >= 0.f) {
                float sn, cs;
                sincosf(__fmul_rn(__fsqrt_rn(s), dzs), &sn, &cs);
                L = make_float2(cs, sn);
            } else {
                L = make_float2(expf((float)(-0.2 * (double)__fsqrt_rn(fabsf(s)) * (double)fabsf(dzs))), 0.f);
            }
            const float2 q = c_mul(v[m], L);
            v[m] = make_float2(q.x * a.inv_sqrt_n, q.y * a.inv_sqrt_n);
        }
        fft_row<N, +1>(v, s_x, s_tw, t, sync);
#pragma unroll
        for (int m = 0; m < 16; m++) {
            v[m] = make_float2(v[m].x * a.inv_sqrt_n, v[m].y * a.inv_sqrt_n);
            urow[t + T * m] = v[m];
        }
    }
}

// The x derivatives of one row per team: X = FFT_x(u), then u_x = IFFT_x(i kx X) / N and
// the unnormalised u_left, u_right (wem.c:838-856, 932-950). CTA of 256 threads.
template <int N>
__global__ void __launch_bounds__(256) wem_angles_xderiv_fft_kernel(const AngleXArgs a)
{
    constexpr int T = N / 16, TEAMS = 256 / T < 1 ? 1 : 256 / T, NT = TEAMS * T;
    constexpr int TW = fft_tw_size<N>(), TWP = (TW + 1) & ~1;
    extern __shared__ float4 smem_raw[];
    float2 *s_tw = reinterpret_cast<float2 *>(smem_raw);
    float2 *s_x = s_tw + TWP;
    const int tid = threadIdx.x, team = tid / T, t = tid - team * T;
    float2 *xbuf = s_x + (size_t)team * pad16(N);
    const unsigned sync = team_sync_handle<N>(tid);
    for (int i = tid; i < TW; i += NT) s_tw[i] = a.twx[i];
    __syncthreads();
    for (long long l = (long long)blockIdx.x * TEAMS + team; l < a.nlines; l += (long long)gridDim.x * TEAMS) {
        const float2 *in = a.u + (size_t)l * N;
        float2 X[16];
#pragma unroll
        for (int m = 0; m < 16; m++) X[m] = in[t + T * m];
        fft_row<N, -1>(X, xbuf, s_tw, t, sync);
        float2 *outs[3] = { a.ux + (size_t)l * N, a.ul + (size_t)l * N, a.ur + (size_t)l * N };
#pragma unroll 1
        for (int mode = 1; mode <= 3; mode++) {
            float2 u[16];
#pragma unroll
            for (int m = 0; m < 16; m++) {
                const int k = t + T * m;
                float kx = axis_k(k, N, a.dkx);
                if (mode == 2) kx = k <= N / 2 ? 0.f : kx;
                if (mode == 3) kx = k <= N / 2 ? kx : 0.f;
                u[m] = make_float2(-kx * X[m].y, kx * X[m].x);
            }
            fft_row<N, +1>(u, xbuf, s_tw, t, sync);
            const float sc = mode == 1 ? 1.f / (float)N : 1.f;
            float2 *o = outs[mode - 1];
#pragma unroll
            for (int m = 0; m < 16; m++) o[t + T * m] = make_float2(u[m].x * sc, u[m].y * sc);
        }
    }
}

// ------------------------------------------------------------------ 2'. derivative convolutions
// A derivative along an axis of L samples (any L <= 2048) is the circular convolution of
// each line with w = IDFT_L(i k mask) * scale (the reference's 3-D transform is separable
// and i k acts on one axis). It runs on M-point rows, M the power of two >= 2L - 1: the line
// zero-padded to M, FFT_M, times H = FFT_M(g) / M with g = w placed at j and M - j (the
// M-point circular convolution then equals the L-point one on the first L outputs), inverse
// FFT_M. Up to three transfer functions (u_x, u_left, u_right) share one forward transform.
template <int M>
__device__ __forceinline__ void conv_line(const float2 (&X)[16], const float2 *H, float2 (&u)[16], float2 *xbuf,
                                          const float2 *tw, int t, unsigned sync)
{
    constexpr int T = M / 16;
#pragma unroll
    for (int m = 0; m < 16; m++) u[m] = c_mul(X[m], __ldg(H + t + T * m));
    fft_row<M, +1>(u, xbuf, tw, t, sync);
}

// Lines of L contiguous samples ([line][L]); one team of M/16 threads per line, 256 threads.
template <int M>
__global__ void __launch_bounds__(256) wem_angles_conv_rows_kernel(const AngleConvArgs a)
{
    constexpr int T = M / 16, TEAMS = 256 / T < 1 ? 1 : 256 / T, NT = TEAMS * T;
    constexpr int TW = fft_tw_size<M>(), TWP = (TW + 1) & ~1;
    extern __shared__ float4 smem_raw[];
    float2 *s_tw = reinterpret_cast<float2 *>(smem_raw);
    const int tid = threadIdx.x, team = tid / T, t = tid - team * T;
    float2 *xbuf = s_tw + TWP + (size_t)team * pad16(M);
    const unsigned sync = team_sync_handle<M>(tid);
    for (int i = tid; i < TW; i += NT) s_tw[i] = a.tw[i];
    __syncthreads();
    const int L = a.L;
    for (long long l = (long long)blockIdx.x * TEAMS + team; l < a.nlines; l += (long long)gridDim.x * TEAMS) {
        const float2 *in = a.u + (size_t)l * L;
        float2 X[16];
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const int x = t + T * m;
            X[m] = x < L ? in[x] : make_float2(0.f, 0.f);
        }
        fft_row<M, -1>(X, xbuf, s_tw, t, sync);
#pragma unroll 1
        for (int o = 0; o < a.nout; o++) {
            float2 u[16];
            conv_line<M>(X, a.H + (size_t)o * M, u, xbuf, s_tw, t, sync);
            float2 *out = a.out[o] + (size_t)l * L;
#pragma unroll
            for (int m = 0; m < 16; m++) {
                const int x = t + T * m;
                if (x < L) out[x] = u[m];
            }
        }
    }
}

// Lines strided across planes: plane p holds L rows of `cols` samples ([p][L][cols]), line
// (p, c) is column c of plane p. A CTA stages a tile of TX adjacent columns of one plane in
// shared memory with coalesced loads along the rows (row pitch TX + 1: conflict-free
// column reads), each of its TX teams transforms one column, and the results leave the
// same way. 512 threads.
template <int M>
__global__ void __launch_bounds__(512) wem_angles_conv_cols_kernel(const AngleConvArgs a)
{
    constexpr int T = M / 16, TX = 512 / T < 1 ? 1 : 512 / T, NT = TX * T, P = TX + 1;
    constexpr int TW = fft_tw_size<M>(), TWP = (TW + 1) & ~1;
    extern __shared__ float4 smem_raw[];
    float2 *s_tw = reinterpret_cast<float2 *>(smem_raw);
    float2 *s_x = s_tw + TWP;
    float2 *tile = s_x + (size_t)TX * pad16(M);
    const int tid = threadIdx.x, team = tid / T, t = tid - team * T;
    float2 *xbuf = s_x + (size_t)team * pad16(M);
    const unsigned sync = team_sync_handle<M>(tid);
    for (int i = tid; i < TW; i += NT) s_tw[i] = a.tw[i];
    const int L = a.L, cols = a.cols;
    const int ntile = (cols + TX - 1) / TX;
    const long long nplanes = a.nlines / cols;
    for (long long b = blockIdx.x; b < nplanes * ntile; b += gridDim.x) {
        const long long pl = b / ntile;
        const int c0 = (int)(b - pl * ntile) * TX;
        const size_t base = (size_t)pl * L * cols;
        __syncthreads();  // the previous tile is written out
        for (int e = tid; e < L * TX; e += NT) {
            const int z = e / TX, j = e - z * TX;
            tile[z * P + j] = c0 + j < cols ? a.u[base + (size_t)z * cols + c0 + j] : make_float2(0.f, 0.f);
        }
        __syncthreads();
        float2 X[16];
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const int z = t + T * m;
            X[m] = z < L ? tile[z * P + team] : make_float2(0.f, 0.f);
        }
        fft_row<M, -1>(X, xbuf, s_tw, t, sync);
#pragma unroll 1
        for (int o = 0; o < a.nout; o++) {
            float2 u[16];
            conv_line<M>(X, a.H + (size_t)o * M, u, xbuf, s_tw, t, sync);
#pragma unroll
            for (int m = 0; m < 16; m++) {
                const int z = t + T * m;
                if (z < L) tile[z * P + team] = u[m];  // only this team touches its column
            }
            __syncthreads();
            float2 *out = a.out[o];
            for (int e = tid; e < L * TX; e += NT) {
                const int z = e / TX, j = e - z * TX;
                if (c0 + j < cols) out[base + (size_t)z * cols + c0 + j] = tile[z * P + j];
            }
            __syncthreads();  // the tile is read out before the next output overwrites it
        }
    }
}

template <int M> static int launch_conv(const AngleConvArgs &a, int nsm, cudaStream_t st)
{
    constexpr int T = M / 16;
    constexpr int TWP = (fft_tw_size<M>() + 1) & ~1;
    if (a.cols > 1) {
        constexpr int TX = 512 / T < 1 ? 1 : 512 / T;
        const size_t smem = sizeof(float2) * ((size_t)TWP + (size_t)TX * pad16(M) + (size_t)a.L * (TX + 1));
        if (cudaFuncSetAttribute(wem_angles_conv_cols_kernel<M>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess)
            return -1;
        const long long tiles = a.nlines / a.cols * ((a.cols + TX - 1) / TX);
        const long long grid = tiles < (long long)nsm * 8 ? tiles : (long long)nsm * 8;
        wem_angles_conv_cols_kernel<M><<<(unsigned)(grid > 0 ? grid : 1), TX * T, smem, st>>>(a);
    } else {
        constexpr int TEAMS = 256 / T < 1 ? 1 : 256 / T;
        const size_t smem = sizeof(float2) * ((size_t)TWP + (size_t)TEAMS * pad16(M));
        if (cudaFuncSetAttribute(wem_angles_conv_rows_kernel<M>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess)
            return -1;
        long long blocks = (a.nlines + TEAMS - 1) / TEAMS;
        if (blocks > (long long)nsm * 16) blocks = (long long)nsm * 16;
        wem_angles_conv_rows_kernel<M><<<(unsigned)(blocks > 0 ? blocks : 1), 256, smem, st>>>(a);
    }
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int angles_conv_length(int L)
{
    if (L < 1 || L > 2048) return 0;
    int m = 32;
    while (m < 2 * L - 1) m *= 2;
    return m;
}

int launch_angles_conv(const AngleConvArgs &a, int nsm, cudaStream_t st)
{
    if (a.nlines <= 0) return 0;
    if (a.cols > 1 && a.nlines % a.cols) return -2;
    switch (angles_conv_length(a.L)) {
    case 32: return launch_conv<32>(a, nsm, st);
    case 64: return launch_conv<64>(a, nsm, st);
    case 128: return launch_conv<128>(a, nsm, st);
    case 256: return launch_conv<256>(a, nsm, st);
    case 512: return launch_conv<512>(a, nsm, st);
    case 1024: return launch_conv<1024>(a, nsm, st);
    case 2048: return launch_conv<2048>(a, nsm, st);
    case 4096: return launch_conv<4096>(a, nsm, st);
    default: return -2;
    }
}

// ------------------------------------------------------------------ 3. accumulation
// One thread per grid point (x, z), frequencies in order; out [nmx][nz].
__global__ void __launch_bounds__(256) wem_angles_accum_kernel(const AngleAccumArgs a)
{
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= (long long)a.nmx * a.nz) return;
    const int z = (int)(p / a.nmx), x = (int)(p - (long long)z * a.nmx);
    const size_t plane = (size_t)a.nmx * a.nz, off = (size_t)z * a.nmx + x;
    float ang = 0.f, sgn = 0.f;
    for (int f = 0; f < a.nwf; f++) {
        const size_t q = (size_t)f * plane + off;
        const float2 u = a.u[q], sx = a.ux[q], ul = a.ul[q], ur = a.ur[q];
        const float2 sz = a.uzp ? make_float2(a.uzp[q + (size_t)f * plane], a.uzp[q + (size_t)f * plane + plane]) : a.uz[q];
        const float au = hypotf(u.x, u.y);
        const float ratio = hypotf(sx.x, sx.y) / (hypotf(sz.x, sz.y) + 1e-10f);
        ang += (float)(57.295779513082323 * (double)atanf(ratio));  // (180/PI)*atanf(...) in double
        const float s = hypotf(ul.x, ul.y) >= hypotf(ur.x, ur.y) ? au : -au;
        sgn += s / (float)a.nw;
    }
    a.angx[(size_t)x * a.nz + z] = ang * ((sgn >= 0.f ? 1.f : -1.f) / (float)a.nfreq_div);
    if (a.angy) a.angy[(size_t)x * a.nz + z] = 0.f;  // 2-D: u_y = 0
}

// 3-D (wem.c:735-754 with both lateral axes): per grid point (cell, z), the frequencies of
// a batch in order, added to the running sums of the earlier batches.
__global__ void __launch_bounds__(256) wem_angles_accum3_kernel(const AngleAccum3Args a)
{
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long np = (long long)a.n * a.nz;
    if (p >= np) return;
    const int z = (int)(p / a.n), cell = (int)(p - (long long)z * a.n);
    const size_t vol = (size_t)a.nz * a.n, off = (size_t)z * a.n + cell, o = (size_t)cell * a.nz + z;
    float ax = a.sum[o], sx = a.sum[np + o], ay = a.sum[2 * np + o], sy = a.sum[3 * np + o];
    for (int f = 0; f < a.nwf; f++) {
        const size_t q = (size_t)f * vol + off;
        const float au = hypotf(a.u[q].x, a.u[q].y);
        const float az = hypotf(a.uz[q].x, a.uz[q].y) + 1e-10f;
        ax += (float)(57.295779513082323 * (double)atanf(hypotf(a.ux[q].x, a.ux[q].y) / az));
        ay += (float)(57.295779513082323 * (double)atanf(hypotf(a.uy[q].x, a.uy[q].y) / az));
        sx += (hypotf(a.lx[q].x, a.lx[q].y) >= hypotf(a.rx[q].x, a.rx[q].y) ? au : -au) / (float)a.nw;
        sy += (hypotf(a.ly[q].x, a.ly[q].y) >= hypotf(a.ry[q].x, a.ry[q].y) ? au : -au) / (float)a.nw;
    }
    if (a.last) {
        a.angx[o] = ax * ((sx >= 0.f ? 1.f : -1.f) / (float)a.nfreq_div);
        a.angy[o] = ay * ((sy >= 0.f ? 1.f : -1.f) / (float)a.nfreq_div);
    } else {
        a.sum[o] = ax;
        a.sum[np + o] = sx;
        a.sum[2 * np + o] = ay;
        a.sum[3 * np + o] = sy;
    }
}

int launch_angles_accum3(const AngleAccum3Args &a, cudaStream_t st)
{
    const long long n = (long long)a.n * a.nz;
    wem_angles_accum3_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_angles_extrap(const AngleArgs &a, cudaStream_t st)
{
    const size_t smem = sizeof(float2) * 3 * (size_t)a.nmx;
    if (cudaFuncSetAttribute(wem_angles_extrap_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return -1;
    wem_angles_extrap_kernel<<<dim3(a.nwf, a.nshot > 0 ? a.nshot : 1), 512, smem, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <int N> static int launch_fft_paths(const AngleArgs &a, const AngleXArgs &x, int which, cudaStream_t st)
{
    constexpr int T = N / 16, TEAMS = 256 / T < 1 ? 1 : 256 / T;
    constexpr int TWP = (fft_tw_size<N>() + 1) & ~1;
    if (which == 0) {
        wem_angles_extrap_fft_kernel<N><<<dim3(a.nwf, a.nshot > 0 ? a.nshot : 1), T < 32 ? 32 : T, 0, st>>>(a);
    } else {
        const size_t smem = sizeof(float2) * ((size_t)TWP + (size_t)TEAMS * pad16(N));
        if (cudaFuncSetAttribute(wem_angles_xderiv_fft_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess)
            return -1;
        long long blocks = (x.nlines + TEAMS - 1) / TEAMS;
        if (blocks > 65535LL * 16) blocks = 65535LL * 16;
        wem_angles_xderiv_fft_kernel<N><<<(unsigned)blocks, 256, smem, st>>>(x);
    }
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// up to 2048: the extrapolation kernel keeps its row buffers in static shared memory
bool angles_fft_supported(int nmx) { return nmx >= 32 && nmx <= 2048 && (nmx & (nmx - 1)) == 0; }

// which = 0: the extrapolation, 1: the x derivatives
int launch_angles_fft(const AngleArgs &a, const AngleXArgs &x, int which, cudaStream_t st)
{
    switch (a.nmx) {
    case 32: return launch_fft_paths<32>(a, x, which, st);
    case 64: return launch_fft_paths<64>(a, x, which, st);
    case 128: return launch_fft_paths<128>(a, x, which, st);
    case 256: return launch_fft_paths<256>(a, x, which, st);
    case 512: return launch_fft_paths<512>(a, x, which, st);
    case 1024: return launch_fft_paths<1024>(a, x, which, st);
    case 2048: return launch_fft_paths<2048>(a, x, which, st);
    default: return -2;
    }
}

// interleaved complex -> planar per entry (the layout of the real block GEMMs)
__global__ void __launch_bounds__(256) wem_planar_kernel(const float2 *in, float *out, long long entry, long long total)
{
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const long long b = e / entry, s = e - b * entry;
        const float2 v = in[e];
        out[2 * b * entry + s] = v.x;
        out[2 * b * entry + entry + s] = v.y;
    }
}

int launch_planar(const float2 *in, float *out, long long entry, long long nentries, cudaStream_t st)
{
    const long long total = entry * nentries;
    long long blocks = (total + 255) / 256;
    if (blocks > 152LL * 64) blocks = 152LL * 64;
    wem_planar_kernel<<<(unsigned)blocks, 256, 0, st>>>(in, out, entry, total);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_angles_accum(const AngleAccumArgs &a, cudaStream_t st)
{
    const long long n = (long long)a.nmx * a.nz;
    wem_angles_accum_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace gbwem
