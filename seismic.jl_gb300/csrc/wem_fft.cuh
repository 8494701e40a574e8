// wem_fft.cuh -- register-resident row FFT for the depth-extrapolation kernels.
//
// A "team" of T = N/E threads transforms one row of N complex samples (N a power
// of two, E = 16 samples per thread). Thread t holds v[m] = row[t + T*m],
// m = 0..E-1, both in the space domain (x = t + T*m) and, after a forward
// transform, in the wavenumber domain (k = t + T*m): the last Stockham pass of the
// decimation-in-time formulation (Govindaraju et al., SC 2008) writes every
// output to the same strided position set the first pass reads from, so a
// forward transform, a pointwise multiply and an inverse transform chain without
// any data movement beyond the exchanges between passes.
//
// Pass p with radix R and span Ns (product of earlier radices), butterfly
// j in [0, N/R):  u[r] = in[j + r N/R] * W_{Ns R}^{r (j mod Ns)},  u = DFT_R(u),
//                 out[(j/Ns) Ns R + (j mod Ns) + r Ns] = u[r].
// Thread t owns butterflies j = t + T*b, b = 0..E/R-1, so its first-pass inputs
// and last-pass outputs are positions t + T*(b + r*E/R).
//
// Exchanges go through a per-team shared buffer indexed with one float2 of
// padding per 16 (pad16), which makes the stride-16 writes of the first pass
// and the strided reads of later passes bank-conflict-free. Twiddles come from
// a per-pass table laid out [j mod Ns][r-1] (see wem_twiddle_table), built in
// double precision on the host and staged in shared memory.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gbwem {

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
__device__ __forceinline__ float2 cmulc(float2 a, float2 b)
{
    return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// multiply by DIR*i  (DIR = -1 forward, +1 inverse)
template <int DIR> __device__ __forceinline__ float2 mul_i(float2 a)
{
    return DIR < 0 ? make_float2(a.y, -a.x) : make_float2(-a.y, a.x);
}

__host__ __device__ constexpr int pad16(int i) { return i + (i >> 4); }

// ---------------------------------------------------------------- small DFTs
// In place, natural order in and out: v[q] <- sum_r v[r] W_R^{rq}, W_R = e^{DIR 2 pi i / R}.
template <int DIR> __device__ __forceinline__ void dft2(float2 *v)
{
    float2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
}

template <int DIR> __device__ __forceinline__ void dft4(float2 *v)
{
    float2 s0 = cadd(v[0], v[2]), d0 = csub(v[0], v[2]);
    float2 s1 = cadd(v[1], v[3]), d1 = mul_i<DIR>(csub(v[1], v[3]));
    v[0] = cadd(s0, s1);
    v[2] = csub(s0, s1);
    v[1] = cadd(d0, d1);
    v[3] = csub(d0, d1);
}

// radix-2 split: X[k] = E[k] + W^k O[k], X[k+R/2] = E[k] - W^k O[k]
template <int DIR> __device__ __forceinline__ void dft8(float2 *v)
{
    float2 e[4] = { v[0], v[2], v[4], v[6] };
    float2 o[4] = { v[1], v[3], v[5], v[7] };
    dft4<DIR>(e);
    dft4<DIR>(o);
    const float h = 0.70710678118654752440f;
    float2 w1 = make_float2(h, DIR * h);                      // W8^1
    float2 t1 = cmul(o[1], w1);
    float2 t2 = mul_i<DIR>(o[2]);                             // W8^2 = DIR i
    float2 t3 = cmul(o[3], make_float2(-h, DIR * h));         // W8^3
    v[0] = cadd(e[0], o[0]); v[4] = csub(e[0], o[0]);
    v[1] = cadd(e[1], t1);   v[5] = csub(e[1], t1);
    v[2] = cadd(e[2], t2);   v[6] = csub(e[2], t2);
    v[3] = cadd(e[3], t3);   v[7] = csub(e[3], t3);
}

template <int DIR> __device__ __forceinline__ void dft16(float2 *v)
{
    float2 e[8], o[8];
#pragma unroll
    for (int i = 0; i < 8; i++) { e[i] = v[2 * i]; o[i] = v[2 * i + 1]; }
    dft8<DIR>(e);
    dft8<DIR>(o);
    const float c1 = 0.92387953251128675613f, s1 = 0.38268343236508977173f;
    const float h = 0.70710678118654752440f;
    float2 t[8];
    t[0] = o[0];
    t[1] = cmul(o[1], make_float2(c1, DIR * s1));
    t[2] = cmul(o[2], make_float2(h, DIR * h));
    t[3] = cmul(o[3], make_float2(s1, DIR * c1));
    t[4] = mul_i<DIR>(o[4]);
    t[5] = cmul(o[5], make_float2(-s1, DIR * c1));
    t[6] = cmul(o[6], make_float2(-h, DIR * h));
    t[7] = cmul(o[7], make_float2(-c1, DIR * s1));
#pragma unroll
    for (int k = 0; k < 8; k++) { v[k] = cadd(e[k], t[k]); v[k + 8] = csub(e[k], t[k]); }
}

template <int R, int DIR> __device__ __forceinline__ void dft(float2 *v)
{
    if constexpr (R == 2) dft2<DIR>(v);
    else if constexpr (R == 4) dft4<DIR>(v);
    else if constexpr (R == 8) dft8<DIR>(v);
    else if constexpr (R == 16) dft16<DIR>(v);
}

// ---------------------------------------------------------------- pass plan
// N = 16^a * rem, rem in {1,2,4,8}; radix-16 passes first, the remainder last.
template <int N> struct FftPlan {
    static constexpr int log2n = (N <= 1) ? 0 : 1 + FftPlan<N / 2>::log2n;
};
template <> struct FftPlan<1> { static constexpr int log2n = 0; };

template <int N> __host__ __device__ constexpr int fft_npass() { return (FftPlan<N>::log2n + 3) / 4; }
template <int N> __host__ __device__ constexpr int fft_radix(int p)
{
    return (p < FftPlan<N>::log2n / 4) ? 16 : (1 << (FftPlan<N>::log2n % 4));
}
template <int N> __host__ __device__ constexpr int fft_span(int p)
{
    int ns = 1;
    for (int q = 0; q < p; q++) ns *= fft_radix<N>(q);
    return ns;
}
// offset (in float2) of pass p's twiddles in the concatenated table
template <int N> __host__ __device__ constexpr int fft_tw_offset(int p)
{
    int off = 0;
    for (int q = 1; q < p; q++) off += fft_span<N>(q) * (fft_radix<N>(q) - 1);
    return off;
}
template <int N> __host__ __device__ constexpr int fft_tw_size() { return fft_tw_offset<N>(fft_npass<N>()); }

// Team barrier. `sync` is the team's named-barrier id (1..15; 0 is __syncthreads) for
// teams of 64 or more threads, and the team's lane mask within its warp for teams of
// a warp or less, so that teams sharing a warp synchronise independently.
template <int T> __device__ __forceinline__ void team_sync(unsigned sync)
{
    if constexpr (T <= 32) __syncwarp(sync);
    else asm volatile("bar.sync %0, %1;" ::"r"(sync), "n"(T) : "memory");
}

// The tensor-core DFT stage (wem_tc.cuh): split16 mode, teams of one warpgroup.
struct TcTeam;
template <int R, int DIR, int T>
__device__ __forceinline__ void tc_dft(float2 (&u)[16], TcTeam &tc, char *a_gen, int t, unsigned bar_id);

// One Stockham pass P of the team's row (compile-time radix and span). TC: the DFTs of
// the pass run on the tensor cores (tc describes the team's operands).
template <int N, int DIR, int P, bool TC = false>
__device__ __forceinline__ void fft_pass(float2 (&v)[16], float2 *xbuf, const float2 *tw, int t, unsigned bar_id,
                                         TcTeam *tc = nullptr)
{
    constexpr int E = 16;
    constexpr int T = N / E;
    constexpr int NP = fft_npass<N>();
    constexpr int R = fft_radix<N>(P);
    constexpr int NS = fft_span<N>(P);
    constexpr int B = E / R;
    constexpr int TWO = fft_tw_offset<N>(P);
    // For T >= 16 every exchange offset added to t (or to a pass base) is a multiple of
    // 16, and pad16(base + 16q) = pad16(base) + 17q: shared addresses are a per-thread
    // base plus a compile-time constant.
    constexpr bool FAST = T >= 16;
    const int pt = t + (t >> 4);  // pad16(t)
    float2 u[E];
    if constexpr (P == 0) {
#pragma unroll
        for (int b = 0; b < B; b++)
#pragma unroll
            for (int r = 0; r < R; r++) u[b * R + r] = v[b + r * B];
    } else {
#pragma unroll
        for (int b = 0; b < B; b++) {
            const int j = t + T * b;
#pragma unroll
            for (int r = 0; r < R; r++)
                u[b * R + r] = FAST ? xbuf[pt + (T * b + r * (N / R)) / 16 * 17] : xbuf[pad16(j + r * (N / R))];
        }
        team_sync<T>(bar_id);  // every thread has read xbuf before it is rewritten
#pragma unroll
        for (int b = 0; b < B; b++) {
            const int j = t + T * b;
            const float2 *tp = tw + TWO + (j % NS) * (R - 1);
#pragma unroll
            for (int r = 1; r < R; r++) {
                const float2 w = tp[r - 1];
                u[b * R + r] = DIR < 0 ? cmul(u[b * R + r], w) : cmulc(u[b * R + r], w);
            }
        }
    }
    if constexpr (TC) {
        tc_dft<R, DIR, T>(u, *tc, reinterpret_cast<char *>(xbuf), t, bar_id);
    } else {
#pragma unroll
        for (int b = 0; b < B; b++) dft<R, DIR>(&u[b * R]);
    }
    if constexpr (P == NP - 1) {
#pragma unroll
        for (int b = 0; b < B; b++)
#pragma unroll
            for (int r = 0; r < R; r++) v[b + r * B] = u[b * R + r];
    } else {
#pragma unroll
        for (int b = 0; b < B; b++) {
            const int j = t + T * b;
            const int base = (j / NS) * NS * R + (j % NS);
            if constexpr (FAST && NS == 1 && R == 16) {
#pragma unroll
                for (int r = 0; r < R; r++) xbuf[17 * t + r] = u[b * R + r];  // B == 1: j == t
            } else if constexpr (FAST && NS >= 16) {
                const int pb = base + (base >> 4);
#pragma unroll
                for (int r = 0; r < R; r++) xbuf[pb + r * (NS / 16) * 17] = u[b * R + r];
            } else {
#pragma unroll
                for (int r = 0; r < R; r++) xbuf[pad16(base + r * NS)] = u[b * R + r];
            }
        }
        team_sync<T>(bar_id);  // writes visible before the next pass reads
        fft_pass<N, DIR, P + 1, TC>(v, xbuf, tw, t, bar_id, tc);
    }
}

// One transform of the team's row, in registers. xbuf: the team's exchange buffer
// of pad16(N) float2. tw: the concatenated per-pass twiddle table (forward sign).
// DIR = -1 forward (e^{-i...}), +1 inverse; unnormalised.
template <int N, int DIR, bool TC = false>
__device__ __forceinline__ void fft_row(float2 (&v)[16], float2 *xbuf, const float2 *tw, int t, unsigned bar_id,
                                        TcTeam *tc = nullptr)
{
    fft_pass<N, DIR, 0, TC>(v, xbuf, tw, t, bar_id, tc);
}

}  // namespace gbwem
