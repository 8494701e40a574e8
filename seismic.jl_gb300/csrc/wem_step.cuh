// wem_step.cuh -- device building blocks of one depth step, shared by the kernels of
// wem_kernels.cu and wem_noalloc.cu: phase tables, the shared-memory layout of a
// CTA, the PSPI selection, the migration step and the modelling step.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
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

// ------------------------------------------------------------------ shared pieces
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

// Shared-memory views of one CTA: twiddles, phase tables, split-step correction,
// one exchange buffer per row team.
template <int N, bool PSPI> struct Smem {
    float2 *tw, *ph, *corr, *x;
    __device__ Smem(float4 *raw, int nref, int nmx)
    {
        using SH = MigShape<N>;
        tw = reinterpret_cast<float2 *>(raw);
        ph = tw + SH::TWP;
        corr = ph + (size_t)(PSPI ? nref : 1) * SH::HALF;
        x = corr + (PSPI ? 0 : ((nmx + 1) & ~1));
    }
};

// Tables of depth step iz at angular frequency w (all threads of the CTA):
// PSPI: one phase table per reference velocity; split-step: the phase table of
// the mean slowness and the correction exp(i w pd dz) * taper (wem.c:326, 353-359).
template <int N, bool PSPI>
__device__ __forceinline__ void build_tables(const MigArgs &a, const Smem<N, PSPI> &sm, float w, float w2, int iz,
                                             int tid, int nthreads)
{
    constexpr int HALF = MigShape<N>::HALF;
    if (PSPI) {
        const float *vr = a.vref + (size_t)iz * a.nref;
        for (int e = tid; e < a.nref * HALF; e += nthreads) {
            const int r = e / HALF, kk = e - r * HALF;
            const float v_ = vr[r];
            const float slow2 = __fdiv_rn(1.0f, __fmul_rn(v_, v_));
            sm.ph[e] = phase_entry(w2, slow2, __fmul_rn(a.dkx, (float)kk), a.dz, a.inv_n);
        }
    } else {
        const float po = a.po[iz];
        const float slow2 = __fmul_rn(po, po);
        for (int e = tid; e < HALF; e += nthreads)
            sm.ph[e] = phase_entry(w2, slow2, __fmul_rn(a.dkx, (float)e), a.dz, a.inv_n);
        const float *pd = a.pd + (size_t)iz * a.nmx;
        for (int x = tid; x < a.nmx; x += nthreads) {
            const float th = __fmul_rn(__fmul_rn(w, pd[x]), a.dz);
            float sn, cs;
            sincosf(th, &sn, &cs);
            const float tp = a.taper[x];
            sm.corr[x] = make_float2(cs * tp, sn * tp);
        }
    }
}

template <int N> __device__ __forceinline__ int kfold(int t, int m)
{
    const int k = t + (N / 16) * m;
    return k <= N / 2 ? k : N - k;
}

// Per-x selection data of depth iz for the thread's 16 positions.
template <int N, int INTERP>
__device__ __forceinline__ void load_sel(const MigArgs &a, int iz, int t, uint32_t (&sel)[16], float (&wl)[16])
{
    constexpr int T = N / 16;
    const uint32_t *selr = a.sel + (size_t)iz * a.nmx;
    const float *wlr = a.wlin + (size_t)iz * a.nmx;
#pragma unroll
    for (int m = 0; m < 16; m++) {
        const int x = t + T * m;
        sel[m] = x < a.nmx ? selr[x] : 0xffffu;  // 0xff never matches a reference index
        wl[m] = (INTERP == 1 && x < a.nmx) ? wlr[x] : 0.f;
    }
}

// Weight of reference r at one position, as the migration applies it after the
// inverse FFTs (wem.c:450-460); `re_only` reports the real-part truncation of
// linear_interp's float return (wem.c:473-478).
template <int INTERP>
__device__ __forceinline__ float sel_weight(uint32_t s_, float wl, int r, bool &re_only)
{
    const int i1 = s_ & 0xff, i2 = (s_ >> 8) & 0xff;
    const bool interp = (s_ & SEL_INTERP) != 0;
    re_only = (INTERP == 0) && interp;
    if (INTERP == 0 || !interp) return r == i1 ? 1.f : 0.f;
    return (r == i1 ? 1.f - wl : 0.f) + (r == i2 ? wl : 0.f);
}

// One depth step of the migration direction (extrap1f adj, wem.c:236-242): PSPI or
// split-step on the team's row v (x-domain, x = t + T*m). CONJ selects -dz (the
// source, and every row of the reference's modelling). Inactive rows keep v.
template <int N, bool PSPI, int INTERP>
__device__ __forceinline__ void step_mig(float2 (&v)[16], bool conj, bool active, const MigArgs &a,
                                         const Smem<N, PSPI> &sm, float2 *xbuf, int iz, int t, int bar)
{
    constexpr int T = N / 16, HALF = MigShape<N>::HALF;
    float2 sp[16];
#pragma unroll
    for (int m = 0; m < 16; m++) sp[m] = v[m];
    fft_row<N, -1>(sp, xbuf, sm.tw, t, bar);
    float2 acc[16];
    if (PSPI) {
        uint32_t sel[16];
        float wl[16];
        load_sel<N, INTERP>(a, iz, t, sel, wl);
#pragma unroll
        for (int m = 0; m < 16; m++) acc[m] = make_float2(0.f, 0.f);
        for (int r = 0; r < a.nref; r++) {
            const float2 *ph = sm.ph + (size_t)r * HALF;
            float2 u[16];
#pragma unroll
            for (int m = 0; m < 16; m++) {
                const float2 P = ph[kfold<N>(t, m)];
                u[m] = conj ? cmulc(sp[m], P) : cmul(sp[m], P);
            }
            fft_row<N, +1>(u, xbuf, sm.tw, t, bar);
#pragma unroll
            for (int m = 0; m < 16; m++) {
                bool re_only;
                const float wgt = sel_weight<INTERP>(sel[m], wl[m], r, re_only);
                if (INTERP == 0) {
                    // the nearest-lower wavefield, whole or its real part
                    if (wgt != 0.f) acc[m] = re_only ? make_float2(u[m].x, 0.f) : u[m];
                } else {
                    acc[m].x += u[m].x * wgt;
                    acc[m].y += u[m].y * wgt;
                }
            }
        }
    } else {
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const float2 P = sm.ph[kfold<N>(t, m)];
            acc[m] = conj ? cmulc(sp[m], P) : cmul(sp[m], P);
        }
        fft_row<N, +1>(acc, xbuf, sm.tw, t, bar);
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const int x = t + T * m;
            if (x < a.nmx) {
                const float2 c = sm.corr[x];
                acc[m] = conj ? cmulc(acc[m], c) : cmul(acc[m], c);
            }
        }
    }
    if (active) {
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const int x = t + T * m;
            v[m] = x < a.nmx ? acc[m] : make_float2(0.f, 0.f);
        }
    }
}

// One upward step of the modelling recursion (wem.c:273-274, -dz, adj=false).
// EXACT=false: the reference's operator -- PSPI as the migration step with -dz
// (interpolation after the inverse FFTs); split-step with the taper and the
// correction applied before the transform (wem.c:322-327).
// EXACT=true: the exact adjoint of the migration step with +dz, for least squares:
// PSPI scatters the row into the reference wavefields with the transposed
// interpolation weights before transforming, y = sum_r F^-1 conj(P_r) F (W_r^T v);
// for split-step the reference's operator already is that adjoint.
template <int N, bool PSPI, int INTERP, bool EXACT>
__device__ __forceinline__ void step_model(float2 (&v)[16], bool active, const MigArgs &a, const Smem<N, PSPI> &sm,
                                           float2 *xbuf, int iz, int t, int bar)
{
    constexpr int T = N / 16, HALF = MigShape<N>::HALF;
    if (PSPI && !EXACT) {
        step_mig<N, PSPI, INTERP>(v, true, active, a, sm, xbuf, iz, t, bar);
        return;
    }
    float2 acc[16];
    if (!PSPI) {
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const int x = t + T * m;
            acc[m] = x < a.nmx ? cmulc(v[m], sm.corr[x]) : make_float2(0.f, 0.f);
        }
        fft_row<N, -1>(acc, xbuf, sm.tw, t, bar);
#pragma unroll
        for (int m = 0; m < 16; m++) acc[m] = cmulc(acc[m], sm.ph[kfold<N>(t, m)]);
    } else {
        uint32_t sel[16];
        float wl[16];
        load_sel<N, INTERP>(a, iz, t, sel, wl);
#pragma unroll
        for (int m = 0; m < 16; m++) acc[m] = make_float2(0.f, 0.f);
        for (int r = 0; r < a.nref; r++) {
            float2 u[16];
#pragma unroll
            for (int m = 0; m < 16; m++) {
                bool re_only;
                const float wgt = sel_weight<INTERP>(sel[m], wl[m], r, re_only);
                u[m] = make_float2(v[m].x * wgt, re_only ? 0.f : v[m].y * wgt);
            }
            fft_row<N, -1>(u, xbuf, sm.tw, t, bar);
            const float2 *ph = sm.ph + (size_t)r * HALF;
#pragma unroll
            for (int m = 0; m < 16; m++) {
                const float2 q = cmulc(u[m], ph[kfold<N>(t, m)]);
                acc[m].x += q.x;
                acc[m].y += q.y;
            }
        }
    }
    fft_row<N, +1>(acc, xbuf, sm.tw, t, bar);
    if (active) {
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const int x = t + T * m;
            v[m] = x < a.nmx ? acc[m] : make_float2(0.f, 0.f);
        }
    }
}

}  // namespace gbwem
