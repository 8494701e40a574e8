// wem_step.cuh -- device building blocks of one depth step, shared by the kernels of
// wem_kernels.cu and wem_noalloc.cu: phase tables, the shared-memory layout of a
// CTA, the PSPI selection, the migration step and the modelling step.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>

#include "wem_fft.cuh"
#include "wem_internal.h"
#include "wem_tc.cuh"

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

// The same entry built in FP64 (the split16 form's tables): s = w^2 / vref^2 - kx^2 with
// w the FP32 frequency of the kernels, vref and kx in double, the square root and the
// sine/cosine (or the evanescent exponential) in double, rounded to FP32 once at the end.
// Explicit roundings keep the table kernel and the in-CTA builder bit-identical.
__device__ __forceinline__ float2 phase_entry_fp64(double wd, double vr, double kx, double dz, double inv_n)
{
    const double s = __dsub_rn(__ddiv_rn(__dmul_rn(wd, wd), __dmul_rn(vr, vr)), __dmul_rn(kx, kx));
    double re, im;
    if (s >= 0.0) {
        sincos(__dmul_rn(__dsqrt_rn(s), dz), &im, &re);
    } else {
        re = exp(-__dmul_rn(__dmul_rn(0.2, __dsqrt_rn(-s)), fabs(dz)));
        im = 0.0;
    }
    return make_float2(__double2float_rn(__dmul_rn(re, inv_n)), __double2float_rn(__dmul_rn(im, inv_n)));
}

// One reference's FP64-built table (entries kk = tid, tid + nth, ... < half), out of line so
// that its double-precision code does not weigh on the registers of the kernels' hot loops
// (it runs only where a CTA builds its own split16 tables).
static __device__ __noinline__ void phase_table_fp64(float2 *ph, int half, double wd, double vr, double dkx, double dz,
                                              double inv_n, int tid, int nth)
{
    for (int kk = tid; kk < half; kk += nth) ph[kk] = phase_entry_fp64(wd, vr, __dmul_rn((double)kk, dkx), dz, inv_n);
}

__device__ __forceinline__ void kahan_add(float2 *slot, float v, float2 s)
{
    const float y = __fsub_rn(v, s.y);
    const float t = __fadd_rn(s.x, y);
    s.y = __fsub_rn(__fsub_rn(t, s.x), y);
    s.x = t;
    *slot = s;
}
__device__ __forceinline__ void kahan_add(float2 *slot, float v) { kahan_add(slot, v, *slot); }

// ------------------------------------------------------------------ shared pieces
template <int N> struct MigShape {
    static constexpr int T = N / 16;           // threads per row team
    static constexpr int HALF = N / 2 + 1;     // phase-table entries per reference
    static constexpr int PHS = N / 2 + 2;      // phase-table stride: a multiple of 16 bytes
    static constexpr int PADN = pad16(N);      // exchange buffer length (float2)
    static constexpr int TW = fft_tw_size<N>();
    static constexpr int TWP = (TW + 1) & ~1;  // keep 16-byte alignment of what follows
};

// Shared-memory views of one CTA: twiddles, phase tables, split-step correction, one
// exchange buffer per team; PSPI CTAs also hold one N-sample selection accumulator per
// team (each thread owning its 16 positions), the depth's selection bytes and
// interpolation weights.
// entries of a team's PSPI selection accumulator: thread t owns entries m*T + t for the
// live positions x = t + T*m < nmx only (the padding is never selected)
template <int N> __host__ __device__ constexpr int sel_entries(int nmx)
{
    return (nmx + N / 16 - 1) / (N / 16) * (N / 16);
}

// Phase-table stride (float2, even: 16-byte aligned tables). Rows of N = nkx samples hold
// N/2 + 1 entries; rows whose transform length L = nkx is not a power of two run on
// N-point transforms with N >= 2L - 1 (Bluestein's chirp form, BLU) and hold L/2 + 1 <=
// N/4 + 1 entries.
template <int N, bool BLU> __host__ __device__ constexpr int ph_stride() { return BLU ? N / 4 + 2 : MigShape<N>::PHS; }

// float2 entries of the phase tables, kept even so that what follows stays 16-byte aligned
template <int N, bool BLU = false> __host__ __device__ constexpr int ph_entries(bool pspi, int nref)
{
    return (pspi ? nref : 1) * ph_stride<N, BLU>();
}

// bytes after the selection rows that the tensor-core stages use (split16 mode):
// the W operands, one mbarrier and 4 floats of reduction scratch per team, the TMEM
// base address and the abort flag
__host__ __device__ constexpr int tc_extra_bytes(int teams) { return 10240 + 8 * teams + 16 * teams + 16; }

// paired: the teams' acc rows are N + 2-sample spectrum buffers (step_mig_paired) instead of
// selection accumulators, and the direct-sum table (N/2 + 1 entries) and the depth's list
// of points taken whole follow the selection bytes.
template <int N> __host__ __device__ constexpr int wdot_entries() { return (N / 2 + 2) & ~1; }

template <int N, bool PSPI, bool BLU = false> struct Smem {
    static constexpr int PHS = ph_stride<N, BLU>();
    float2 *tw, *ph, *corr, *x, *acc;
    uint8_t *selb;
    float *wl;
    float2 *wd;      // paired form: e^{+2 pi i e / N}, e = 0 .. N/2
    int *wpos;       // paired form: count and positions of the points taken whole
    char *tcx;       // split16 mode: the tensor-core region (128-byte aligned)
    int acc_stride;  // float2 per team in acc
    __device__ Smem(float4 *raw, int nref, int nmx, int teams, bool paired = false)
    {
        using SH = MigShape<N>;
        tw = reinterpret_cast<float2 *>(raw);
        ph = tw + SH::TWP;
        corr = ph + ph_entries<N, BLU>(PSPI, nref);
        x = corr + (PSPI ? 0 : ((nmx + 1) & ~1));
        acc = x + (size_t)teams * SH::PADN;
        acc_stride = PSPI ? (paired ? N + 2 : sel_entries<N>(nmx)) : 0;
        wl = reinterpret_cast<float *>(acc + (size_t)teams * acc_stride);
        selb = reinterpret_cast<uint8_t *>(wl + (PSPI ? ((nmx + 3) & ~3) : 0));
        const size_t off = (size_t)(selb + (PSPI ? ((nmx + 15) & ~15) : 0) - reinterpret_cast<uint8_t *>(raw));
        wd = reinterpret_cast<float2 *>(reinterpret_cast<char *>(raw) + off);
        wpos = reinterpret_cast<int *>(wd + wdot_entries<N>());
        tcx = reinterpret_cast<char *>(raw) + ((off + 127) & ~(size_t)127);
    }
};

// shared-memory footprint (bytes) of one CTA with `teams` row teams
template <int N>
__host__ __device__ constexpr size_t mig_smem_bytes(bool pspi, int nref, int nmx, int teams, bool tc = false,
                                                    bool paired = false, bool blu = false)
{
    using SH = MigShape<N>;
    const size_t base =
        sizeof(float2) * ((size_t)SH::TWP + (size_t)(blu ? ph_entries<N, true>(pspi, nref) : ph_entries<N>(pspi, nref)) + (size_t)(pspi ? 0 : ((nmx + 1) & ~1)) +
                          (size_t)teams * SH::PADN +
                          (pspi ? (size_t)teams * (paired ? (size_t)N + 2 : (size_t)sel_entries<N>(nmx)) : 0)) +
        (pspi ? sizeof(float) * (size_t)((nmx + 3) & ~3) + (size_t)((nmx + 15) & ~15) : 0);
    if (paired) return base + sizeof(float2) * (size_t)wdot_entries<N>() + sizeof(int) * 8;
    return tc ? ((base + 127) & ~(size_t)127) + (size_t)tc_extra_bytes(teams) : base;
}

// references some grid point of depth iz takes its wavefield from (bit r)
__device__ __forceinline__ unsigned long long ref_mask(const MigArgs &a, int iz)
{
    return a.refmask ? a.refmask[iz] : ~0ull;
}

// references some grid point of depth iz takes whole (complex) in the nearest-lower mode
// (vref2 - vref1 <= 10 there, wem.c:457-458); the others give real parts only
__device__ __forceinline__ unsigned long long cx_mask(const MigArgs &a, int iz)
{
    return a.cxmask ? a.cxmask[iz] : ~0ull;
}

// Tables of depth step iz at angular frequency w (all threads of the CTA):
// PSPI: one phase table per reference velocity and the depth's selection row;
// split-step: the phase table of the mean slowness and the correction
// exp(i w pd dz) * taper (wem.c:326, 353-359).
// F64 (split16 PSPI): the phase tables in FP64 (phase_entry_fp64).
template <int N, bool PSPI, int INTERP, bool BLU = false, bool F64 = false>
__device__ __forceinline__ void build_tables(const MigArgs &a, const Smem<N, PSPI, BLU> &sm, float w, float w2, int iz,
                                             int tid, int nthreads)
{
    const int HALF = BLU ? a.nlog / 2 + 1 : MigShape<N>::HALF;
    if (PSPI) {
        const float *sl = a.slow2 + (size_t)iz * a.nref;
        const unsigned long long used = ref_mask(a, iz);
        for (int r = 0; r < a.nref; r++) {
            if (!((used >> r) & 1ull)) continue;  // no grid point takes this reference
            const float slow2 = sl[r];
            float2 *ph = sm.ph + (size_t)r * sm.PHS;
            if constexpr (F64) {
                phase_table_fp64(ph, HALF, (double)w, a.vref64[(size_t)iz * a.nref + r], a.dkx64, (double)a.dz,
                                 1.0 / (double)a.nlog, tid, nthreads);
            } else {
                for (int kk = tid; kk < HALF; kk += nthreads)
                    ph[kk] = phase_entry(w2, slow2, __fmul_rn(a.dkx, (float)kk), a.dz, a.inv_n);
            }
        }
        const uint8_t *sr = a.selb + (size_t)iz * a.nmx;
        for (int x = tid; x < a.nmx; x += nthreads) sm.selb[x] = sr[x];
        if (INTERP == 1) {
            const float *wr = a.wlin + (size_t)iz * a.nmx;
            for (int x = tid; x < a.nmx; x += nthreads) sm.wl[x] = wr[x];
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

// |k| of position m of thread t: k = t + T*m is at most N/2 exactly for m < 8 (or
// m == 8, t == 0, where both forms give N/2), and the folded index N - k is T*(16-m) - t.
template <int N> __device__ __forceinline__ int kfold(int t, int m)
{
    constexpr int T = N / 16;
    return m < 8 ? t + T * m : T * (16 - m) - t;
}

// |k| (phase-table index) of position m of thread t for a transform of length L: k for
// k <= L/2, L - k above (the reference's kx of wem.c:340-341, 430-431); positions k >= L
// of an N-point row carrying a shorter transform (BLU) hold zeros and read entry 0.
template <int N, bool BLU> __device__ __forceinline__ int kidx(int t, int m, int L)
{
    if constexpr (!BLU) {
        return kfold<N>(t, m);
    } else {
        const int k = t + (N / 16) * m;
        return k < L ? (2 * k <= L ? k : L - k) : 0;
    }
}

// The row transform of the depth step. Rows of N = nkx samples: the N-point FFT, the
// spectrum at k = t + T*m. BLU: a transform of length L = a.nlog (not a power of two) as
// circular convolutions of length N >= 2L - 1 (Bluestein, IEEE Trans. Audio Electroacoust.
// 18 (1970); chirp b[n] = e^{i pi n^2 / L}, nk = (n^2 + k^2 - (k - n)^2) / 2):
//   forward  Z[k] = sum_n (x[n] conj b[n]) b[k - n] = X[k] b[k]   (k < L; zero above),
//   inverse  x[n] = b[n] sum_k W[k] conj b[n - k],  W[k] = U[k] b[k].
// The spectrum is kept as Z = X b: a pointwise multiplier P[|k|] maps Z to U b, so the
// chirps between the two transforms cancel and each one is two N-point FFTs around a
// multiply by G/N (a.bfft, G = FFT_N of b placed at j and N - j) or its conjugate.
// a.chirp holds b[n] for n < L (built in FP64 on the host). Unnormalised like the FFT:
// the 1/L of the pair is in the phase tables.
template <int N, int DIR, bool TC, bool BLU>
__device__ __forceinline__ void xform(float2 (&v)[16], float2 *xbuf, const float2 *tw, int t, unsigned sync,
                                      TcTeam *tc, const MigArgs &a)
{
    if constexpr (!BLU) {
        fft_row<N, DIR, TC>(v, xbuf, tw, t, sync, tc);
    } else {
        constexpr int T = N / 16;
        const int L = a.nlog;
        if constexpr (DIR < 0) {
#pragma unroll
            for (int m = 0; m < 16; m++) {
                const int x = t + T * m;
                v[m] = x < L ? cmulc(v[m], __ldg(a.chirp + x)) : make_float2(0.f, 0.f);
            }
        }
        fft_row<N, -1>(v, xbuf, tw, t, sync);
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const float2 G = __ldg(a.bfft + t + T * m);
            v[m] = DIR < 0 ? cmul(v[m], G) : cmulc(v[m], G);
        }
        fft_row<N, +1>(v, xbuf, tw, t, sync);
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const int k = t + T * m;
            if (k >= L) v[m] = make_float2(0.f, 0.f);
            else if (DIR > 0) v[m] = cmul(v[m], __ldg(a.chirp + k));
        }
    }
}

// The thread's selection bytes of the current depth (from shared memory), four per
// register: bits 0-6 iref1, bit 7 set where the reference interpolates
// (vref2 - vref1 > 10, wem.c:454); positions beyond nmx get 0x7f, which matches no
// reference. Linear mode also loads the weight of iref2 (= iref1 + 1 there).
template <int N, int INTERP, bool PSPI, bool BLU = false>
__device__ __forceinline__ void load_sel(const Smem<N, PSPI, BLU> &sm, int nmx, int t, uint32_t (&selp)[4], float (&wl)[16])
{
    constexpr int T = N / 16;
#pragma unroll
    for (int q = 0; q < 4; q++) selp[q] = 0;
#pragma unroll
    for (int m = 0; m < 16; m++) {
        const int x = t + T * m;
        const uint32_t b = x < nmx ? sm.selb[x] : 0x7fu;
        selp[m >> 2] |= b << (8 * (m & 3));
        wl[m] = (INTERP == 1 && x < nmx) ? sm.wl[x] : 0.f;
    }
}

// Weight of reference r at position m, as the migration applies it after the
// inverse FFTs (wem.c:450-460); `re_only` reports the real-part truncation of
// linear_interp's float return (wem.c:473-478).
template <int INTERP>
__device__ __forceinline__ float sel_weight(const uint32_t (&selp)[4], const float (&wl)[16], int m, int r, bool &re_only)
{
    const uint32_t b = (selp[m >> 2] >> (8 * (m & 3))) & 0xffu;
    const int i1 = (int)(b & 0x7fu);
    const bool interp = (b & 0x80u) != 0;
    re_only = (INTERP == 0) && interp;
    if (INTERP == 0 || !interp) return r == i1 ? 1.f : 0.f;
    return r == i1 ? 1.f - wl[m] : (r == i1 + 1 ? wl[m] : 0.f);
}

// One depth step of the migration direction (extrap1f adj, wem.c:236-242): PSPI or
// split-step on the team's row v (x-domain, x = t + T*m), in place. CONJ selects
// -dz (the source, and every row of the reference's modelling). Called by active
// teams only; `sync` is the team's barrier id (teams of 64+ threads) or warp mask.
// TC (split16 mode): the FFTs run their DFT stages on the tensor cores; the row is
// scaled by a power of two into the operands' range first and back at the end.
// used: the references in use at this depth (ref_mask); the others are skipped.
// step_mig_tail is everything after the forward transform (v holds the spectrum at
// k = t + T*m; inv_s undoes the split16 row scaling), step_mig the whole step.
template <int N, bool PSPI, int INTERP, bool TC = false, bool BLU = false>
__device__ __forceinline__ void step_mig_tail(float2 (&v)[16], bool conj, const MigArgs &a, const Smem<N, PSPI, BLU> &sm,
                                              float2 *xbuf, float2 *sacc, int t, unsigned sync, TcTeam *tc,
                                              unsigned long long used, float inv_s)
{
    constexpr int T = N / 16;
    if (PSPI) {
        // sacc: this team's selection accumulator; thread t owns entries m*T + t
        uint32_t selp[4];
#pragma unroll
        for (int q = 0; q < 4; q++) selp[q] = 0;
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const int x = t + T * m;
            selp[m >> 2] |= (x < a.nmx ? (uint32_t)sm.selb[x] : 0x7fu) << (8 * (m & 3));
        }
        uint32_t i1p[4];  // the 16 positions' lower reference, four per word
#pragma unroll
        for (int q = 0; q < 4; q++) i1p[q] = selp[q] & 0x7f7f7f7fu;
        for (int r = 0; r < a.nref; r++) {
            if (!((used >> r) & 1ull)) continue;  // CTA-uniform
            const float2 *ph = sm.ph + (size_t)r * sm.PHS;
            float2 u[16];
#pragma unroll
            for (int m = 0; m < 16; m++) {
                const float2 P = ph[kidx<N, BLU>(t, m, a.nlog)];
                u[m] = conj ? cmulc(v[m], P) : cmul(v[m], P);
            }
            xform<N, +1, TC, BLU>(u, xbuf, sm.tw, t, sync, tc, a);
            if constexpr (INTERP == 0) {
                // the nearest-lower wavefield, whole or its real part (wem.c:454-459, 477):
                // the positions that take reference r, found four at a time
                const uint32_t rr = (uint32_t)r * 0x01010101u;
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const uint32_t eq = __vcmpeq4(i1p[q], rr);
                    if (eq == 0u) continue;
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        const int m = 4 * q + j;
                        if ((eq >> (8 * j)) & 1u) {
                            const bool interp = ((selp[q] >> (8 * j + 7)) & 1u) != 0;
                            sacc[m * T + t] = interp ? make_float2(u[m].x, 0.f) : u[m];
                        }
                    }
                }
            } else {
#pragma unroll
                for (int m = 0; m < 16; m++) {
                    const uint32_t b = (selp[m >> 2] >> (8 * (m & 3))) & 0xffu;
                    const int i1 = (int)(b & 0x7fu);
                    const bool interp = (b & 0x80u) != 0;
                    float2 *dst = sacc + m * T + t;
                    if (!interp) {
                        if (r == i1) *dst = u[m];
                    } else if (r == i1) {
                        const float w1 = 1.f - sm.wl[t + T * m];
                        *dst = make_float2(u[m].x * w1, u[m].y * w1);
                    } else if (r == i1 + 1) {
                        const float w2 = sm.wl[t + T * m];
                        const float2 q = *dst;
                        *dst = make_float2(q.x + u[m].x * w2, q.y + u[m].y * w2);
                    }
                }
            }
        }
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const int x = t + T * m;
            v[m] = x < a.nmx ? (TC ? cscale(sacc[m * T + t], inv_s) : sacc[m * T + t]) : make_float2(0.f, 0.f);
        }
    } else {
        float2 acc[16];
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const float2 P = sm.ph[kidx<N, BLU>(t, m, a.nlog)];
            acc[m] = conj ? cmulc(v[m], P) : cmul(v[m], P);
        }
        xform<N, +1, TC, BLU>(acc, xbuf, sm.tw, t, sync, tc, a);
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const int x = t + T * m;
            if constexpr (TC) acc[m] = cscale(acc[m], inv_s);
            v[m] = x < a.nmx ? (conj ? cmulc(acc[m], sm.corr[x]) : cmul(acc[m], sm.corr[x])) : make_float2(0.f, 0.f);
        }
    }
}

template <int N, bool PSPI, int INTERP, bool TC = false, bool BLU = false>
__device__ __forceinline__ void step_mig(float2 (&v)[16], bool conj, const MigArgs &a, const Smem<N, PSPI, BLU> &sm,
                                         float2 *xbuf, float2 *sacc, int t, unsigned sync, TcTeam *tc = nullptr,
                                         unsigned long long used = ~0ull)
{
    constexpr int T = N / 16;
    float inv_s = 1.f;
    if constexpr (TC) {
        float s;
        row_scale<T>(v, tc->red, t, sync, s, inv_s);
#pragma unroll
        for (int m = 0; m < 16; m++) v[m] = cscale(v[m], s);
    }
    xform<N, -1, TC, BLU>(v, xbuf, sm.tw, t, sync, tc, a);  // v now holds the spectrum at k = t + T*m
    step_mig_tail<N, PSPI, INTERP, TC, BLU>(v, conj, a, sm, xbuf, sacc, t, sync, tc, used, inv_s);
}

// e^{+2 pi i e / N}, e in [0, N), from the table of e in [0, N/2]
template <int N> __device__ __forceinline__ float2 wpow(const float2 *wd, int e)
{
    if (e <= N / 2) return wd[e];
    const float2 w = wd[N - e];
    return make_float2(w.x, -w.y);
}

// The PSPI migration step of the nearest-lower mode (INTERP = 0, FP32) with the real
// parts of two reference wavefields taken from one inverse transform.
// Where vref2 - vref1 > 10 a grid point keeps Re(dref[iref1]) only (wem.c:454-455 through
// linear_interp's float return, wem.c:473-478), so a reference r whose every taker is such
// a point needs only Re(IFFT(a Q_r)) = IFFT(X_r), X_r[k] = (a[k] Q_r[k] + conj(a[-k] Q_r[-k]))/2
// (a the row's spectrum, Q_r the phase, which depends on |k| only). X_r is Hermitian, so
// IFFT(X_r1 + i X_r2) = Re(dref[r1]) + i Re(dref[r2]): with p = a[k], q = conj(a[-k]),
//     z[k] = (p (Q1 + i Q2) + q (conj Q1 + i conj Q2)) / 2.
// References taken whole somewhere (cx) and an odd one left over get a transform of their
// own, as in step_mig. The spectrum is kept in the team's buffer spec (N samples) so that
// every thread can read a[-k]; the selected row builds up in v.
// At a depth with at most WHOLE_MAX points taken whole (wpos) every reference is paired,
// and the imaginary parts at those points are direct sums.
// First part: the forward transform, its spectrum to spec. The second part
// (paired_inverse) follows a barrier that makes spec and the depth's tables visible.
template <int N>
__device__ __forceinline__ void paired_forward(float2 (&v)[16], float2 *xbuf, float2 *spec, const float2 *tw, int t,
                                               unsigned sync)
{
    constexpr int T = N / 16;
    fft_row<N, -1>(v, xbuf, tw, t, sync);  // v: the spectrum at k = t + T*m
#pragma unroll
    for (int m = 0; m < 16; m++) spec[t + T * m] = v[m];
    if (t == 0) spec[N] = v[0];  // a[N] = a[0]: a[-k] = spec[N - k] needs no wrap
}

template <int N>
__device__ __forceinline__ void paired_inverse(float2 (&v)[16], bool conj, const MigArgs &a, const Smem<N, true> &sm,
                                               float2 *xbuf, const float2 *spec, int t, unsigned sync,
                                               unsigned long long used, unsigned long long cx)
{
    constexpr int T = N / 16;
    uint32_t selp[4];
#pragma unroll
    for (int q = 0; q < 4; q++) selp[q] = 0;
#pragma unroll
    for (int m = 0; m < 16; m++) {
        const int x = t + T * m;
        selp[m >> 2] |= (x < a.nmx ? (uint32_t)sm.selb[x] : 0x7fu) << (8 * (m & 3));
    }
    uint32_t i1p[4];
#pragma unroll
    for (int q = 0; q < 4; q++) i1p[q] = selp[q] & 0x7f7f7f7fu;
#pragma unroll
    for (int m = 0; m < 16; m++) v[m] = make_float2(0.f, 0.f);  // positions >= nmx stay 0
    used &= a.nref >= 64 ? ~0ull : ((1ull << a.nref) - 1ull);
    unsigned long long ro = used & ~cx, whole = used & cx;  // CTA-uniform
    while (ro | whole) {
        int r1, r2 = -1;
        if (ro) {
            r1 = __ffsll((long long)ro) - 1;
            ro &= ro - 1ull;
            if (ro) {
                r2 = __ffsll((long long)ro) - 1;
                ro &= ro - 1ull;
            }
        } else {
            r1 = __ffsll((long long)whole) - 1;
            whole &= whole - 1ull;
        }
        const float2 *ph1 = sm.ph + (size_t)r1 * MigShape<N>::PHS;
        float2 u[16];
        if (r2 < 0) {
#pragma unroll
            for (int m = 0; m < 16; m++) {
                const float2 P = ph1[kfold<N>(t, m)];
                const float2 p = spec[t + T * m];
                u[m] = conj ? cmulc(p, P) : cmul(p, P);
            }
        } else {
            // 2 z: the factor 1/2 is applied to the selected values
            const float2 *ph2 = sm.ph + (size_t)r2 * MigShape<N>::PHS;
            const float2 *sq = spec + N - t;  // a[-k] = sq[-T*m], k = t + T*m
#pragma unroll
            for (int m = 0; m < 16; m++) {
                const int kf = kfold<N>(t, m);
                float2 Q1 = ph1[kf], Q2 = ph2[kf];
                if (conj) {
                    Q1.y = -Q1.y;
                    Q2.y = -Q2.y;
                }
                const float2 p = spec[t + T * m];
                const float2 qm = sq[-T * m];
                const float2 q = make_float2(qm.x, -qm.y);
                const float2 M = make_float2(Q1.x - Q2.y, Q1.y + Q2.x);   // Q1 + i Q2
                const float2 Pc = make_float2(Q1.x + Q2.y, Q2.x - Q1.y);  // conj Q1 + i conj Q2
                u[m] = cadd(cmul(p, M), cmul(q, Pc));
            }
        }
        fft_row<N, +1>(u, xbuf, sm.tw, t, sync);
        const uint32_t rr1 = (uint32_t)r1 * 0x01010101u;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const uint32_t eq = __vcmpeq4(i1p[q], rr1);
            if (eq == 0u) continue;
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int m = 4 * q + j;
                if ((eq >> (8 * j)) & 1u) {
                    const bool re = r2 >= 0 || ((selp[q] >> (8 * j + 7)) & 1u) != 0;
                    v[m] = re ? make_float2(r2 >= 0 ? 0.5f * u[m].x : u[m].x, 0.f) : u[m];
                }
            }
        }
        if (r2 >= 0) {
            const uint32_t rr2 = (uint32_t)r2 * 0x01010101u;
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const uint32_t eq = __vcmpeq4(i1p[q], rr2);
                if (eq == 0u) continue;
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int m = 4 * q + j;
                    if ((eq >> (8 * j)) & 1u) v[m] = make_float2(0.5f * u[m].y, 0.f);
                }
            }
        }
    }
    // Points taken whole at a depth that has at most WHOLE_MAX of them: their references were
    // paired like the others (real parts), and the imaginary part is the direct sum
    // Im dref_r[x] = Im sum_k a[k] Q_r[k] e^{+2 pi i k x / N} over the team, in a fixed order.
    const int nj = sm.wpos[0];  // CTA-uniform
    if (nj > 0) {
        constexpr int NW = T >= 32 ? T / 32 : 1;  // partial sums per team
        const unsigned lanes = T >= 32 ? 0xffffffffu : sync;
        float *scr = reinterpret_cast<float *>(xbuf);  // free after the last inverse transform
        for (int j = 0; j < nj; j++) {
            const int xj = sm.wpos[1 + j];
            const float2 *ph = sm.ph + (size_t)(sm.selb[xj] & 0x7f) * MigShape<N>::PHS;
            // sum_m b_m W^(e0 + m c) = W^e0 (...((b_15 z + b_14) z + ...) z + b_0), z = W^c:
            // e0 = t xj, c = T xj (mod N); W^e = e^{+2 pi i e / N} from the half table
            const float2 z = wpow<N>(sm.wd, (T * xj) & (N - 1));
            float2 h = make_float2(0.f, 0.f);
#pragma unroll
            for (int m = 15; m >= 0; m--) {
                const int kf = kfold<N>(t, m);
                const float2 P = ph[kf];
                const float2 b = conj ? cmulc(spec[t + T * m], P) : cmul(spec[t + T * m], P);
                h = cadd(cmul(h, z), b);
            }
            const float2 w0 = wpow<N>(sm.wd, (t * xj) & (N - 1));
            float acc = h.x * w0.y + h.y * w0.x;  // Im(h W^e0)
#pragma unroll
            for (int off = (T >= 32 ? 16 : T / 2); off > 0; off >>= 1) acc += __shfl_xor_sync(lanes, acc, off);
            if ((t & 31) == 0) scr[j * NW + (t >> 5)] = acc;
        }
        team_sync<T>(sync);
        for (int j = 0; j < nj; j++) {
            const int xj = sm.wpos[1 + j];
            if (xj % T == t) {
                float im = 0.f;
                for (int w = 0; w < NW; w++) im += scr[j * NW + w];
                const int mj = xj / T;
#pragma unroll
                for (int m = 0; m < 16; m++)
                    if (m == mj) v[m].y = im;
            }
        }
        team_sync<T>(sync);  // the sums are read before the exchange buffer is reused
    }
}

template <int N>
__device__ __forceinline__ void step_mig_paired(float2 (&v)[16], bool conj, const MigArgs &a, const Smem<N, true> &sm,
                                                float2 *xbuf, float2 *spec, int t, unsigned sync,
                                                unsigned long long used, unsigned long long cx)
{
    paired_forward<N>(v, xbuf, spec, sm.tw, t, sync);
    team_sync<N / 16>(sync);  // the whole spectrum is in spec
    paired_inverse<N>(v, conj, a, sm, xbuf, spec, t, sync, used, cx);
}

// The depth's PSPI tables from the precomputed phase tables (a.ptab [nwf][nz][nref][PHS]):
// the phase tables of the references in use, the padded selection row, the linear weights
// (INTERP = 1) and the list of points taken whole (PAIR), copied by every thread of the
// CTA with 16-byte asynchronous copies (cp.async); the caller waits (cp_async_wait_all) and
// synchronises the CTA before reading them.
__device__ __forceinline__ void cp_async16(void *dst, const void *src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

template <int N, int INTERP, bool PAIR, bool BLU = false>
__device__ __forceinline__ void copy_tables_async(const MigArgs &a, const Smem<N, true, BLU> &sm, int iwi, int iz, int tid,
                                                  int nthreads, unsigned long long used)
{
    constexpr int PHS = Smem<N, true, BLU>::PHS, CH = PHS / 2;  // 16-byte chunks per table
    const float4 *src = reinterpret_cast<const float4 *>(a.ptab + ((size_t)iwi * a.nz + iz) * a.nref * PHS);
    float4 *dst = reinterpret_cast<float4 *>(sm.ph);
    used &= (a.nref >= 64 ? ~0ull : ((1ull << a.nref) - 1ull));
    while (used) {
        const int r = __ffsll((long long)used) - 1;
        used &= used - 1ull;
        for (int c = tid; c < CH; c += nthreads) cp_async16(dst + (size_t)r * CH + c, src + (size_t)r * CH + c);
    }
    const int nsel = (a.nmx + 15) / 16;
    const float4 *ss = reinterpret_cast<const float4 *>(a.selbp + (size_t)iz * nsel * 16);
    for (int c = tid; c < nsel; c += nthreads) cp_async16(reinterpret_cast<float4 *>(sm.selb) + c, ss + c);
    if (INTERP == 1) {
        const int nwl = (a.nmx + 3) / 4;
        const float4 *ws = reinterpret_cast<const float4 *>(a.wlinp + (size_t)iz * nwl * 4);
        for (int c = tid; c < nwl; c += nthreads) cp_async16(reinterpret_cast<float4 *>(sm.wl) + c, ws + c);
    }
    if (PAIR && tid < 2)
        cp_async16(reinterpret_cast<float4 *>(sm.wpos) + tid, reinterpret_cast<const float4 *>(a.wpos + (size_t)iz * WPOS_STRIDE) + tid);
    cp_async_commit();
}
template <int N, int INTERP, bool PAIR, bool BLU = false>
__device__ __forceinline__ void copy_tables_async(const MigArgs &a, const Smem<N, true, BLU> &sm, int iwi, int iz, int tid,
                                                  int nthreads)
{
    copy_tables_async<N, INTERP, PAIR, BLU>(a, sm, iwi, iz, tid, nthreads, ref_mask(a, iz));
}

// The same tables with the bulk-copy (TMA) engine: one thread issues one cp.async.bulk per
// contiguous piece (each used reference's phase table, the selection row, the linear
// weights, the list of points taken whole) -- this GPU's own global memory into this CTA's
// shared memory, no multicast -- and they complete on the CTA's mbarrier `mbar` with the
// byte count armed first. Every piece starts 16-byte aligned on both sides and is a
// multiple of 16 bytes long (the table stride, the padded selection and weight rows). The
// generic-proxy reads of the previous depth's tables are ordered before the asynchronous
// writes by the caller's barrier and the proxy fence here. Call from one thread; every
// thread then waits on the mbarrier's phase (tables_bulk_wait).
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint32_t mbar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(mbar)
                 : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t mbar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}

template <int N, int INTERP, bool PAIR, bool BLU = false>
__device__ __forceinline__ void copy_tables_bulk(const MigArgs &a, const Smem<N, true, BLU> &sm, int iwi, int iz,
                                                 unsigned long long used, uint32_t mbar)
{
    constexpr int PHS = Smem<N, true, BLU>::PHS;
    constexpr uint32_t TB = PHS * sizeof(float2);
    used &= (a.nref >= 64 ? ~0ull : ((1ull << a.nref) - 1ull));
    const uint32_t nsel = (uint32_t)((a.nmx + 15) / 16) * 16, nwl = (uint32_t)((a.nmx + 3) / 4) * 16;
    const uint32_t total = (uint32_t)__popcll(used) * TB + nsel + (INTERP == 1 ? nwl : 0u) + (PAIR ? 32u : 0u);
    fence_async_smem();
    mbar_expect_tx(mbar, total);
    const float2 *src = a.ptab + ((size_t)iwi * a.nz + iz) * a.nref * PHS;
    while (used) {
        const int r = __ffsll((long long)used) - 1;
        used &= used - 1ull;
        bulk_g2s(sm.ph + (size_t)r * PHS, src + (size_t)r * PHS, TB, mbar);
    }
    bulk_g2s(sm.selb, a.selbp + (size_t)iz * nsel, nsel, mbar);
    if (INTERP == 1) bulk_g2s(sm.wl, a.wlinp + (size_t)iz * (nwl / 4), nwl, mbar);
    if (PAIR) bulk_g2s(sm.wpos, a.wpos + (size_t)iz * WPOS_STRIDE, 32u, mbar);
}

// Wait for the depth's bulk copies (all threads): bounded; on a timeout the error word is
// set, *abort records it (later depths stop waiting) and the kernel's end waits once more.
__device__ __forceinline__ void tables_bulk_wait(uint32_t mbar, uint32_t &phase, int *abort, int *err)
{
    if (!*abort && !mbar_wait_bounded(mbar, phase)) {
        *abort = 1;
        atomicExch(err, 2);
    }
    phase ^= 1u;
}

// One upward step of the modelling recursion (wem.c:273-274, -dz, adj=false), in
// place, active teams only.
// EXACT=false: the reference's operator -- PSPI as the migration step with -dz
// (interpolation after the inverse FFTs); split-step with the taper and the
// correction applied before the transform (wem.c:322-327).
// EXACT=true: the exact adjoint of the migration step with +dz, for least squares:
// PSPI scatters the row into the reference wavefields with the transposed
// interpolation weights before transforming, y = sum_r F^-1 conj(P_r) F (W_r^T v);
// for split-step the reference's operator already is that adjoint.
template <int N, bool PSPI, int INTERP, bool EXACT, bool BLU = false>
__device__ __forceinline__ void step_model(float2 (&v)[16], const MigArgs &a, const Smem<N, PSPI, BLU> &sm, float2 *xbuf,
                                           float2 *sacc, int t, unsigned sync, unsigned long long used = ~0ull)
{
    constexpr int T = N / 16;
    if (PSPI && !EXACT) {
        step_mig<N, PSPI, INTERP, false, BLU>(v, true, a, sm, xbuf, sacc, t, sync, nullptr, used);
        return;
    }
    float2 acc[16];
    if (!PSPI) {
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const int x = t + T * m;
            acc[m] = x < a.nmx ? cmulc(v[m], sm.corr[x]) : make_float2(0.f, 0.f);
        }
        xform<N, -1, false, BLU>(acc, xbuf, sm.tw, t, sync, nullptr, a);
#pragma unroll
        for (int m = 0; m < 16; m++) acc[m] = cmulc(acc[m], sm.ph[kidx<N, BLU>(t, m, a.nlog)]);
    } else {
        uint32_t selp[4];
        float wl[16];
        load_sel<N, INTERP, PSPI>(sm, a.nmx, t, selp, wl);
#pragma unroll
        for (int m = 0; m < 16; m++) acc[m] = make_float2(0.f, 0.f);
        for (int r = 0; r < a.nref; r++) {
            if (!((used >> r) & 1ull)) continue;  // every weight of this reference is zero
            float2 u[16];
#pragma unroll
            for (int m = 0; m < 16; m++) {
                bool re_only;
                const float wgt = sel_weight<INTERP>(selp, wl, m, r, re_only);
                u[m] = make_float2(v[m].x * wgt, re_only ? 0.f : v[m].y * wgt);
            }
            xform<N, -1, false, BLU>(u, xbuf, sm.tw, t, sync, nullptr, a);
            const float2 *ph = sm.ph + (size_t)r * sm.PHS;
#pragma unroll
            for (int m = 0; m < 16; m++) {
                const float2 q = cmulc(u[m], ph[kidx<N, BLU>(t, m, a.nlog)]);
                acc[m].x += q.x;
                acc[m].y += q.y;
            }
        }
    }
    xform<N, +1, false, BLU>(acc, xbuf, sm.tw, t, sync, nullptr, a);
#pragma unroll
    for (int m = 0; m < 16; m++) {
        const int x = t + T * m;
        v[m] = x < a.nmx ? acc[m] : make_float2(0.f, 0.f);
    }
}

// Barrier handle of a row team: a named-barrier id for teams of 64 or more threads,
// the team's lane mask within its warp otherwise.
template <int N> __device__ __forceinline__ unsigned team_sync_handle(int tid)
{
    constexpr int T = N / 16;
    if constexpr (T >= 64) return 1u + (unsigned)(tid / T);
    else if constexpr (T == 32) return 0xffffffffu;
    else return ((1u << T) - 1u) << ((tid & 31) / T * T);
}

// Barrier of a pair of row teams (2T threads starting at team 2*pair): the pair's warp
// lanes when it fits in a warp, else a named barrier (ids 8..15, above the ids
// team_sync_handle hands out to CTAs of up to 512 threads).
template <int N> __device__ __forceinline__ void team_pair_sync(int pair, int tid)
{
    constexpr int T = N / 16;
    if constexpr (2 * T <= 32) {
        constexpr unsigned lanes = (2 * T == 32) ? 0xffffffffu : ((1u << (2 * T)) - 1u);
        __syncwarp(2 * T == 32 ? lanes : lanes << ((tid & 31) / (2 * T) * (2 * T)));
    } else {
        asm volatile("bar.sync %0, %1;" ::"r"(8 + pair), "n"(2 * T) : "memory");
    }
}

}  // namespace gbwem
