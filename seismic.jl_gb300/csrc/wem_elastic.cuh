// wem_elastic.cuh -- the elastic depth kernels (see wem_elastic.cu) as templates over the row
// length N, instantiated one N per translation unit (wem_elastic_n<N>.cu) so that the build
// compiles them in parallel.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "wem_fft.cuh"
#include "wem_internal.h"
#include "wem_step.cuh"

namespace gbwem {

struct EwemArgs {
    MigArgs m;           // nmx, nz, nwf, ifmin, nshot, dw, dz, dkx, inv_n; nlog/chirp/bfft for Bluestein rows
    int nkx;             // transform length L (the row length N, or shorter on Bluestein rows)
    float gz, sz, oz;
    float inv_max_source;  // 1 / max_t |wav| / sqrtf(ntfft) (ewem.c:145)
    float inv_sqt;         // 1 / sqrtf(ntfft)
    const float *po_p, *po_s;   // [nz] layer slownesses
    const float *pd_p, *pd_s;   // [nz][nmx] slowness perturbations
    const float *vp_mean, *vs_mean;  // [nz] 1/po (the separation's velocities, ewem.c:314)
    const float *taper;         // [nmx] boundary_condition (ewem.c:533-551)
    const float2 *twid;         // FFT twiddles of N
    const float2 *srcw;         // [nwf] wavelet spectrum / sqrtf(ntfft)
    const int *igx;             // [nshot]
    const float2 *recv_x, *recv_z;  // [nshot][nwf][nmx] receiver spectra / sqrtf(ntfft) (adj)
    float2 *slots;              // adj: [2][grid][nz][nmx] (sum, compensation) of the P and S2 images
    float2 *smig;               // forward: [grid][nz][nmx] source wavefield of every depth
    const float *img_p, *img_s;  // forward: [nz][nmx] images (depth-major)
    float2 *dg_x, *dg_z;        // forward: [nshot][nwf][nmx] modelled spectra / sqrtf(ntfft)
    // per-(frequency, depth) tables of the frequencies [wbase, wbase + nwc) (wem_ewem_tables_kernel),
    // one record of EwemRec::floats floats per (frequency - wbase, depth), frequency-major
    float *tabs;
    int wbase, nwc;
    int dbuf;  // two record buffers in shared memory: the next depth's copy overlaps this depth
};

// Layout of one table record, in floats, every part a multiple of 16 bytes:
//   php[rh], phs[rh]   float2 phase entries of the P and S layer slownesses, k < L/2 + 1
//   cp[nmxp], cs[nmxp] float2 exp(i w pd dz) of the P and S slowness perturbations
//   kxp, kzp, kxs, kzs, norm [lp] each: the separation coefficients at every k < L
struct EwemRec {
    int rh, nmxp, lp;
    __host__ __device__ EwemRec(int L, int nmx) : rh(((L / 2 + 1) + 1) & ~1), nmxp((nmx + 1) & ~1), lp((L + 3) & ~3) {}
    __host__ __device__ int php() const { return 0; }
    __host__ __device__ int phs() const { return 2 * rh; }
    __host__ __device__ int cp() const { return 4 * rh; }
    __host__ __device__ int cs() const { return 4 * rh + 2 * nmxp; }
    __host__ __device__ int sep() const { return 4 * rh + 4 * nmxp; }
    __host__ __device__ int floats() const { return 4 * rh + 4 * nmxp + 5 * lp; }
};

// signed wavenumber of position k of a transform of length L: ikx < L/2. ? dkx ikx :
// -(dkx L - dkx ikx), float operations of ewem.c:414, 614
__device__ __forceinline__ float kx_signed(int k, int L, float dkx)
{
    return 2 * k < L ? __fmul_rn(dkx, (float)k) : -__fsub_rn(__fmul_rn(dkx, (float)L), __fmul_rn(dkx, (float)k));
}

// The separation coefficients of ewem.c:598-611 at wavenumber kx; `on` where the potentials
// are separated (norm >= 0.1 and w >= 20; NaN compares false, as in the reference).
struct SepCoef {
    float kxp, kzp, kxs, kzs, norm;
    bool on;
};
__device__ __forceinline__ SepCoef sep_coef(float kx, float w, float vp, float vs)
{
    SepCoef c;
    const float w2 = __fmul_rn(w, w), kx2 = __fmul_rn(kx, kx);
    const float sp = __fsub_rn(__fdiv_rn(w2, __fmul_rn(vp, vp)), kx2);
    const float ss = __fsub_rn(__fdiv_rn(w2, __fmul_rn(vs, vs)), kx2);
    float kzp = sp > 0.f ? __fsqrt_rn(sp) : 0.f;
    float kzs = ss > 0.f ? __fsqrt_rn(ss) : 0.f;
    const float np_ = __fsqrt_rn(__fadd_rn(kx2, __fmul_rn(kzp, kzp)));
    const float ns_ = __fsqrt_rn(__fadd_rn(kx2, __fmul_rn(kzs, kzs)));
    c.kxp = __fdiv_rn(kx, np_);
    c.kxs = __fdiv_rn(kx, ns_);
    c.kzp = __fdiv_rn(kzp, np_);
    c.kzs = __fdiv_rn(kzs, ns_);
    c.norm = __fadd_rn(__fmul_rn(c.kxp, c.kxs), __fmul_rn(c.kzp, c.kzs));
    c.on = (double)c.norm >= 0.1 && (double)w >= 20.0;
    return c;
}

__device__ __forceinline__ float2 c_axpy(float a, float2 x, float b, float2 y)
{
    return make_float2(a * x.x + b * y.x, a * x.y + b * y.y);
}

// ssop of ewem.c:368-456 on a team's row (x-domain in v, zero at x >= nmx), both directions:
// adj (migration and the source): transform, phase, inverse, then exp(i w pd dz) and the taper;
// forward (modelling, -dz): the taper and exp(i w pd dz) first. ph: the phase table of the
// layer slowness (entries / L folded, +dz), corr: exp(i w pd dz) of the row (+dz); conj selects
// -dz.
template <int N, bool BLU>
__device__ __forceinline__ void ssop_row(float2 (&v)[16], bool adj, bool conj, const float2 *ph, const float2 *corr,
                                         const float *taper, float2 *xbuf, const float2 *tw, int t, unsigned sync,
                                         const MigArgs &m)
{
    constexpr int T = N / 16;
    const int nmx = m.nmx;
    if (!adj) {
#pragma unroll
        for (int q = 0; q < 16; q++) {
            const int x = t + T * q;
            if (x < nmx) {
                const float2 c = corr[x];
                const float tp = taper[x];
                const float2 u = make_float2(v[q].x * tp, v[q].y * tp);
                v[q] = conj ? cmulc(u, c) : cmul(u, c);
            } else {
                v[q] = make_float2(0.f, 0.f);
            }
        }
    }
    xform<N, -1, false, BLU>(v, xbuf, tw, t, sync, nullptr, m);
#pragma unroll
    for (int q = 0; q < 16; q++) {
        const float2 P = ph[kidx<N, BLU>(t, q, m.nlog)];
        v[q] = conj ? cmulc(v[q], P) : cmul(v[q], P);
    }
    xform<N, +1, false, BLU>(v, xbuf, tw, t, sync, nullptr, m);
#pragma unroll
    for (int q = 0; q < 16; q++) {
        const int x = t + T * q;
        if (x < nmx) {
            if (adj) {
                const float2 c = corr[x];
                const float tp = taper[x];
                const float2 u = conj ? cmulc(v[q], c) : cmul(v[q], c);
                v[q] = make_float2(u.x * tp, u.y * tp);
            }
        } else {
            v[q] = make_float2(0.f, 0.f);
        }
    }
}

// The mixing of elastic_separate_3d at the team's wavenumbers: the team's own spectrum is in
// v (Z form on Bluestein rows, which the per-wavenumber mixing keeps), the two spectra in
// sa (x or P) and sb (z or S2). role 0 computes the first output (P, or ux), role 1 the second
// (S2, or uz). sep: components -> potentials; otherwise potentials -> components. adj picks
// the reference's two variants. The 1/L of the transform pair is applied here.
template <int N, bool BLU>
__device__ __forceinline__ void mix_row(float2 (&v)[16], int role, bool sep, bool adj, const float2 *sa,
                                        const float2 *sb, bool w_on, const float *tab, int lp, int t,
                                        const MigArgs &m)
{
    constexpr int T = N / 16;
    const int L = BLU ? m.nlog : N;
    const float s = m.inv_n;
#pragma unroll
    for (int q = 0; q < 16; q++) {
        const int k = t + T * q;
        if (BLU && k >= L) {
            v[q] = make_float2(0.f, 0.f);
            continue;
        }
        const float2 A = sa[k], B = sb[k];
        SepCoef c;
        c.kxp = tab[k];
        c.kzp = tab[lp + k];
        c.kxs = tab[2 * lp + k];
        c.kzs = tab[3 * lp + k];
        c.norm = tab[4 * lp + k];
        c.on = (double)c.norm >= 0.1 && w_on;
        float2 r;
        if (sep) {
            if (!c.on) {
                r = role == 0 ? B : A;                                   // up = uz, us2 = ux
            } else if (adj) {
                r = role == 0 ? c_axpy(c.kxp, A, c.kzp, B) : c_axpy(-c.kzs, A, c.kxs, B);
            } else {
                const float2 q0 = role == 0 ? c_axpy(c.kxs, A, c.kzs, B) : c_axpy(-c.kzp, A, c.kxp, B);
                r = make_float2(__fdiv_rn(q0.x, c.norm), __fdiv_rn(q0.y, c.norm));
            }
        } else {
            if (!c.on) {
                r = role == 0 ? B : A;                                   // ux = us2, uz = up
            } else if (!adj) {
                r = role == 0 ? c_axpy(c.kxp, A, -c.kzs, B) : c_axpy(c.kzp, A, c.kxs, B);
            } else {
                const float2 q0 = role == 0 ? c_axpy(c.kxs, A, -c.kzp, B) : c_axpy(c.kzs, A, c.kxp, B);
                r = make_float2(__fdiv_rn(q0.x, c.norm), __fdiv_rn(q0.y, c.norm));
            }
        }
        v[q] = make_float2(r.x * s, r.y * s);
    }
}

// Shots per CTA: three for power-of-two rows up to 1024 points (one source team then advances
// three source rows while three receiver pairs continue theirs, six transforms each per depth
// step), else one (the register budget of longer rows and of the chirp form).
__host__ __device__ constexpr int ewem_group(int N, bool blu) { return (!blu && N <= 1024) ? 3 : 1; }

template <int N, bool BLU> struct EwemShape {
    static constexpr int T = N / 16, EG = ewem_group(N, BLU), NTEAM = 2 * EG + 1, NT = NTEAM * T;
    static constexpr int PADN = pad16(N);
    static constexpr int TW = fft_tw_size<N>(), TWP = (TW + 1) & ~1;
    static constexpr int MINB = (!BLU && NT <= 224) ? 2 : 1;  // CTAs per SM the register budget aims at
};

__host__ __device__ inline size_t ewem_smem_floats2(int N, int EG, int TWP, int PADN, int L, int nmx, int dbuf)
{
    return (size_t)TWP + (size_t)(dbuf ? 2 : 1) * EwemRec(L, nmx).floats() / 2 + 3 * (size_t)EG * N +
           (2 * (size_t)EG + 1) * PADN;
}

__device__ __forceinline__ void cp_async_wait_newest_pending()
{
    asm volatile("cp.async.wait_group 1;" ::: "memory");
}

// The depth recursion of EG shots of one frequency per CTA: ADJ migration, otherwise modelling.
// Teams 0..2EG-1 are the receiver pairs (pair j = teams 2j, 2j+1: the x / P and z / S2 rows of
// shot j of the group; warp-aligned, so a pair synchronises on its own), team 2EG the source.
// In migration the source team keeps the EG source rows in shared memory (srow_j) and continues
// them one after the other at every depth step, while each receiver pair separates, continues and
// recombines its rows; the images of shot j go to accumulator slot (CTA, j). In modelling the
// first EG teams take one source row each down through every depth (smig of slot (CTA, j)), then
// the receiver pairs go up.
template <int N, bool BLU, bool ADJ>
__global__ void __launch_bounds__(EwemShape<N, BLU>::NT, EwemShape<N, BLU>::MINB) wem_ewem_kernel(const EwemArgs a)
{
    using SH = EwemShape<N, BLU>;
    constexpr int T = SH::T, NT = SH::NT, PADN = SH::PADN, EG = SH::EG, SRC = 2 * EG;
    const MigArgs &m = a.m;
    const int nmx = m.nmx, nz = m.nz;
    const EwemRec R(a.nkx, nmx);
    extern __shared__ float4 smem_raw[];
    float2 *tw = reinterpret_cast<float2 *>(smem_raw);
    float *rec0 = reinterpret_cast<float *>(tw + SH::TWP);  // record buffer(s): depth iz in buffer iz & 1
    const float2 *php, *phs, *cp, *cs;
    const float *sept;
    auto use_record = [&](int iz) {
        const float *rec = rec0 + (a.dbuf ? (iz & 1) * R.floats() : 0);
        php = reinterpret_cast<const float2 *>(rec + R.php());
        phs = reinterpret_cast<const float2 *>(rec + R.phs());
        cp = reinterpret_cast<const float2 *>(rec + R.cp());
        cs = reinterpret_cast<const float2 *>(rec + R.cs());
        sept = rec + R.sep();
    };
    float2 *rows = reinterpret_cast<float2 *>(rec0 + (a.dbuf ? 2 : 1) * R.floats());  // per shot j: specA, specB, srow
    float2 *xb = rows + 3 * EG * N;
    const int tid = threadIdx.x, team = tid / T, t = tid - team * T;
    const int pair = team >> 1, role = team & 1;  // receiver teams
    float2 *xbuf = xb + (size_t)team * PADN;
    const unsigned sync = team_sync_handle<N>(tid);
    for (int i = tid; i < SH::TW; i += NT) tw[i] = a.twid[i];
    const int nsb = (m.nshot + EG - 1) / EG;  // shot blocks per frequency
    const int ngroups = nsb * a.nwc;
    const int recf4 = R.floats() / 4;

    for (int g = blockIdx.x; g < ngroups; g += gridDim.x) {
        const int iwc = g / nsb, sb = g % nsb, iwi = a.wbase + iwc;
        const int iw = m.ifmin + iwi;
        const float w = __fmul_rn((float)iw, m.dw);
        const bool w_on = (double)w >= 20.0;
        const float factor = iw == 0 ? 1.f : 2.f;
        // the receiver pair's shot (teams below SRC)
        const int jj = team < SRC ? pair : 0;
        const int shot = sb * EG + jj;
        const bool valid = team < SRC && shot < m.nshot;
        float2 *specA = rows + (size_t)3 * jj * N, *specB = specA + N, *srow = specB + N;

        // The record of depth iz into shared memory (all threads). Double-buffered: issue(next)
        // starts the asynchronous copy of the next depth's record into the other buffer (a
        // commit group per call, empty when there is none), ready(iz) waits for every group
        // but that newest one; the callers' barriers before and after order the buffers.
        // Single buffer: ready(iz) copies synchronously.
        auto issue = [&](int iz) {
            if (a.dbuf) {
                if (iz >= 0 && iz < nz) {
                    const float4 *src = reinterpret_cast<const float4 *>(a.tabs + ((size_t)iwc * nz + iz) * R.floats());
                    float4 *dst = reinterpret_cast<float4 *>(rec0 + (iz & 1) * R.floats());
                    for (int i = tid; i < recf4; i += NT) cp_async16(dst + i, src + i);
                }
                cp_async_commit();
            }
        };
        auto ready = [&](int iz) {
            if (a.dbuf) {
                cp_async_wait_newest_pending();
            } else {
                const float4 *src = reinterpret_cast<const float4 *>(a.tabs + ((size_t)iwc * nz + iz) * R.floats());
                float4 *dst = reinterpret_cast<float4 *>(rec0);
                for (int i = tid; i < recf4; i += NT) dst[i] = __ldg(src + i);
            }
            use_record(iz);
        };
        // the record of the next depth towards L2, so that its copy does not wait on DRAM
        auto prefetch = [&](int iz) {
            if (iz < 0 || iz >= nz) return;
            const char *src = reinterpret_cast<const char *>(a.tabs + ((size_t)iwc * nz + iz) * R.floats());
            for (int o = tid * 128; o < recf4 * 16; o += NT * 128) asm volatile("prefetch.global.L2 [%0];" ::"l"(src + o));
        };
        // a receiver pair's separation or recombination: forward transforms, spectra to shared
        // memory, mixing at each wavenumber, inverse transforms
        auto mix = [&](float2 (&v)[16], bool sep) {
            xform<N, -1, false, BLU>(v, xbuf, tw, t, sync, nullptr, m);
            float2 *dst = role == 0 ? specA : specB;
#pragma unroll
            for (int q = 0; q < 16; q++) dst[t + T * q] = v[q];
            team_pair_sync<N>(pair, tid);
            mix_row<N, BLU>(v, role, sep, ADJ, specA, specB, w_on, sept, R.lp, t, m);
            xform<N, +1, false, BLU>(v, xbuf, tw, t, sync, nullptr, m);
#pragma unroll
            for (int q = 0; q < 16; q++)
                if (t + T * q >= nmx) v[q] = make_float2(0.f, 0.f);
        };

        __syncthreads();  // the previous group's rows and spectra are read
        float2 v[16];
        if (ADJ) {
            if (team == SRC) {  // the source spikes of the group's shots
                for (int j = 0; j < EG; j++) {
                    const int sj = sb * EG + j;
                    if (sj >= m.nshot) break;
                    const int igx = a.igx[sj];
                    float2 *sr = rows + (size_t)(3 * j + 2) * N;
#pragma unroll
                    for (int q = 0; q < 16; q++) {
                        const int x = t + T * q;
                        sr[x] = (x == igx && x < nmx) ? a.srcw[iwi] : make_float2(0.f, 0.f);
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < 16; q++) {
                const int x = t + T * q;
                v[q] = (valid && x < nmx) ? (role == 0 ? a.recv_x : a.recv_z)[((size_t)shot * m.nwf + iwi) * nmx + x]
                                          : make_float2(0.f, 0.f);
            }
            const size_t nzx = (size_t)nz * nmx;
            float2 *slot = a.slots + ((size_t)role * gridDim.x * EG + (size_t)blockIdx.x * EG + jj) * nzx;
            issue(0);
            for (int iz = 0; iz < nz; iz++) {
                const float z = __fadd_rn(a.oz, __fmul_rn(m.dz, (float)iz));
                const bool src_on = z >= a.sz, rec_on = z >= a.gz;
                __syncthreads();  // the previous depth's tables, spectra and source rows are read
                issue(iz + 1);
                ready(iz);
                prefetch(iz + 2);
                __syncthreads();
                if (team == SRC) {
                    if (src_on) {
                        for (int j = 0; j < EG; j++) {
                            if (sb * EG + j >= m.nshot) break;
                            float2 *sr = rows + (size_t)(3 * j + 2) * N;
#pragma unroll
                            for (int q = 0; q < 16; q++) v[q] = sr[t + T * q];
                            ssop_row<N, BLU>(v, true, true, php, cp, a.taper, xbuf, tw, t, sync, m);
#pragma unroll
                            for (int q = 0; q < 16; q++) sr[t + T * q] = v[q];
                        }
                    }
                } else if (valid && rec_on) {
                    mix(v, true);  // components -> potentials
                    ssop_row<N, BLU>(v, true, false, role == 0 ? php : phs, role == 0 ? cp : cs, a.taper, xbuf, tw, t,
                                     sync, m);
                }
                if (!rec_on) continue;  // CTA-uniform
                __syncthreads();  // the source rows are continued; the spectra were read
                if (valid) {
                    float2 *acc = slot + (size_t)iz * nmx;
#pragma unroll
                    for (int q = 0; q < 16; q++) {
                        const int x = t + T * q;
                        if (x < nmx) {
                            const float2 s0 = srow[x];
                            const float2 s_ = src_on ? make_float2(s0.x * a.inv_max_source, s0.y * a.inv_max_source)
                                                     : make_float2(0.f, 0.f);
                            kahan_add(&acc[x], factor * (s_.x * v[q].x + s_.y * v[q].y));  // Re(conj(smig) u)
                        }
                    }
                    mix(v, false);  // potentials -> components
                }
            }
        } else {
            // source, downward, every depth kept: team j < EG takes the group's shot j
            const int sj = sb * EG + team;
            const bool sv = team < EG && sj < m.nshot;
            float2 *smig = a.smig + ((size_t)blockIdx.x * EG + (team < EG ? team : 0)) * nz * nmx;
            {
                const int igx = sv ? a.igx[sj] : -1;
#pragma unroll
                for (int q = 0; q < 16; q++) {
                    const int x = t + T * q;
                    v[q] = (x == igx && x < nmx) ? a.srcw[iwi] : make_float2(0.f, 0.f);
                }
            }
            issue(0);
            for (int iz = 0; iz < nz; iz++) {
                const float z = __fadd_rn(a.oz, __fmul_rn(m.dz, (float)iz));
                __syncthreads();
                issue(iz + 1);
                ready(iz);
                prefetch(iz + 2);
                __syncthreads();
                if (sv) {
                    float2 *row = smig + (size_t)iz * nmx;
                    if (z >= a.sz) ssop_row<N, BLU>(v, true, true, php, cp, a.taper, xbuf, tw, t, sync, m);
#pragma unroll
                    for (int q = 0; q < 16; q++) {
                        const int x = t + T * q;
                        if (x < nmx)
                            row[x] = z >= a.sz ? make_float2(v[q].x * a.inv_max_source, v[q].y * a.inv_max_source)
                                               : make_float2(0.f, 0.f);
                    }
                }
            }
            __syncthreads();  // smig written by the source teams is read by the receiver pairs below
            // receiver, upward with the images injected
            const float2 *smr = a.smig + ((size_t)blockIdx.x * EG + jj) * nz * nmx;
#pragma unroll
            for (int q = 0; q < 16; q++) v[q] = make_float2(0.f, 0.f);
            // the receiver's depths: z >= gz, the deepest ones (z grows with iz)
            int iz_lo = nz;
            while (iz_lo > 0 && __fadd_rn(a.oz, __fmul_rn(m.dz, (float)(iz_lo - 1))) >= a.gz) iz_lo--;
            if (a.dbuf) cp_async_wait_all();  // the source pass's last (empty) group
            issue(nz - 1 >= iz_lo ? nz - 1 : -1);
            for (int iz = nz - 1; iz >= iz_lo; iz--) {
                __syncthreads();
                issue(iz - 1 >= iz_lo ? iz - 1 : -1);
                ready(iz);
                prefetch(iz - 2 >= iz_lo ? iz - 2 : -1);
                __syncthreads();
                if (valid) {
                    mix(v, true);
                    const float2 *row = smr + (size_t)iz * nmx;
                    const float *img = (role == 0 ? a.img_p : a.img_s) + (size_t)iz * nmx;
#pragma unroll
                    for (int q = 0; q < 16; q++) {
                        const int x = t + T * q;
                        if (x < nmx) {
                            const float2 s_ = row[x];
                            const float mv = img[x];
                            v[q].x += s_.x * mv;
                            v[q].y += s_.y * mv;
                        }
                    }
                    ssop_row<N, BLU>(v, false, true, role == 0 ? php : phs, role == 0 ? cp : cs, a.taper, xbuf, tw, t,
                                     sync, m);
                    team_pair_sync<N>(pair, tid);  // the spectra of the separation were read
                    mix(v, false);
                }
            }
            if (valid) {  // ux_g_wx, uz_g_wx = u / sqrtf(ntfft) (ewem.c:357-361)
                float2 *out = (role == 0 ? a.dg_x : a.dg_z) + ((size_t)shot * m.nwf + iwi) * nmx;
#pragma unroll
                for (int q = 0; q < 16; q++) {
                    const int x = t + T * q;
                    if (x < nmx) out[x] = make_float2(v[q].x * a.inv_sqt, v[q].y * a.inv_sqt);
                }
            }
        }
    }
}

template <int N, bool BLU, bool ADJ>
int ewem_launch_t(const EwemArgs *a, int nsm, int nitems, cudaStream_t st, int *grid_out, size_t *smem_out)
{
    using SH = EwemShape<N, BLU>;
    auto k = wem_ewem_kernel<N, BLU, ADJ>;
    // double-buffered records where the second buffer keeps the CTAs per SM of a single one
    int bps = 0, dbuf = 0;
    size_t smem = 0;
    for (int db = 1; db >= 0; db--) {
        const size_t sz = sizeof(float2) * ewem_smem_floats2(N, SH::EG, SH::TWP, SH::PADN, a->nkx, a->m.nmx, db);
        int b = 0;
        if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sz) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k, SH::NT, sz) != cudaSuccess) {
            b = 0;
            (void)cudaGetLastError();  // a size above the opt-in limit: not an error of the launch
        }
        if (db == 1) {
            bps = b;
            smem = sz;
            dbuf = 1;
        } else if (b > bps || bps < 1) {
            bps = b;
            smem = sz;
            dbuf = 0;
        }
    }
    if (bps < 1 || cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return -1;
    *smem_out = smem;
    const long long cap = (long long)nsm * bps;
    const long long ngroups = (long long)a->nwc * ((a->m.nshot + SH::EG - 1) / SH::EG);
    (void)nitems;
    const int grid = (int)std::max<long long>(1, std::min<long long>(cap, ngroups));
    *grid_out = grid;
    if (!a->slots && !a->smig) return 0;  // sizing only
    EwemArgs b = *a;
    b.dbuf = dbuf;
    k<<<grid, SH::NT, smem, st>>>(b);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <int N>
int ewem_launch_n(int blu, int adj, const EwemArgs *a, int nsm, int nitems, cudaStream_t st, int *grid, size_t *smem)
{
    if (blu) return adj ? ewem_launch_t<N, true, true>(a, nsm, nitems, st, grid, smem)
                        : ewem_launch_t<N, true, false>(a, nsm, nitems, st, grid, smem);
    return adj ? ewem_launch_t<N, false, true>(a, nsm, nitems, st, grid, smem)
               : ewem_launch_t<N, false, false>(a, nsm, nitems, st, grid, smem);
}

#define WEM_EWEM_DECLARE_N(N)                                                                            \
    extern template int ewem_launch_n<N>(int, int, const EwemArgs *, int, int, cudaStream_t, int *, size_t *);
WEM_EWEM_DECLARE_N(64)
WEM_EWEM_DECLARE_N(128)
WEM_EWEM_DECLARE_N(256)
WEM_EWEM_DECLARE_N(512)
WEM_EWEM_DECLARE_N(1024)
WEM_EWEM_DECLARE_N(2048)
#undef WEM_EWEM_DECLARE_N

}  // namespace gbwem
