// wem_elastic3d.cu -- elastic shot-profile migration and its forward operator on 3-D grids
// (nmy > 1): the reference's ewem / elastic_extrap1f / elastic_separate_3d / ssop with their
// rank-2 transforms over (x, y) planes (src/Imaging/c/ewem.c:3-741; plans at ewem.c:84-96).
//
// A padded plane of nkx x nky samples does not fit in shared memory, so every depth step of the
// items (shot, frequency) in flight is a short sequence of batched passes over device memory:
//   * row passes: transforms along y, one team of nky/16 threads per row x (nky samples in its
//     registers, the register-resident FFT of wem_fft.cuh). Between the inverse and the forward
//     transform sit the x-domain operations: the crop to the grid (y >= nmy zeroed), the
//     1/sqrt(nkx nky) scales, the slowness correction exp(i w pd dz) and the boundary taper of
//     ssop, the imaging condition, and the image injection of the forward operator;
//   * column passes: transforms along x, one team of nkx/16 threads per ky column, the teams of
//     a CTA on adjacent columns. Between the forward and the inverse transform sit the k-domain
//     operations: the separation and recombination mixes of elastic_separate_3d (per kx, the
//     same for every ky, as in the reference), and the split-step phase of ssop at (kx, ky).
// Between passes a plane stays in the (x, ky) form of the y transform, K[item][plane][x][ky] for
// x < nmx: the rows the reference pads with zeros (x >= nmx) are zero-filled by the column pass,
// whose inverse transform keeps x < nmx only -- the reference's crop in x.
// Planes: 0 = ux, then P; 1 = uz, then S2 (the separation and the recombination overwrite them
// in place); 2 = the source. The y component and S1 stay zero, as in the reference (its S1 and
// uy separation is commented out, ewem.c:579-587, 628-634).
// Migration images Re(conj(smig) P) and Re(conj(smig) S2): the row team of (chunk of items, x)
// sums its chunk's items in registers and adds the sum into that chunk's compensated
// accumulators; a fixed-order reduction over the chunks follows, so the result is deterministic.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "../../include/shotwem_gb300.h"
#include "wem_elastic.cuh"

namespace gbwem {
int set_error(int code, const char *msg);  // wem_api.cu: records wem_last_error()

struct E3Args {
    int nmx, nmy, nkx, nky, nz, nwf, ifmin;
    int item0, nitems;  // the batch: items item0 .. item0 + nitems - 1 of the list
    int ipc;            // row passes: items per unit (the imaging chunk), 1 otherwise
    int iz, op, mask;   // depth step, operation, planes (bit p)
    int adj;            // 1 migration, 0 forward operator
    float dw, dz, dkx, dky;
    float inv_s;        // 1 / sqrtf(nkx * nky)
    float inv_max_source, inv_sqt;
    const int *item_iwi, *item_shot;  // [all items]
    const int *src_cell;              // [nshot] igx * nmy + igy
    const float2 *srcw;               // [nwf] wavelet spectrum / sqrt(ntfft)
    const float2 *recv_x, *recv_z;    // [nshot][nwf][nmx * nmy] component spectra / sqrt(ntfft)
    const float *po_p, *po_s;         // [nz] layer slownesses
    const float *vpm, *vsm;           // [nz] 1 / po (the separation's velocities)
    const float *pd_p, *pd_s;         // [nz][nmx * nmy] slowness perturbations
    const float *tapx, *tapy;         // boundary_condition weights along x and y
    const float2 *twx, *twy;          // FFT twiddle tables of nkx and nky
    float2 *K;                        // [batch item][3][nmx][nky]
    float2 *acc_p, *acc_s;            // [chunk][nz][nmx * nmy] (sum, compensation)
    float2 *smig;                     // forward: [batch item][nz][nmx * nmy]
    const float *mpp, *mps2;          // forward: [nz][nmx * nmy] images, depth-major
    float2 *out_x, *out_z;            // forward: [nshot][nwf][nmx * nmy] modelled spectra
};

// row operations
enum { E3R_LOAD_REC = 0, E3R_LOAD_SRC, E3R_MID, E3R_IMG, E3R_SRC_STORE, E3R_INJ, E3R_OUT };
// column operations
enum { E3C_SEP = 0, E3C_SSOP, E3C_RECOMB };

constexpr int E3_THREADS = 256;

// exp(i w pd dz) at (iz, cell), the float operations of ewem.c:430
__device__ __forceinline__ float2 e3_corr(float w, float pd, float dz)
{
    float sn, cs;
    sincosf(__fmul_rn(__fmul_rn(w, pd), dz), &sn, &cs);
    return make_float2(cs, sn);
}

// The split-step phase of ewem.c:416-421 at (kx, ky): s = w^2 po^2 - kx^2 - ky^2 (float, in that
// order); exp(i sqrt(s) dz), or exp(-0.2 sqrt(|s|) |dz|) where evanescent.
__device__ __forceinline__ float2 e3_phase(float w, float po, float kx, float ky, float dz)
{
    const float s = __fsub_rn(__fsub_rn(__fmul_rn(__fmul_rn(w, w), __fmul_rn(po, po)), __fmul_rn(kx, kx)),
                              __fmul_rn(ky, ky));
    if (s >= 0.f) {
        float sn, cs;
        sincosf(__fmul_rn(__fsqrt_rn(s), dz), &sn, &cs);
        return make_float2(cs, sn);
    }
    return make_float2(expf(-__fmul_rn(__fmul_rn(0.2f, __fsqrt_rn(-s)), fabsf(dz))), 0.f);
}

// ------------------------------------------------------------------ row passes (along y)
// twiddles, one exchange buffer per team, and per team the depth's source row (imaging form)
template <int NY> __host__ __device__ constexpr size_t e3_rows_smem()
{
    return sizeof(float2) *
           ((size_t)((fft_tw_size<NY>() + 1) & ~1) + (size_t)(E3_THREADS / (NY / 16)) * (pad16(NY) + NY));
}

// OP: the row operation (E3R_*), a template parameter so that each form gets its own register
// budget; two CTAs per SM.
template <int NY, int OP>
__global__ void __launch_bounds__(E3_THREADS, 2) wem_e3_rows_kernel(const E3Args a)
{
    constexpr int T = NY / 16, TEAMS = E3_THREADS / T, TW = fft_tw_size<NY>();
    extern __shared__ float4 e3r_smem[];
    float2 *s_tw = reinterpret_cast<float2 *>(e3r_smem);
    const int tid = threadIdx.x, team = tid / T, t = tid - team * T;
    float2 *xbuf = s_tw + ((TW + 1) & ~1) + (size_t)team * pad16(NY);
    // the team's source row of the depth (smig / max_source at y = t + T m, entry m T + t)
    float2 *sm = s_tw + ((TW + 1) & ~1) + (size_t)TEAMS * pad16(NY) + (size_t)team * NY;
    const unsigned sync = team_sync_handle<NY>(tid);
    for (int i = tid; i < TW; i += E3_THREADS) s_tw[i] = a.twy[i];
    __syncthreads();

    const int nmx = a.nmx, nmy = a.nmy, nky = a.nky, nn = nmx * nmy, iz = a.iz;
    const int nchunk = (a.nitems + a.ipc - 1) / a.ipc;
    const int unit = blockIdx.x * TEAMS + team;
    if (unit >= nchunk * nmx) return;  // whole teams leave; no CTA-wide barrier follows
    const int x = unit % nmx, chunk = unit / nmx;
    const int i0 = chunk * a.ipc, i1 = min(a.nitems, i0 + a.ipc);
    const size_t plane = (size_t)nmx * nky;
    const float tx = a.tapx[x];
    const size_t zc = (size_t)iz * nn + (size_t)x * nmy;  // (iz, x, y = 0) in the [nz][nn] arrays

    float imp[16], ims[16];
#pragma unroll
    for (int m = 0; m < 16; m++) imp[m] = ims[m] = 0.f;

    for (int li = i0; li < i1; li++) {
        const int item = a.item0 + li;
        const int iwi = a.item_iwi[item], shot = a.item_shot[item];
        const int iw = a.ifmin + iwi;
        const float w = __fmul_rn((float)iw, a.dw);
        float2 *Kx = a.K + (size_t)li * 3 * plane + (size_t)x * nky;  // row x of plane 0
        float2 v[16];
        if constexpr (OP == E3R_LOAD_REC || OP == E3R_LOAD_SRC) {
            // the initial planes (ewem.c:109, 295-300): the component spectra, the source spike
            const int p0 = OP == E3R_LOAD_REC ? 0 : 2, p1 = OP == E3R_LOAD_REC ? 1 : 2;
            for (int p = p0; p <= p1; p++) {
#pragma unroll
                for (int m = 0; m < 16; m++) {
                    const int y = t + T * m;
                    float2 u = make_float2(0.f, 0.f);
                    if (y < nmy) {
                        const int cell = x * nmy + y;
                        if (p == 2) u = cell == a.src_cell[shot] ? a.srcw[iwi] : u;
                        else u = (p == 0 ? a.recv_x : a.recv_z)[((size_t)shot * a.nwf + iwi) * nn + cell];
                    }
                    v[m] = u;
                }
                fft_row<NY, -1>(v, xbuf, s_tw, t, sync);
                float2 *row = Kx + (size_t)p * plane;
#pragma unroll
                for (int m = 0; m < 16; m++) row[t + T * m] = v[m];
            }
            continue;
        } else {
            // the source at this depth (E3R_IMG, E3R_SRC_STORE): smig = ssop(source) / max_source
            if constexpr (OP == E3R_IMG || OP == E3R_SRC_STORE) {
#pragma unroll
                for (int m = 0; m < 16; m++) sm[T * m + t] = make_float2(0.f, 0.f);
            }
            if ((OP == E3R_IMG || OP == E3R_SRC_STORE) && (a.mask & 4)) {
                float2 *row = Kx + 2 * plane;
#pragma unroll
                for (int m = 0; m < 16; m++) v[m] = row[t + T * m];
                fft_row<NY, +1>(v, xbuf, s_tw, t, sync);
#pragma unroll
                for (int m = 0; m < 16; m++) {
                    const int y = t + T * m;
                    if (y < nmy) {
                        // ssop with -dz, adj (ewem.c:427-437): b exp(-i w pd dz) / sqrt(nkx nky), then the taper
                        const float2 c = e3_corr(w, a.pd_p[zc + y], a.dz);
                        float2 u = cmulc(v[m], c);
                        const float tp = __fmul_rn(tx, a.tapy[y]);
                        u = make_float2(u.x * a.inv_s * tp, u.y * a.inv_s * tp);
                        v[m] = u;
                        sm[T * m + t] = make_float2(u.x * a.inv_max_source, u.y * a.inv_max_source);
                    } else {
                        v[m] = make_float2(0.f, 0.f);
                    }
                }
                if (OP == E3R_SRC_STORE) {
                    float2 *sg = a.smig + ((size_t)li * a.nz) * nn + zc;
#pragma unroll
                    for (int m = 0; m < 16; m++) {
                        const int y = t + T * m;
                        if (y < nmy) sg[y] = sm[T * m + t];
                    }
                }
                fft_row<NY, -1>(v, xbuf, s_tw, t, sync);
#pragma unroll
                for (int m = 0; m < 16; m++) row[t + T * m] = v[m];
            }
            if (OP == E3R_SRC_STORE) continue;
            const float factor = iw == 0 ? 1.f : 2.f;  // ewem.c:290-291
            for (int p = 0; p < 2; p++) {
                if (!((a.mask >> p) & 1)) continue;
                float2 *row = Kx + (size_t)p * plane;
#pragma unroll
                for (int m = 0; m < 16; m++) v[m] = row[t + T * m];
                fft_row<NY, +1>(v, xbuf, s_tw, t, sync);
                const float *pd = p == 0 ? a.pd_p : a.pd_s;
                float2 *out = OP == E3R_OUT ? (p == 0 ? a.out_x : a.out_z) + ((size_t)shot * a.nwf + iwi) * nn + (size_t)x * nmy
                                              : nullptr;
#pragma unroll
                for (int m = 0; m < 16; m++) {
                    const int y = t + T * m;
                    if (y >= nmy) {
                        v[m] = make_float2(0.f, 0.f);
                        continue;
                    }
                    float2 u = v[m];
                    if (OP == E3R_IMG) {
                        // ssop with +dz, adj: b exp(i w pd dz) / sqrt(nkx nky), the taper, then the
                        // imaging condition (ewem.c:313-323)
                        u = cmul(u, e3_corr(w, pd[zc + y], a.dz));
                        const float tp = __fmul_rn(tx, a.tapy[y]);
                        u = make_float2(u.x * a.inv_s * tp, u.y * a.inv_s * tp);
                        const float2 q = sm[T * m + t];
                        const float r = __fmul_rn(factor, __fadd_rn(__fmul_rn(q.x, u.x), __fmul_rn(q.y, u.y)));
                        if (p == 0) imp[m] = __fadd_rn(imp[m], r);
                        else ims[m] = __fadd_rn(ims[m], r);
                    } else {
                        u = make_float2(u.x * a.inv_s, u.y * a.inv_s);  // the inverse transform's 1/sqrt(nkx nky)
                        if (OP == E3R_INJ) {
                            // the forward operator (ewem.c:331-339): the potential plus smig * image,
                            // then ssop with -dz, adj = false: the taper, exp(-i w pd dz)
                            const float mv = (p == 0 ? a.mpp : a.mps2)[zc + y];
                            const float2 s = a.smig[((size_t)li * a.nz) * nn + zc + y];
                            u = make_float2(__fadd_rn(u.x, __fmul_rn(s.x, mv)), __fadd_rn(u.y, __fmul_rn(s.y, mv)));
                            const float tp = __fmul_rn(tx, a.tapy[y]);
                            u = make_float2(u.x * tp, u.y * tp);
                            u = cmulc(u, e3_corr(w, pd[zc + y], a.dz));
                        } else if (OP == E3R_OUT) {
                            out[y] = make_float2(u.x * a.inv_sqt, u.y * a.inv_sqt);  // ewem.c:345-349
                        }
                    }
                    v[m] = u;
                }
                if (OP == E3R_OUT) continue;
                fft_row<NY, -1>(v, xbuf, s_tw, t, sync);
#pragma unroll
                for (int m = 0; m < 16; m++) row[t + T * m] = v[m];
            }
        }
    }
    if (OP == E3R_IMG && (a.mask & 3)) {
        float2 *ap = a.acc_p + (size_t)chunk * a.nz * nn + zc, *as = a.acc_s + (size_t)chunk * a.nz * nn + zc;
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const int y = t + T * m;
            if (y < nmy) {
                kahan_add(&ap[y], imp[m]);
                kahan_add(&as[y], ims[m]);
            }
        }
    }
}

// ------------------------------------------------------------------ column passes (along x)
// CTA: CW = 4096/NX adjacent ky columns of one item (at most nky), one team of NX/16 threads per
// column. The block's columns of every plane the operation touches reach a shared-memory tile by
// asynchronous copies of row segments (a warp copies 2 .. 8 rows of 128 .. 32 bytes, each line
// once), the teams transform their columns from and back into the tile, and the CTA writes the
// tile back row segment by row segment. One CTA per (item, block of columns), so that the copies
// of one CTA overlap the transforms of the others on the SM.
template <int NX> __host__ __device__ constexpr int e3_cols_cw_max() { return E3_THREADS / (NX / 16); }
// twiddles, exchange buffers, the tile of the CTA's columns (one [nmx][cw + 1] block per plane of
// the operation), the mix coefficients
template <int NX> __host__ __device__ inline size_t e3_cols_smem(int cw, int nmx, int nplanes)
{
    return sizeof(float2) * ((size_t)((fft_tw_size<NX>() + 1) & ~1) + (size_t)cw * pad16(NX) +
                             (size_t)nplanes * nmx * (cw + 1)) +
           sizeof(float) * 5 * (size_t)NX + (size_t)NX;
}

__device__ __forceinline__ void cp_async8(void *dst, const void *src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
                 : "memory");
}

template <int NX, int OP>
__global__ void __launch_bounds__(E3_THREADS, 2) wem_e3_cols_kernel(const E3Args a)
{
    constexpr int T = NX / 16, TW = fft_tw_size<NX>();
    constexpr bool MIX = OP != E3C_SSOP;
    extern __shared__ float4 e3c_smem[];
    const int nt = blockDim.x, cw = nt / T;
    const int nmx = a.nmx, nky = a.nky, iz = a.iz;
    const int RS = cw + 1;  // tile row stride (odd: the teams' column reads spread over the banks)
    float2 *s_tw = reinterpret_cast<float2 *>(e3c_smem);
    float2 *s_x = s_tw + ((TW + 1) & ~1);
    float2 *s_tile = s_x + (size_t)cw * pad16(NX);                              // [planes][nmx][RS]
    float *s_cf = reinterpret_cast<float *>(s_tile + (size_t)__popc(a.mask & 7) * nmx * RS);  // [5][NX]
    uint8_t *s_on = reinterpret_cast<uint8_t *>(s_cf + 5 * NX);
    const int tid = threadIdx.x, c = tid / T, t = tid - c * T;
    float2 *xbuf = s_x + (size_t)c * pad16(NX);
    const unsigned sync = team_sync_handle<NX>(tid);
    const int nblk = nky / cw;
    const int li = blockIdx.x / nblk, ky0 = (blockIdx.x - li * nblk) * cw, ky = ky0 + c;
    const int item = a.item0 + li;
    const int iw = a.ifmin + a.item_iwi[item];
    const float w = __fmul_rn((float)iw, a.dw);
    const size_t plane = (size_t)nmx * nky;
    float2 *Kg = a.K + (size_t)li * 3 * plane + ky0;  // the block's first column, plane 0
    const int lcw = __ffs(cw) - 1;                     // cw is a power of two
    // the block's columns of every plane of the operation into the tile: 8-byte asynchronous
    // copies, consecutive threads on consecutive columns of a row (a 32 .. 128-byte segment)
    for (int p = 0, q = 0; p < 3; p++) {
        if (!((a.mask >> p) & 1)) continue;
        for (int e = tid; e < nmx * cw; e += nt) {
            const int x = e >> lcw, j = e & (cw - 1);
            cp_async8(s_tile + ((size_t)q * nmx + x) * RS + j, Kg + (size_t)p * plane + (size_t)x * nky + j);
        }
        q++;
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
    for (int i = tid; i < TW; i += nt) s_tw[i] = a.twx[i];
    if constexpr (MIX) {
        // elastic_separate_3d's coefficients of every kx (ewem.c:596-611): the layer's vp, vs
        const float vp = a.vpm[iz], vs = a.vsm[iz];
        for (int k = tid; k < NX; k += nt) {
            const SepCoef cf = sep_coef(kx_signed(k, NX, a.dkx), w, vp, vs);
            s_cf[k] = cf.kxp;
            s_cf[NX + k] = cf.kzp;
            s_cf[2 * NX + k] = cf.kxs;
            s_cf[3 * NX + k] = cf.kzs;
            s_cf[4 * NX + k] = cf.norm;
            s_on[k] = cf.on ? 1 : 0;
        }
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    __syncthreads();
    // the team's column in the tile's first plane from this thread's first sample x = t: sample
    // x = t + T m at K[m * sT]; tile planes nmx * RS apart, in the order of the operation's planes
    float2 *K = s_tile + (size_t)t * RS + c;
    const size_t sT = (size_t)T * RS;
    const size_t tplane = (size_t)nmx * RS;
    float2 v[16];
    if constexpr (!MIX) {
        const float kyv = kx_signed(ky, nky, a.dky);
        for (int p = 0; p < 3; p++) {
            if (!((a.mask >> p) & 1)) continue;
            float2 *col = K + (size_t)__popc(a.mask & ((1 << p) - 1)) * tplane;
#pragma unroll
            for (int m = 0; m < 16; m++) {
                const int x = t + T * m;
                v[m] = x < nmx ? col[m * sT] : make_float2(0.f, 0.f);
            }
            fft_row<NX, -1>(v, xbuf, s_tw, t, sync);
            // the source goes down with -dz; the forward operator's receivers go up with -dz
            const bool neg = p == 2 || !a.adj;
            const float po = p == 1 ? a.po_s[iz] : a.po_p[iz];
#pragma unroll
            for (int m = 0; m < 16; m++) {
                const float kx = kx_signed(t + T * m, NX, a.dkx);
                float2 L = e3_phase(w, po, kx, kyv, a.dz);
                if (neg) L.y = -L.y;  // sqrtf(s) * (-dz) = -(sqrtf(s) * dz)
                const float2 u = cmul(v[m], L);
                v[m] = make_float2(u.x * a.inv_s, u.y * a.inv_s);
            }
            fft_row<NX, +1>(v, xbuf, s_tw, t, sync);
#pragma unroll
            for (int m = 0; m < 16; m++) {
                const int x = t + T * m;
                if (x < nmx) col[m * sT] = v[m];
            }
        }
    } else {
        float2 u[16];
        float2 *c0 = K, *c1 = K + tplane;  // planes 0 and 1 (mask 3)
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const int x = t + T * m;
            v[m] = x < nmx ? c0[m * sT] : make_float2(0.f, 0.f);
            u[m] = x < nmx ? c1[m * sT] : make_float2(0.f, 0.f);
        }
        fft_row<NX, -1>(v, xbuf, s_tw, t, sync);
        fft_row<NX, -1>(u, xbuf, s_tw, t, sync);
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const int k = t + T * m;
            const float2 A = make_float2(v[m].x * a.inv_s, v[m].y * a.inv_s);  // first plane / sqrt(nkx nky)
            const float2 B = make_float2(u[m].x * a.inv_s, u[m].y * a.inv_s);
            float2 o0, o1;
            if (s_on[k]) {
                const float kxp = s_cf[k], kzp = s_cf[NX + k], kxs = s_cf[2 * NX + k], kzs = s_cf[3 * NX + k],
                            nrm = s_cf[4 * NX + k];
                if (OP == E3C_SEP) {
                    // (ux, uz) -> (P, S2), ewem.c:612-620
                    if (a.adj) {
                        o0 = c_axpy(kxp, A, kzp, B);
                        o1 = c_axpy(-kzs, A, kxs, B);
                    } else {
                        o0 = c_axpy(kxs, A, kzs, B);
                        o1 = c_axpy(-kzp, A, kxp, B);
                        o0 = make_float2(__fdiv_rn(o0.x, nrm), __fdiv_rn(o0.y, nrm));
                        o1 = make_float2(__fdiv_rn(o1.x, nrm), __fdiv_rn(o1.y, nrm));
                    }
                } else {
                    // (P, S2) -> (ux, uz), ewem.c:696-704
                    if (a.adj) {
                        o0 = c_axpy(kxs, A, -kzp, B);
                        o1 = c_axpy(kzs, A, kxp, B);
                        o0 = make_float2(__fdiv_rn(o0.x, nrm), __fdiv_rn(o0.y, nrm));
                        o1 = make_float2(__fdiv_rn(o1.x, nrm), __fdiv_rn(o1.y, nrm));
                    } else {
                        o0 = c_axpy(kxp, A, -kzs, B);
                        o1 = c_axpy(kzp, A, kxs, B);
                    }
                }
            } else {
                // the swap where the potentials are not separated (ewem.c:622-625, 706-709)
                o0 = B;
                o1 = A;
            }
            v[m] = o0;
            u[m] = o1;
        }
        fft_row<NX, +1>(v, xbuf, s_tw, t, sync);
        fft_row<NX, +1>(u, xbuf, s_tw, t, sync);
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const int x = t + T * m;
            if (x < nmx) {
                c0[m * sT] = v[m];
                c1[m * sT] = u[m];
            }
        }
    }
    __syncthreads();  // the tile holds every team's results
    for (int p = 0, q = 0; p < 3; p++) {
        if (!((a.mask >> p) & 1)) continue;
        for (int e = tid; e < nmx * cw; e += nt) {
            const int x = e >> lcw, j = e & (cw - 1);
            Kg[(size_t)p * plane + (size_t)x * nky + j] = s_tile[((size_t)q * nmx + x) * RS + j];
        }
        q++;
    }
}

template <int NY, int OP> int e3_rows_launch_op(const E3Args &a, cudaStream_t st)
{
    constexpr int TEAMS = E3_THREADS / (NY / 16);
    const size_t smem = e3_rows_smem<NY>();
    if (cudaFuncSetAttribute(wem_e3_rows_kernel<NY, OP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return -1;
    const long long units = (long long)((a.nitems + a.ipc - 1) / a.ipc) * a.nmx;
    if (units <= 0) return 0;
    wem_e3_rows_kernel<NY, OP><<<(unsigned)((units + TEAMS - 1) / TEAMS), E3_THREADS, smem, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <int NY> int e3_rows_launch(const E3Args &a, cudaStream_t st)
{
    switch (a.op) {
    case E3R_LOAD_REC: return e3_rows_launch_op<NY, E3R_LOAD_REC>(a, st);
    case E3R_LOAD_SRC: return e3_rows_launch_op<NY, E3R_LOAD_SRC>(a, st);
    case E3R_MID: return e3_rows_launch_op<NY, E3R_MID>(a, st);
    case E3R_IMG: return e3_rows_launch_op<NY, E3R_IMG>(a, st);
    case E3R_SRC_STORE: return e3_rows_launch_op<NY, E3R_SRC_STORE>(a, st);
    case E3R_INJ: return e3_rows_launch_op<NY, E3R_INJ>(a, st);
    case E3R_OUT: return e3_rows_launch_op<NY, E3R_OUT>(a, st);
    default: return -2;
    }
}

template <int NX, int OP> int e3_cols_launch_op(const E3Args &a, cudaStream_t st)
{
    const int cw = std::min(e3_cols_cw_max<NX>(), a.nky);
    const size_t smem = e3_cols_smem<NX>(cw, a.nmx, __builtin_popcount(a.mask & 7));
    if (smem > 227 * 1024) return -2;
    if (cudaFuncSetAttribute(wem_e3_cols_kernel<NX, OP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return -1;
    const long long jobs = (long long)a.nitems * (a.nky / cw);
    if (jobs <= 0) return 0;
    wem_e3_cols_kernel<NX, OP><<<(unsigned)jobs, cw * (NX / 16), smem, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <int NX> int e3_cols_launch(const E3Args &a, cudaStream_t st)
{
    switch (a.op) {
    case E3C_SEP: return e3_cols_launch_op<NX, E3C_SEP>(a, st);
    case E3C_SSOP: return e3_cols_launch_op<NX, E3C_SSOP>(a, st);
    case E3C_RECOMB: return e3_cols_launch_op<NX, E3C_RECOMB>(a, st);
    default: return -2;
    }
}

int e3_rows(int nky, const E3Args &a, cudaStream_t st)
{
    switch (nky) {
    case 64: return e3_rows_launch<64>(a, st);
    case 128: return e3_rows_launch<128>(a, st);
    case 256: return e3_rows_launch<256>(a, st);
    case 512: return e3_rows_launch<512>(a, st);
    case 1024: return e3_rows_launch<1024>(a, st);
    default: return -2;
    }
}

int e3_cols(int nkx, const E3Args &a, cudaStream_t st)
{
    switch (nkx) {
    case 64: return e3_cols_launch<64>(a, st);
    case 128: return e3_cols_launch<128>(a, st);
    case 256: return e3_cols_launch<256>(a, st);
    case 512: return e3_cols_launch<512>(a, st);
    case 1024: return e3_cols_launch<1024>(a, st);
    default: return -2;
    }
}

bool e3_pow2(int n) { return n >= 64 && n <= 1024 && (n & (n - 1)) == 0; }

}  // namespace gbwem

// ------------------------------------------------------------------ host side
namespace {
using namespace gbwem;

struct Bufs3 {
    std::vector<void *> ptrs;
    ~Bufs3()
    {
        for (void *q : ptrs) cudaFree(q);
    }
    template <class T> T *get(size_t n)
    {
        void *q = nullptr;
        if (cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) return nullptr;
        ptrs.push_back(q);
        return static_cast<T *>(q);
    }
};

// boundary_condition's weights along one axis (ewem.c:533-551): 30 tapered cells at each end
// when the axis has more than 100
void taper_axis(int n, std::vector<float> &t)
{
    t.assign(n, 1.f);
    const int l = n > 100 ? 30 : 0;
    for (int i = 0; i < n; i++) {
        if (i < l) t[i] = expf(-powf(0.015 * ((float)l - i), 2.));
        if (i > n - l) t[i] = expf(-powf(0.015 * ((float)i - n + l), 2.));
    }
}
}  // namespace

#define E3CK(call)                                                                                        \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess) return set_error(WEM_ERR_CUDA, cudaGetErrorString(e_));                   \
    } while (0)
#define E3LAUNCH(call)                                                                                    \
    do {                                                                                                  \
        if ((call) != 0) return set_error(WEM_ERR_CUDA, "wem_elastic: 3-D pass launch failed");          \
    } while (0)

namespace gbwem {

// wem_elastic on a 3-D grid (nmy > 1); the arguments as there, every array over the
// nmx * nmy cells (cell = imx * nmy + imy, the reference's ix). *ms: the device time.
int wem_elastic3d(int device, const wem_params &p, const float *vp, const float *vs, const float *wav, int nshot,
                  const float *sx, const float *sy, float *ux, float *uz, float *mpp, float *mps2, int adj, float *ms)
{
    if (!sy) return set_error(WEM_ERR_ARG, "wem_elastic: 3-D grids need the sources' y positions");
    if (p.nt < 2 || p.nmx < 2 || p.nmy < 2 || p.nz < 1 || p.padt < 1 || p.padx < 1 || !(p.dt > 0) || !(p.dmx > 0) ||
        !(p.dmy > 0))
        return set_error(WEM_ERR_ARG, "wem_elastic: invalid grid");
    const int nmx = p.nmx, nmy = p.nmy, nz = p.nz, nt = p.nt, nn = nmx * nmy;
    // grids with ewem.c's own float expressions (ewem.c:44-57)
    const int ntfft = (int)2 * truncf(p.padt * ((float)nt) / 2);
    const int nw = (int)truncf(ntfft / 2) + 1;
    const int nkx = p.padx * nmx, nky = p.padx * nmy;
    const float dkx = 2 * 3.141592653589793 / ((float)nkx) / p.dmx;
    const float dky = 2 * 3.141592653589793 / ((float)nky) / p.dmy;
    const float dw = 2 * 3.141592653589793 / ((float)ntfft) / p.dt;
    int ifmax, ifmin;
    if (p.fmax * p.dt * ntfft + 1 < nw) ifmax = trunc(p.fmax * p.dt * ntfft) + 1;
    else ifmax = nw;
    if (p.fmin * p.dt * ntfft + 1 < ifmax) ifmin = trunc(p.fmin * p.dt * ntfft);
    else ifmin = 0;
    const int nwf = ifmax - ifmin, nf = (nw - 1) * 2;
    if (!e3_pow2(nkx) || !e3_pow2(nky))
        return set_error(WEM_ERR_SIZE, "wem_elastic: on 3-D grids padx*nmx and padx*nmy must be powers of two in [64, 1024]");
    // slowness split of ewem.c:63-82 over the nmx*nmy cells (float accumulation, double reciprocals)
    std::vector<float> po_p(nz), po_s(nz), pd_p((size_t)nz * nn), pd_s((size_t)nz * nn), vpm(nz), vsm(nz);
    for (int iz = 0; iz < nz; iz++) {
        float sp = 0.f, ss = 0.f;
        for (int ix = 0; ix < nn; ix++) {
            sp += vp[(size_t)ix * nz + iz];
            ss += vs[(size_t)ix * nz + iz];
        }
        sp /= (float)nmx * nmy;
        ss /= (float)nmx * nmy;
        po_p[iz] = 1. / sp;
        po_s[iz] = 1. / ss;
        for (int ix = 0; ix < nn; ix++) {
            pd_p[(size_t)iz * nn + ix] = 1.0 / vp[(size_t)ix * nz + iz] - po_p[iz];
            pd_s[(size_t)iz * nn + ix] = 1.0 / vs[(size_t)ix * nz + iz] - po_s[iz];
        }
        vpm[iz] = 1. / po_p[iz];
        vsm[iz] = 1. / po_s[iz];
    }
    std::vector<float> tapx, tapy;
    taper_axis(nmx, tapx);
    taper_axis(nmy, tapy);
    std::vector<int> cell(nshot);
    for (int s = 0; s < nshot; s++) {
        const int igx = (int)truncf((sx[s] - p.omx) / p.dmx), igy = (int)truncf((sy[s] - p.omy) / p.dmy);  // ewem.c:99-100
        if (igx < 0 || igx >= nmx || igy < 0 || igy >= nmy)
            return set_error(WEM_ERR_ARG, "wem_elastic: a source falls outside the grid");
        cell[s] = igx * nmy + igy;
    }
    float max_source = 0.f;
    for (int it = 0; it < nt; it++)
        if (max_source < fabsf(wav[it]) / sqrtf((float)ntfft)) max_source = fabsf(wav[it]) / sqrtf((float)ntfft);
    if (!(max_source > 0.f)) return set_error(WEM_ERR_ARG, "wem_elastic: the wavelet is zero");
    std::vector<float2> twx(twiddle_table_size(nkx) + 1), twy(twiddle_table_size(nky) + 1);
    twiddle_table_host(nkx, twx.data());
    twiddle_table_host(nky, twy.data());
    std::vector<float2> wtab(nf);
    for (int k = 0; k < nf; k++) {
        const double an = -6.283185307179586476925286766559 * (double)k / (double)nf;
        wtab[k] = make_float2((float)cos(an), (float)sin(an));
    }
    const float sq = sqrtf((float)ntfft);
    std::vector<float> sc_in(std::max(nwf, 1), 1.f / sq), sc_out(std::max(nwf, 1));
    for (int i = 0; i < nwf; i++) {
        const int iw = ifmin + i;
        sc_out[i] = (iw == 0 || 2 * iw == nf) ? 1.f : 2.f;
    }
    // items (shot, frequency), frequency-major
    const int nall = nshot * std::max(nwf, 0);
    std::vector<int> it_iwi(std::max(nall, 1)), it_shot(std::max(nall, 1));
    for (int i = 0; i < nall; i++) {
        it_iwi[i] = i / nshot;
        it_shot[i] = i % nshot;
    }

    E3CK(cudaSetDevice(device));
    int nsm = 0;
    E3CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device));
    cudaStream_t st = nullptr;
    E3CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    struct StreamGuard {
        cudaStream_t s;
        ~StreamGuard() { cudaStreamDestroy(s); }
    } sg{ st };
    Bufs3 B;
    const size_t ntr = (size_t)nshot * nn, nzn = (size_t)nz * nn, nsp = ntr * std::max(nwf, 1);
    float *d_po_p = B.get<float>(nz), *d_po_s = B.get<float>(nz), *d_vpm = B.get<float>(nz), *d_vsm = B.get<float>(nz);
    float *d_pd_p = B.get<float>(nzn), *d_pd_s = B.get<float>(nzn);
    float *d_tx = B.get<float>(nmx), *d_ty = B.get<float>(nmy);
    float2 *d_twx = B.get<float2>(twx.size()), *d_twy = B.get<float2>(twy.size()), *d_wtab = B.get<float2>(nf);
    float *d_scin = B.get<float>(sc_in.size()), *d_scout = B.get<float>(sc_out.size());
    int *d_cell = B.get<int>(nshot), *d_iwi = B.get<int>(it_iwi.size()), *d_shot = B.get<int>(it_shot.size());
    float *d_wav = B.get<float>(nt);
    float2 *d_srcw = B.get<float2>(std::max(nwf, 1));
    int64_t *d_base = B.get<int64_t>(ntr), *d_zero = B.get<int64_t>(1);
    float *d_ux = B.get<float>(ntr * nt), *d_uz = B.get<float>(ntr * nt);
    float2 *d_sx = B.get<float2>(nsp), *d_sz = B.get<float2>(nsp);
    float *d_mp = B.get<float>(nzn), *d_ms = B.get<float>(nzn);
    if (!d_po_p || !d_po_s || !d_vpm || !d_vsm || !d_pd_p || !d_pd_s || !d_tx || !d_ty || !d_twx || !d_twy || !d_wtab ||
        !d_scin || !d_scout || !d_cell || !d_iwi || !d_shot || !d_wav || !d_srcw || !d_base || !d_zero || !d_ux ||
        !d_uz || !d_sx || !d_sz || !d_mp || !d_ms)
        return set_error(WEM_ERR_NOMEM, "wem_elastic: out of device memory");
    std::vector<int64_t> base(ntr);
    for (size_t i = 0; i < ntr; i++) base[i] = (int64_t)((i / nn) * nwf) * nn + (int64_t)(i % nn);
    const int64_t zero = 0;
    E3CK(cudaMemcpyAsync(d_po_p, po_p.data(), sizeof(float) * nz, cudaMemcpyHostToDevice, st));
    E3CK(cudaMemcpyAsync(d_po_s, po_s.data(), sizeof(float) * nz, cudaMemcpyHostToDevice, st));
    E3CK(cudaMemcpyAsync(d_vpm, vpm.data(), sizeof(float) * nz, cudaMemcpyHostToDevice, st));
    E3CK(cudaMemcpyAsync(d_vsm, vsm.data(), sizeof(float) * nz, cudaMemcpyHostToDevice, st));
    E3CK(cudaMemcpyAsync(d_pd_p, pd_p.data(), sizeof(float) * nzn, cudaMemcpyHostToDevice, st));
    E3CK(cudaMemcpyAsync(d_pd_s, pd_s.data(), sizeof(float) * nzn, cudaMemcpyHostToDevice, st));
    E3CK(cudaMemcpyAsync(d_tx, tapx.data(), sizeof(float) * nmx, cudaMemcpyHostToDevice, st));
    E3CK(cudaMemcpyAsync(d_ty, tapy.data(), sizeof(float) * nmy, cudaMemcpyHostToDevice, st));
    E3CK(cudaMemcpyAsync(d_twx, twx.data(), sizeof(float2) * twx.size(), cudaMemcpyHostToDevice, st));
    E3CK(cudaMemcpyAsync(d_twy, twy.data(), sizeof(float2) * twy.size(), cudaMemcpyHostToDevice, st));
    E3CK(cudaMemcpyAsync(d_wtab, wtab.data(), sizeof(float2) * nf, cudaMemcpyHostToDevice, st));
    E3CK(cudaMemcpyAsync(d_scin, sc_in.data(), sizeof(float) * sc_in.size(), cudaMemcpyHostToDevice, st));
    E3CK(cudaMemcpyAsync(d_scout, sc_out.data(), sizeof(float) * sc_out.size(), cudaMemcpyHostToDevice, st));
    E3CK(cudaMemcpyAsync(d_cell, cell.data(), sizeof(int) * nshot, cudaMemcpyHostToDevice, st));
    E3CK(cudaMemcpyAsync(d_iwi, it_iwi.data(), sizeof(int) * it_iwi.size(), cudaMemcpyHostToDevice, st));
    E3CK(cudaMemcpyAsync(d_shot, it_shot.data(), sizeof(int) * it_shot.size(), cudaMemcpyHostToDevice, st));
    E3CK(cudaMemcpyAsync(d_wav, wav, sizeof(float) * nt, cudaMemcpyHostToDevice, st));
    E3CK(cudaMemcpyAsync(d_base, base.data(), sizeof(int64_t) * ntr, cudaMemcpyHostToDevice, st));
    E3CK(cudaMemcpyAsync(d_zero, &zero, sizeof(int64_t), cudaMemcpyHostToDevice, st));
    if (adj) {
        E3CK(cudaMemcpyAsync(d_ux, ux, sizeof(float) * ntr * nt, cudaMemcpyHostToDevice, st));
        E3CK(cudaMemcpyAsync(d_uz, uz, sizeof(float) * ntr * nt, cudaMemcpyHostToDevice, st));
    } else {
        // the images to depth-major planes for the injection
        float *tmp = B.get<float>(nzn);
        if (!tmp) return set_error(WEM_ERR_NOMEM, "wem_elastic: out of device memory");
        E3CK(cudaMemcpyAsync(tmp, mpp, sizeof(float) * nzn, cudaMemcpyHostToDevice, st));
        if (launch_transpose(tmp, nn, nz, d_mp, st)) return set_error(WEM_ERR_CUDA, "wem_elastic: transpose");
        E3CK(cudaStreamSynchronize(st));
        E3CK(cudaMemcpyAsync(tmp, mps2, sizeof(float) * nzn, cudaMemcpyHostToDevice, st));
        if (launch_transpose(tmp, nn, nz, d_ms, st)) return set_error(WEM_ERR_CUDA, "wem_elastic: transpose");
    }
    cudaEvent_t e0, e1;
    E3CK(cudaEventCreate(&e0));
    E3CK(cudaEventCreate(&e1));
    struct EvGuard {
        cudaEvent_t a, b;
        ~EvGuard()
        {
            cudaEventDestroy(a);
            cudaEventDestroy(b);
        }
    } eg{ e0, e1 };
    E3CK(cudaEventRecord(e0, st));
    if (nwf > 0) {
        SpectraArgs sa{};
        // f_op's r2c of length (nw - 1) * 2 (ewem.c:465-471); an odd nt with padt = 1 transforms nt - 1 samples
        sa.d = d_wav; sa.ntr = 1; sa.nt = std::min(nt, nf); sa.ld = nt; sa.ntfft = nf; sa.ifmin = ifmin; sa.nwf = nwf;
        sa.out_base = d_zero; sa.out_fstride = 1; sa.wtab = d_wtab; sa.scale = d_scin; sa.out = d_srcw;
        if (launch_spectra(sa, st)) return set_error(WEM_ERR_CUDA, "wem_elastic: wavelet spectrum launch");
        if (adj) {
            sa.ntr = (int)ntr; sa.out_base = d_base; sa.out_fstride = nn;
            sa.d = d_ux; sa.out = d_sx;
            if (launch_spectra(sa, st)) return set_error(WEM_ERR_CUDA, "wem_elastic: spectra launch");
            sa.d = d_uz; sa.out = d_sz;
            if (launch_spectra(sa, st)) return set_error(WEM_ERR_CUDA, "wem_elastic: spectra launch");
        } else {
            E3CK(cudaMemsetAsync(d_sx, 0, sizeof(float2) * nsp, st));
            E3CK(cudaMemsetAsync(d_sz, 0, sizeof(float2) * nsp, st));
        }
    }
    E3Args a{};
    a.nmx = nmx; a.nmy = nmy; a.nkx = nkx; a.nky = nky; a.nz = nz; a.nwf = nwf; a.ifmin = ifmin; a.adj = adj;
    a.dw = dw; a.dz = p.dz; a.dkx = dkx; a.dky = dky;
    a.inv_s = 1.f / sqrtf((float)nkx * nky);
    a.inv_max_source = 1.f / max_source;
    a.inv_sqt = 1.f / sq;
    a.item_iwi = d_iwi; a.item_shot = d_shot; a.src_cell = d_cell; a.srcw = d_srcw; a.recv_x = d_sx; a.recv_z = d_sz;
    a.po_p = d_po_p; a.po_s = d_po_s; a.vpm = d_vpm; a.vsm = d_vsm; a.pd_p = d_pd_p; a.pd_s = d_pd_s;
    a.tapx = d_tx; a.tapy = d_ty; a.twx = d_twx; a.twy = d_twy;
    a.mpp = d_mp; a.mps2 = d_ms; a.out_x = d_sx; a.out_z = d_sz;
    // depth flags (ewem.c:303-304, 310, 328)
    std::vector<uint8_t> src_on(nz), rec_on(nz);
    for (int iz = 0; iz < nz; iz++) {
        const float z = p.oz + p.dz * iz;
        src_on[iz] = z >= p.sz;
        rec_on[iz] = z >= p.gz;
    }
    // items in flight per batch: the planes (and, forward, the source of every depth) within
    // a quarter of the free memory and 8 GiB; the imaging chunks sized to fill the GPU
    size_t free_b = 0, total_b = 0;
    E3CK(cudaMemGetInfo(&free_b, &total_b));
    const size_t per_item = sizeof(float2) * ((size_t)3 * nmx * nky + (adj ? 0 : nzn));
    const size_t budget = std::min<size_t>((size_t)8 << 30, free_b / 4);
    int batch = (int)std::max<size_t>(1, std::min<size_t>((size_t)std::max(nall, 1), budget / per_item));
    if (const char *e = getenv("WEM_E3_BATCH")) {  // a smaller batch (tests of the batch loop)
        const int b = atoi(e);
        if (b > 0 && b < batch) batch = b;
    }
    const int rows_teams = E3_THREADS / (nky / 16);
    int nchunk = std::max(1, std::min(batch, (nsm * 8 * rows_teams + nmx - 1) / nmx));
    const size_t acc_bytes = sizeof(float2) * nzn;  // per chunk and image
    nchunk = (int)std::max<size_t>(1, std::min<size_t>((size_t)nchunk, (free_b / 8) / (2 * acc_bytes)));
    if (nall > 0) {
        a.K = B.get<float2>((size_t)batch * 3 * nmx * nky);
        if (!a.K) return set_error(WEM_ERR_NOMEM, "wem_elastic: out of device memory");
        if (adj) {
            a.acc_p = B.get<float2>((size_t)nchunk * nzn);
            a.acc_s = B.get<float2>((size_t)nchunk * nzn);
            if (!a.acc_p || !a.acc_s) return set_error(WEM_ERR_NOMEM, "wem_elastic: out of device memory");
            E3CK(cudaMemsetAsync(a.acc_p, 0, sizeof(float2) * nchunk * nzn, st));
            E3CK(cudaMemsetAsync(a.acc_s, 0, sizeof(float2) * nchunk * nzn, st));
        } else {
            a.smig = B.get<float2>((size_t)batch * nzn);
            if (!a.smig) return set_error(WEM_ERR_NOMEM, "wem_elastic: out of device memory");
        }
    }
    auto rows = [&](int op, int mask, int iz, int ipc) {
        a.op = op; a.mask = mask; a.iz = iz; a.ipc = ipc;
        return e3_rows(nky, a, st);
    };
    auto cols = [&](int op, int mask, int iz) {
        a.op = op; a.mask = mask; a.iz = iz;
        return e3_cols(nkx, a, st);
    };
    for (int i0 = 0; i0 < nall; i0 += batch) {
        a.item0 = i0;
        a.nitems = std::min(batch, nall - i0);
        const int ipc_img = (a.nitems + std::min(nchunk, a.nitems) - 1) / std::min(nchunk, a.nitems);
        E3CK(cudaMemsetAsync(a.K, 0, sizeof(float2) * (size_t)a.nitems * 3 * nmx * nky, st));
        if (adj) {
            // source and receivers go down together (elastic_extrap1f, ewem.c:301-325)
            bool src_started = false, rec_started = false;
            for (int iz = 0; iz < nz; iz++) {
                if (src_on[iz] && !src_started) {
                    E3LAUNCH(rows(E3R_LOAD_SRC, 4, iz, 1));
                    src_started = true;
                }
                if (rec_on[iz] && !rec_started) {
                    E3LAUNCH(rows(E3R_LOAD_REC, 3, iz, 1));
                    rec_started = true;
                }
                const int planes = (src_on[iz] ? 4 : 0) | (rec_on[iz] ? 3 : 0);
                if (!planes) continue;
                if (rec_on[iz]) {
                    E3LAUNCH(cols(E3C_SEP, 3, iz));
                    E3LAUNCH(rows(E3R_MID, 3, iz, 1));
                }
                E3LAUNCH(cols(E3C_SSOP, planes, iz));
                // the image only where the receivers are continued; the source alone otherwise
                E3LAUNCH(rows(E3R_IMG, planes, iz, rec_on[iz] ? ipc_img : 1));
                if (rec_on[iz]) {
                    E3LAUNCH(cols(E3C_RECOMB, 3, iz));
                    E3LAUNCH(rows(E3R_MID, 3, iz, 1));
                }
            }
        } else {
            // the source down with every depth kept, then the receivers up (ewem.c:301-309, 326-350)
            E3CK(cudaMemsetAsync(a.smig, 0, sizeof(float2) * (size_t)a.nitems * nzn, st));
            bool src_started = false;
            for (int iz = 0; iz < nz; iz++) {
                if (!src_on[iz]) continue;
                if (!src_started) {
                    E3LAUNCH(rows(E3R_LOAD_SRC, 4, iz, 1));
                    src_started = true;
                }
                E3LAUNCH(cols(E3C_SSOP, 4, iz));
                E3LAUNCH(rows(E3R_SRC_STORE, 4, iz, 1));
            }
            int last = -1;  // the shallowest depth the receivers reach
            for (int iz = 0; iz < nz && last < 0; iz++)
                if (rec_on[iz]) last = iz;
            for (int iz = nz - 1; iz >= 0 && last >= 0; iz--) {
                if (!rec_on[iz]) continue;
                E3LAUNCH(cols(E3C_SEP, 3, iz));
                E3LAUNCH(rows(E3R_INJ, 3, iz, 1));
                E3LAUNCH(cols(E3C_SSOP, 3, iz));
                E3LAUNCH(rows(E3R_MID, 3, iz, 1));
                E3LAUNCH(cols(E3C_RECOMB, 3, iz));
                E3LAUNCH(rows(iz == last ? E3R_OUT : E3R_MID, 3, iz, 1));
            }
        }
    }
    if (adj) {
        if (nall > 0) {
            if (launch_image_reduce(a.acc_p, nchunk, nz, nn, d_mp, st) ||
                launch_image_reduce(a.acc_s, nchunk, nz, nn, d_ms, st))
                return set_error(WEM_ERR_CUDA, "wem_elastic: reduce launch");
        } else {
            E3CK(cudaMemsetAsync(d_mp, 0, sizeof(float) * nzn, st));
            E3CK(cudaMemsetAsync(d_ms, 0, sizeof(float) * nzn, st));
        }
    } else {
        SynthArgs sy{};
        sy.nwf = nwf; sy.ifmin = ifmin; sy.nt = nt; sy.nf = nf; sy.ntr = (int)ntr; sy.in_base = d_base;
        sy.in_fstride = nn; sy.wtab = d_wtab; sy.scale = d_scout;
        sy.dg = d_sx; sy.out = d_ux;
        if (nwf > 0 && launch_synth(sy, st)) return set_error(WEM_ERR_CUDA, "wem_elastic: synthesis launch");
        sy.dg = d_sz; sy.out = d_uz;
        if (nwf > 0 && launch_synth(sy, st)) return set_error(WEM_ERR_CUDA, "wem_elastic: synthesis launch");
        if (nwf <= 0) {
            E3CK(cudaMemsetAsync(d_ux, 0, sizeof(float) * ntr * nt, st));
            E3CK(cudaMemsetAsync(d_uz, 0, sizeof(float) * ntr * nt, st));
        }
    }
    E3CK(cudaEventRecord(e1, st));
    if (adj) {
        E3CK(cudaMemcpyAsync(mpp, d_mp, sizeof(float) * nzn, cudaMemcpyDeviceToHost, st));
        E3CK(cudaMemcpyAsync(mps2, d_ms, sizeof(float) * nzn, cudaMemcpyDeviceToHost, st));
    } else {
        E3CK(cudaMemcpyAsync(ux, d_ux, sizeof(float) * ntr * nt, cudaMemcpyDeviceToHost, st));
        E3CK(cudaMemcpyAsync(uz, d_uz, sizeof(float) * ntr * nt, cudaMemcpyDeviceToHost, st));
    }
    E3CK(cudaStreamSynchronize(st));
    E3CK(cudaEventElapsedTime(ms, e0, e1));
    return WEM_OK;
}

}  // namespace gbwem
