// wem_3d.cu -- the 3-D depth recursion (nmy > 1): the x-y plane of a wavefield
// (padx*nmx by padx*nmy complex samples, 2 MB at 512 x 512) does not fit in shared
// memory, so one depth step of every (shot, frequency) in flight is three batched
// passes over device memory (the planes stay L2/HBM resident between them):
//
//   pass A  rows:    U[x][y]  --FFT_y-->  Y[x][ky]                          (x < nmx)
//   pass B  columns: Y[:, ky] --FFT_x--> A[kx][ky]; for every reference r:
//                    A * P_r(kx, ky) --IFFT_x--> C_r[x][ky]                 (x < nmx)
//   pass C  rows:    C_r[x][:] --IFFT_y--> select/interpolate over r (or the
//                    split-step correction) --> U[x][y]; imaging condition
//
// which is the 2-D transform pair of pspiop/ssop (wem.c:380-471, 289-378: p1/p2 are
// rank-2 FFTW plans over (nkx, nky), wem.c:100-104) split by axis. The source and the
// receiver wavefield of an item are processed by the same CTA in every pass: pass B
// shares the phase values between them (the source uses their conjugates) and pass C
// forms the image. Pass C sums the image over a chunk of items in registers and
// writes one partial image per chunk; wem_image_reduce_kernel adds the chunks.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "wem_fft.cuh"
#include "wem_internal.h"
#include "wem_step.cuh"

namespace gbwem {

// wavefield w (0 source, 1 receiver) steps at this depth: its zflag bit, and in the
// modelling and angle modes only the wavefield being continued (1, 3: source; 2: receiver)
__device__ __forceinline__ bool m3_active(const Mig3dArgs &a, uint8_t zf, int w)
{
    if ((a.mode == 1 || a.mode == 3) && w != 0) return false;
    if ((a.mode == 2 || a.mode == 4) && w != 1) return false;
    return (zf & (w == 0 ? Z_SRC : Z_REC)) != 0;
}

// ---------------------------------------------------------------- pass A
template <int NY>
__global__ void __launch_bounds__(256) wem3d_rows_fwd_kernel(const Mig3dArgs a)
{
    constexpr int TY = NY / 16, TEAMS = 256 / TY;
    constexpr int TW = fft_tw_size<NY>(), TWP = (TW + 1) & ~1;
    extern __shared__ float4 smem_raw[];
    float2 *s_tw = reinterpret_cast<float2 *>(smem_raw);
    float2 *s_x = s_tw + TWP;
    const int tid = threadIdx.x, team = tid / TY, t = tid - team * TY;
    float2 *xbuf = s_x + (size_t)team * pad16(NY);
    const unsigned sync = team_sync_handle<NY>(tid);
    for (int i = tid; i < TW; i += 256) s_tw[i] = a.twy[i];
    __syncthreads();
    const uint8_t zf = a.zflag[a.iz];
    const int n = a.nmx * a.nmy;
    const long long njobs = (long long)a.nitems * 2 * a.nmx;
    for (long long job = (long long)blockIdx.x * TEAMS + team; job < njobs; job += (long long)gridDim.x * TEAMS) {
        const int item = (int)(job / (2 * a.nmx));
        const int rem = (int)(job - (long long)item * 2 * a.nmx);
        const int w = rem / a.nmx, x = rem - w * a.nmx;
        if (!m3_active(a, zf, w)) continue;  // team-uniform
        const float2 *urow = a.U + ((size_t)item * 2 + w) * n + (size_t)x * a.nmy;
        float2 v[16];
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const int y = t + TY * m;
            v[m] = y < a.nmy ? urow[y] : make_float2(0.f, 0.f);
        }
        if (a.mode == 2 || a.mode == 3) {
            // mode 2, receiver going up: inject m * smig (wem.c:270-272); modes 2 and 3 (the
            // angle computation's source, ssop_source wem.c:763-776): for split-step the
            // taper and the correction come before the transform (ssop adj=false, wem.c:321-330)
            const size_t zrow = (size_t)a.iz * n + (size_t)x * a.nmy;
            const float2 *sm = a.smig + ((size_t)item * a.nz + a.iz) * n + (size_t)x * a.nmy;
            const float wv = __fmul_rn((float)(a.ifmin + a.item_iwi[item]), a.dw);
#pragma unroll
            for (int m = 0; m < 16; m++) {
                const int y = t + TY * m;
                if (y < a.nmy) {
                    if (a.mode == 2) {
                        const float mv = a.mimg[zrow + y];
                        const float2 s_ = sm[y];
                        v[m].x += mv * s_.x;
                        v[m].y += mv * s_.y;
                    }
                    if (!a.pspi) {
                        const float tp = a.taper[x] * a.tapery[y];
                        float sn, cs;
                        sincosf(__fmul_rn(__fmul_rn(wv, a.pd[zrow + y]), -a.dz), &sn, &cs);
                        v[m] = cmul(make_float2(v[m].x * tp, v[m].y * tp), make_float2(cs, sn));
                    }
                }
            }
        }
        {
            // the team's next row to L2 while this one is transformed (64 bytes per thread)
            const long long nj = job + (long long)gridDim.x * TEAMS;
            if (nj < njobs && 8 * t < a.nmy) {
                const int item_n = (int)(nj / (2 * a.nmx));
                const int rem_n = (int)(nj - (long long)item_n * 2 * a.nmx);
                const int w_n = rem_n / a.nmx, x_n = rem_n - w_n * a.nmx;
                const float2 *nrow = a.U + ((size_t)item_n * 2 + w_n) * n + (size_t)x_n * a.nmy;
                asm volatile("prefetch.global.L2 [%0];" ::"l"(nrow + 8 * t));
            }
        }
        fft_row<NY, -1>(v, xbuf, s_tw, t, sync);
        float2 *yrow = a.Y + (((size_t)item * 2 + w) * a.nmx + x) * NY;
#pragma unroll
        for (int m = 0; m < 16; m++) yrow[t + TY * m] = v[m];
    }
}

// e^{+2 pi i e / n}, e in [0, n) (n a power of two): sincospif of the exact fraction 2e/n
__device__ __forceinline__ float2 expi_frac(int e, int n)
{
    float sn, cs;
    sincospif(__fdiv_rn(2.f * (float)e, (float)n), &sn, &cs);
    return make_float2(cs, sn);
}

// sum over the team (T <= 32 threads, aligned lanes): every thread gets the total
template <int T> __device__ __forceinline__ float2 team_sum2(float2 v, unsigned lanes)
{
    static_assert(T <= 32, "team within a warp");
#pragma unroll
    for (int off = T / 2; off > 0; off >>= 1) {
        v.x += __shfl_xor_sync(lanes, v.x, off);
        v.y += __shfl_xor_sync(lanes, v.y, off);
    }
    return v;
}

// ---------------------------------------------------------------- pass B
// CTA: 2*CW teams of TX = NX/16 threads -- CW columns of the source (teams 0..CW-1) and of
// the receiver (teams CW..2CW-1) of one item. A job's columns are CW/2 columns ky of the
// first half (1..nky/2) and their mirrors nky - ky, which share the phase table (it
// depends on ky^2); the mirror of the Nyquist column nky/2 is itself, so the last job
// takes column 0 in its place, with a table row of its own.
template <int NX> struct ColShape {
    static constexpr int TX = NX / 16;
    static constexpr int CW = (2 * TX >= 512) ? 1 : (512 / (2 * TX) > 16 ? 16 : 512 / (2 * TX));
    static constexpr int NT = 2 * CW * TX;
    static constexpr int HALF = NX / 2 + 1;
    static constexpr int ROWS = CW / 2 + 1;  // phase-table rows of a job
    static constexpr int TW = fft_tw_size<NX>(), TWP = (TW + 1) & ~1;
};

// ky index of column cc of job block b (see pass B)
__device__ __forceinline__ int col_ky(int b, int cc, int half_cols, int nky)
{
    const int base = 1 + b * half_cols;
    if (cc < half_cols) return base + cc;
    const int kym = nky - (base + cc - half_cols);
    return kym == nky / 2 ? 0 : kym;
}

// the column tile is [2][CW][P] with P = tile_pitch(nmx): a team (one column) walks x with
// unit stride, and P = 2 mod 16 puts the 8 columns x 2 rows a half-warp touches in the
// global copies on 16 different 8-byte banks
__host__ __device__ constexpr int tile_pitch(int nmx) { return ((nmx + 15) & ~15) + 2; }
// two phase tables and two column tiles: reference r works in buffer r % 2 while the
// result of reference r - 1 is copied out of the other; with paired planes (a.plan) the
// two tables hold the pair's references and the columns' spectra follow ([2][CW][NX + 2])
__host__ __device__ constexpr size_t col_smem_bytes(int twp, int half, int cw, int teams, int padn, int nmx,
                                                    int nx = 0, bool paired = false)
{
    return sizeof(float2) * ((size_t)twp + (size_t)2 * (cw / 2 + 1) * half + (size_t)teams * padn +
                             (size_t)2 * 2 * tile_pitch(nmx) * cw + (paired ? (size_t)2 * cw * (nx + 2) : 0));
}

template <int NX, bool PSPI>
__global__ void __launch_bounds__(ColShape<NX>::NT) wem3d_cols_kernel(const Mig3dArgs a)
{
    using CS = ColShape<NX>;
    constexpr int TX = CS::TX, CW = CS::CW, NT = CS::NT, HALF = CS::HALF;
    extern __shared__ float4 smem_raw[];
    float2 *s_tw = reinterpret_cast<float2 *>(smem_raw);
    float2 *s_ph0 = s_tw + CS::TWP;                    // [2][ROWS][HALF] phase tables
    float2 *s_x = s_ph0 + (size_t)2 * CS::ROWS * HALF;  // exchange buffers
    const int pitch = tile_pitch(a.nmx);
    float2 *s_tile0 = s_x + (size_t)2 * CW * pad16(NX);  // [2][2][CW][pitch] column tiles
    const size_t tile_sz = (size_t)2 * CW * pitch;
    float2 *s_spec = s_tile0 + 2 * tile_sz;                // paired planes: [2][CW][NX + 2] spectra
    const int *plan = PSPI && a.plan ? a.plan + (size_t)a.iz * PLAN3_STRIDE : nullptr;
    const int *wp = plan && a.wpos ? a.wpos + (size_t)a.iz * WPOS_STRIDE : nullptr;  // points taken whole
    const int tid = threadIdx.x, team = tid / TX, t = tid - team * TX;
    const int w = team / CW, c = team - w * CW;
    float2 *xbuf = s_x + (size_t)team * pad16(NX);
    const unsigned sync = team_sync_handle<NX>(tid);
    for (int i = tid; i < CS::TW; i += NT) s_tw[i] = a.twx[i];
    const uint8_t zf = a.zflag[a.iz];
    const bool active = m3_active(a, zf, w);
    const bool conj = w == 0 || a.mode == 2;  // -dz: the source, and the modelling receiver
    const int nmx = a.nmx, nky = a.nky, nref = PSPI ? a.nref : 1;
    const int nblk = nky / CW;
    const int iz = a.iz;
    for (int job = blockIdx.x; job < a.nitems * nblk; job += gridDim.x) {
        const int item = job / nblk, blk = job - item * nblk;
        constexpr int H = CW / 2;
        const int ky_c = col_ky(blk, c, H, nky);
        const int row_c = c < H ? c : (ky_c == 0 ? H : c - H);
        const bool zero_col = col_ky(blk, CW - 1, H, nky) == 0;  // this job holds column 0
        const int iw = a.ifmin + a.item_iwi[item];
        const float wv = __fmul_rn((float)iw, a.dw);
        const float w2 = __fmul_rn(wv, wv);
        // columns of tile b to C for reference rr (the wavefields active at this depth)
        // (element e of a wavefield's tile: column cc = e % CW fastest, then x = e / CW)
        auto copy_out = [&](const float2 *tile, int rr) {
            for (int ww = 0; ww < 2; ww++) {
                if (!m3_active(a, zf, ww)) continue;
                float2 *dst = a.C + (((size_t)item * 2 + ww) * nref + rr) * nmx * nky;
                for (int e = tid; e < nmx * CW; e += NT) {
                    const int x = e / CW, cc = e - x * CW;
                    dst[(size_t)x * nky + col_ky(blk, cc, H, nky)] = tile[((size_t)ww * CW + cc) * pitch + x];
                }
            }
        };
        __syncthreads();  // the previous job no longer uses the tiles or the tables
        for (int ww = 0; ww < 2; ww++) {
            const float2 *src = a.Y + ((size_t)item * 2 + ww) * nmx * nky;
            for (int e = tid; e < nmx * CW; e += NT) {
                const int x = e / CW, cc = e - x * CW;
                s_tile0[((size_t)ww * CW + cc) * pitch + x] = src[(size_t)x * nky + col_ky(blk, cc, H, nky)];
            }
        }
        __syncthreads();
        float2 v[16];
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const int x = t + TX * m;
            v[m] = x < nmx ? s_tile0[((size_t)w * CW + c) * pitch + x] : make_float2(0.f, 0.f);
        }
        if (active) fft_row<NX, -1>(v, xbuf, s_tw, t, sync);
        const float slow_po = PSPI ? 0.f : __fmul_rn(a.po[iz], a.po[iz]);
        if (plan) {
            if (active) {
                // the column's spectrum for the pairs' a(-kx, -ky) reads; entry NX = entry 0
                float2 *sp = s_spec + ((size_t)w * CW + c) * (NX + 2);
#pragma unroll
                for (int m = 0; m < 16; m++) sp[t + TX * m] = v[m];
                if (t == 0) sp[NX] = v[0];
            }
            // the column holding -ky: the mirror half, or itself for ky = 0 and nky/2
            const int pc = (ky_c == 0 || ky_c == nky / 2) ? c : (c < H ? c + H : c - H);
            const float2 *sq = s_spec + ((size_t)w * CW + pc) * (NX + 2) + NX - t;  // a(-k) = sq[-TX*m]
            const int np = plan[0];
            for (int sl = 0; sl < np; sl++) {
                const int r1 = plan[1 + 2 * sl], r2 = plan[2 + 2 * sl];
                float2 *s_tile = s_tile0 + (size_t)(sl & 1) * tile_sz;
                // w^2 / vref^2 of the pair's references, read once per slot
                const float wsl1 = r1 >= 0 ? __fmul_rn(w2, a.slow2[(size_t)iz * a.nref + r1]) : 0.f;
                const float wsl2 = r2 >= 0 ? __fmul_rn(w2, a.slow2[(size_t)iz * a.nref + r2]) : 0.f;
                const int half_e = (zero_col ? H + 1 : H) * HALF;
                // every thread is past the previous slot's products before its tables change
                __syncthreads();
                for (int e = tid; e < 2 * half_e; e += NT) {
                    const int which = e >= half_e ? 1 : 0, ee = e - which * half_e;
                    const int rr = ee / HALF, kk = ee - rr * HALF;
                    const int r = which ? r2 : r1;
                    if (r < 0) continue;
                    const int kyi = rr < H ? col_ky(blk, rr, H, nky) : 0;
                    const float ky = __fmul_rn(a.dky, (float)kyi);
                    const float kx = __fmul_rn(a.dkx, (float)kk);
                    const float s2 = __fsub_rn(__fsub_rn(which ? wsl2 : wsl1, __fmul_rn(kx, kx)), __fmul_rn(ky, ky));
                    float2 P;
                    if (s2 >= 0.f) {
                        float sn, cs;
                        sincosf(__fmul_rn(__fsqrt_rn(s2), a.dz), &sn, &cs);
                        P = make_float2(cs, sn);
                    } else {
                        P = make_float2(expf(-__fmul_rn(__fmul_rn(0.2f, __fsqrt_rn(-s2)), fabsf(a.dz))), 0.f);
                    }
                    s_ph0[(size_t)which * CS::ROWS * HALF + ee] = make_float2(P.x * a.inv_n, P.y * a.inv_n);
                }
                __syncthreads();  // tables complete; tile sl % 2 free
                if (active) {
                    const float2 *ph1 = s_ph0 + (size_t)row_c * HALF;
                    const float2 *ph2 = s_ph0 + (size_t)CS::ROWS * HALF + (size_t)row_c * HALF;
                    if constexpr (TX <= 32) {
                        // points taken whole whose reference is in this plane: the column's
                        // sum over kx, S(ky) = sum a(kx) Q(kx, ky) e^{+2 pi i kx x0 / NX}, by
                        // Horner's rule over the thread's wavenumbers, for pass C's sum over ky
                        const int nj = wp ? wp[0] : 0;
                        for (int j = 0; j < nj; j++) {
                            const int cell = wp[1 + j];
                            const int rj = a.selb[(size_t)iz * a.nmx * a.nmy + cell] & 0x7f;
                            if (rj != r1 && rj != r2) continue;
                            const int x0 = cell / a.nmy;
                            const float2 *ph = rj == r1 ? ph1 : ph2;
                            const float2 zz = expi_frac((TX * x0) & (NX - 1), NX);
                            float2 h = make_float2(0.f, 0.f);
#pragma unroll
                            for (int m = 15; m >= 0; m--) {
                                const int k = t + TX * m;
                                const float2 P = ph[k <= NX / 2 ? k : NX - k];
                                h = cadd(cmul(h, zz), conj ? cmulc(v[m], P) : cmul(v[m], P));
                            }
                            const float2 sj = team_sum2<TX>(cmul(h, expi_frac((t * x0) & (NX - 1), NX)), sync);
                            if (t == 0) a.dsum[(((size_t)item * 2 + w) * WHOLE_MAX + j) * nky + ky_c] = sj;
                        }
                    }
                    float2 u[16];
                    if (r2 < 0) {
#pragma unroll
                        for (int m = 0; m < 16; m++) {
                            const int k = t + TX * m;
                            const float2 P = ph1[k <= NX / 2 ? k : NX - k];
                            u[m] = conj ? cmulc(v[m], P) : cmul(v[m], P);
                        }
                    } else {
                        // 2 z = p (Q1 + i Q2) + conj(a(-k)) (conj Q1 + i conj Q2); the 1/2 is
                        // applied where pass C selects the real parts
#pragma unroll
                        for (int m = 0; m < 16; m++) {
                            const int k = t + TX * m, kf = k <= NX / 2 ? k : NX - k;
                            float2 Q1 = ph1[kf], Q2 = ph2[kf];
                            if (conj) {
                                Q1.y = -Q1.y;
                                Q2.y = -Q2.y;
                            }
                            const float2 qm = sq[-TX * m];
                            const float2 M = make_float2(Q1.x - Q2.y, Q1.y + Q2.x);
                            const float2 Pc = make_float2(Q1.x + Q2.y, Q2.x - Q1.y);
                            u[m] = cadd(cmul(v[m], M), cmulc(Pc, qm));
                        }
                    }
                    fft_row<NX, +1>(u, xbuf, s_tw, t, sync);
#pragma unroll
                    for (int m = 0; m < 16; m++) {
                        const int x = t + TX * m;
                        if (x < nmx) s_tile[((size_t)w * CW + c) * pitch + x] = u[m];
                    }
                }
                if (sl > 0) copy_out(s_tile0 + (size_t)((sl - 1) & 1) * tile_sz, sl - 1);
            }
            __syncthreads();
            if (np > 0) copy_out(s_tile0 + (size_t)((np - 1) & 1) * tile_sz, np - 1);
            continue;
        }
        for (int r = 0; r < nref; r++) {
            float2 *s_ph = s_ph0 + (size_t)(r & 1) * CS::ROWS * HALF;
            float2 *s_tile = s_tile0 + (size_t)(r & 1) * tile_sz;
            // phase of reference r: row rr < H for first-half column rr (and its mirror),
            // row H for column 0 when the job holds it; entry [rr][kk], |kx| = kk
            const float slow2 = PSPI ? a.slow2[(size_t)iz * a.nref + r] : slow_po;
            for (int e = tid; e < (zero_col ? H + 1 : H) * HALF; e += NT) {
                const int rr = e / HALF, kk = e - rr * HALF;
                const int kyi = rr < H ? col_ky(blk, rr, H, nky) : 0;  // first half: 1..nky/2
                const float ky = __fmul_rn(a.dky, (float)kyi);
                const float kx = __fmul_rn(a.dkx, (float)kk);
                const float s = __fsub_rn(__fsub_rn(__fmul_rn(w2, slow2), __fmul_rn(kx, kx)), __fmul_rn(ky, ky));
                float2 P;
                if (s >= 0.f) {
                    float sn, cs;
                    sincosf(__fmul_rn(__fsqrt_rn(s), a.dz), &sn, &cs);
                    P = make_float2(cs, sn);
                } else {
                    P = make_float2(expf(-__fmul_rn(__fmul_rn(0.2f, __fsqrt_rn(-s)), fabsf(a.dz))), 0.f);
                }
                s_ph[e] = make_float2(P.x * a.inv_n, P.y * a.inv_n);
            }
            // table r is complete; tile r % 2 is free (its copy-out of reference r - 2 and
            // every read of the input tile came before this barrier in each thread)
            __syncthreads();
            if (active) {
                float2 u[16];
#pragma unroll
                for (int m = 0; m < 16; m++) {
                    const int k = t + TX * m;
                    const float2 P = s_ph[(size_t)row_c * HALF + (k <= NX / 2 ? k : NX - k)];
                    u[m] = conj ? cmulc(v[m], P) : cmul(v[m], P);
                }
                fft_row<NX, +1>(u, xbuf, s_tw, t, sync);
#pragma unroll
                for (int m = 0; m < 16; m++) {
                    const int x = t + TX * m;
                    if (x < nmx) s_tile[((size_t)w * CW + c) * pitch + x] = u[m];
                }
            }
            // reference r - 1 finished before the barrier above: copy it out meanwhile
            if (r > 0) copy_out(s_tile0 + (size_t)((r - 1) & 1) * tile_sz, r - 1);
        }
        __syncthreads();
        copy_out(s_tile0 + (size_t)((nref - 1) & 1) * tile_sz, nref - 1);
    }
}

// ---------------------------------------------------------------- pass C
// CTA of 256 threads: pairs of teams (source, receiver) of TY = NY/16 threads, one
// pair per row x; each pair runs the items of one chunk in turn and keeps the
// chunk's image row in registers.
template <int NY, bool PSPI, int INTERP>
__global__ void __launch_bounds__(256, 2) wem3d_rows_inv_kernel(const Mig3dArgs a)
{
    constexpr int TY = NY / 16, TEAMS = 256 / TY, PAIRS = TEAMS / 2;
    constexpr int TW = fft_tw_size<NY>(), TWP = (TW + 1) & ~1;
    extern __shared__ float4 smem_raw[];
    float2 *s_tw = reinterpret_cast<float2 *>(smem_raw);
    float2 *s_x = s_tw + TWP;
    const int tid = threadIdx.x, team = tid / TY, t = tid - team * TY;
    const int pair = team >> 1, w = team & 1;
    float2 *xbuf = s_x + (size_t)team * pad16(NY);
    const unsigned sync = team_sync_handle<NY>(tid);
    for (int i = tid; i < TW; i += 256) s_tw[i] = a.twy[i];
    __syncthreads();
    const int iz = a.iz, nmx = a.nmx, nmy = a.nmy, nky = a.nky, n = nmx * nmy;
    const int nref = PSPI ? a.nref : 1;
    const uint8_t zf = a.zflag[iz];
    const bool active = m3_active(a, zf, w);
    const int nchunk = (a.nitems + a.chunk - 1) / a.chunk;
    const long long njobs = (long long)nchunk * nmx;
    // the pair's partner buffer for the imaging condition: the source team's xbuf
    float2 *src_buf = s_x + (size_t)(pair * 2) * pad16(NY);
    for (long long job = (long long)blockIdx.x * PAIRS + pair; job < njobs; job += (long long)gridDim.x * PAIRS) {
        const int ch = (int)(job / nmx), x = (int)(job - (long long)ch * nmx);
        const int it0 = ch * a.chunk, it1 = min(a.nitems, it0 + a.chunk);
        float img[16];
#pragma unroll
        for (int m = 0; m < 16; m++) img[m] = 0.f;
        // per-position selection of this depth and row
        uint32_t selp[4] = { 0, 0, 0, 0 };
        if (PSPI) {
#pragma unroll
            for (int m = 0; m < 16; m++) {
                const int y = t + TY * m;
                const uint32_t b = y < nmy ? a.selb[(size_t)iz * n + (size_t)x * nmy + y] : 0x7fu;
                selp[m >> 2] |= b << (8 * (m & 3));
            }
        }
        for (int item = it0; item < it1; item++) {
            const int iwi = a.item_iwi[item];
            const int iw = a.ifmin + iwi;
            const float wv = __fmul_rn((float)iw, a.dw);
            const float factor = iw == 0 ? 1.f : 2.f;
            float2 *urow = a.U + ((size_t)item * 2 + w) * n + (size_t)x * nmy;
            float2 unew[16];
            if (active) {
                float2 acc[16];
#pragma unroll
                for (int m = 0; m < 16; m++) acc[m] = make_float2(0.f, 0.f);
                // planes: one per reference, or (paired planes, a.plan) the real parts of two
                // references in one plane and one plane per reference taken whole
                const int *plan = (PSPI && INTERP == 0 && a.plan) ? a.plan + (size_t)iz * PLAN3_STRIDE : nullptr;
                const int np = a.mode == 4 ? 0 : (plan ? plan[0] : nref);
                if (a.mode == 4) {
                    // the exact adjoint's receiver (pass B summed the references): one plane in Y
                    const float2 *yrow = a.Y + (((size_t)item * 2 + w) * nmx + x) * nky;
#pragma unroll
                    for (int m = 0; m < 16; m++) acc[m] = yrow[t + TY * m];
                    fft_row<NY, +1>(acc, xbuf, s_tw, t, sync);
                }
                for (int pl = 0; pl < np; pl++) {
                    const float2 *crow = a.C + ((((size_t)item * 2 + w) * nref + pl) * nmx + x) * nky;
                    float2 u[16];
#pragma unroll
                    for (int m = 0; m < 16; m++) u[m] = crow[t + TY * m];
                    // the next plane's row (or the next item's first) to L2 while this one is
                    // transformed: 128 bytes per thread cover the row (NY samples, NY/16 threads)
                    if (pl + 1 < np || item + 1 < it1) {
                        const float2 *nrow = pl + 1 < np ? crow + (size_t)nmx * nky
                                                         : a.C + ((((size_t)(item + 1) * 2 + w) * nref) * nmx + x) * nky;
                        asm volatile("prefetch.global.L2 [%0];" ::"l"(nrow + 16 * t));
                    }
                    fft_row<NY, +1>(u, xbuf, s_tw, t, sync);
                    if (plan) {
                        const int r1 = plan[1 + 2 * pl], r2 = plan[2 + 2 * pl];
#pragma unroll
                        for (int m = 0; m < 16; m++) {
                            const uint32_t b = (selp[m >> 2] >> (8 * (m & 3))) & 0xffu;
                            const int i1 = (int)(b & 0x7fu);
                            if (i1 == r1) {
                                if (r2 >= 0) acc[m] = make_float2(0.5f * u[m].x, 0.f);
                                else acc[m] = (b & 0x80u) ? make_float2(u[m].x, 0.f) : u[m];
                            } else if (r2 >= 0 && i1 == r2) {
                                acc[m] = make_float2(0.5f * u[m].y, 0.f);
                            }
                        }
                        continue;
                    }
                    const int r = pl;  // one plane per reference
#pragma unroll
                    for (int m = 0; m < 16; m++) {
                        if (PSPI) {
                            const uint32_t b = (selp[m >> 2] >> (8 * (m & 3))) & 0xffu;
                            const int i1 = (int)(b & 0x7fu);
                            const bool interp = (b & 0x80u) != 0;
                            if (INTERP == 0) {
                                if (r == i1) acc[m] = interp ? make_float2(u[m].x, 0.f) : u[m];
                            } else if (!interp) {
                                if (r == i1) acc[m] = u[m];
                            } else if (r == i1 || r == i1 + 1) {
                                const int y = t + TY * m;
                                const float wl = a.wlin[(size_t)iz * n + (size_t)x * nmy + y];
                                const float g = r == i1 ? 1.f - wl : wl;
                                acc[m].x += u[m].x * g;
                                acc[m].y += u[m].y * g;
                            }
                        } else {
                            acc[m] = u[m];
                        }
                    }
                }
                if constexpr (PSPI && INTERP == 0 && TY <= 32) {
                    // points of this row taken whole: Im dref(x0, y0) = Im sum_ky S(ky)
                    // e^{+2 pi i ky y0 / NY} over pass B's column sums (Horner, team sum)
                    const int *wp = (a.plan && a.wpos && a.mode != 4) ? a.wpos + (size_t)iz * WPOS_STRIDE : nullptr;
                    const int nj = wp ? wp[0] : 0;
                    for (int j = 0; j < nj; j++) {
                        const int cell = wp[1 + j];
                        if (cell / nmy != x) continue;
                        const int y0 = cell - x * nmy;
                        const float2 *ds = a.dsum + (((size_t)item * 2 + w) * WHOLE_MAX + j) * nky;
                        const float2 zz = expi_frac((TY * y0) & (NY - 1), NY);
                        float2 h = make_float2(0.f, 0.f);
#pragma unroll
                        for (int m = 15; m >= 0; m--) h = cadd(cmul(h, zz), ds[t + TY * m]);
                        const float2 tot = team_sum2<TY>(cmul(h, expi_frac((t * y0) & (NY - 1), NY)), sync);
                        if (t == y0 % TY) {
                            const int mj = y0 / TY;
#pragma unroll
                            for (int m = 0; m < 16; m++)
                                if (m == mj) acc[m].y = tot.y;
                        }
                    }
                }
#pragma unroll
                for (int m = 0; m < 16; m++) {
                    const int y = t + TY * m;
                    float2 q = make_float2(0.f, 0.f);
                    if (y < nmy) {
                        q = acc[m];
                        if (!PSPI && a.mode != 2 && a.mode != 3) {
                            // split-step correction and taper (wem.c:349-359), -dz for the source
                            const float th = __fmul_rn(__fmul_rn(wv, a.pd[(size_t)iz * n + (size_t)x * nmy + y]), a.dz);
                            float sn, cs;
                            sincosf(th, &sn, &cs);
                            const float tp = a.taper[x] * a.tapery[y];
                            const float2 cr = make_float2(cs * tp, sn * tp);
                            q = w == 0 ? cmulc(q, cr) : cmul(q, cr);
                        }
                        urow[y] = q;
                    }
                    unew[m] = q;
                }
                if (a.mode == 1 || a.mode == 3) {  // keep the source of this depth (wem.c:260, 720)
                    float2 *sm = a.smig + ((size_t)item * a.nz + iz) * n + (size_t)x * nmy;
#pragma unroll
                    for (int m = 0; m < 16; m++) {
                        const int y = t + TY * m;
                        if (y < nmy) sm[y] = unew[m];
                    }
                }
            } else {
#pragma unroll
                for (int m = 0; m < 16; m++) {
                    const int y = t + TY * m;
                    unew[m] = y < nmy ? urow[y] : make_float2(0.f, 0.f);
                }
            }
            if ((a.mode == 1 || a.mode == 3) && w == 0 && !active) {  // none above its depth (wem.c:262-264)
                float2 *sm = a.smig + ((size_t)item * a.nz + iz) * n + (size_t)x * nmy;
#pragma unroll
                for (int m = 0; m < 16; m++) {
                    const int y = t + TY * m;
                    if (y < nmy) sm[y] = make_float2(0.f, 0.f);
                }
            }
            if (a.mode == 0 && (zf & Z_REC)) {
                // imaging condition (wem.c:243-247): the pair meets in the source team's buffer
                team_pair_sync<NY>(pair, tid);
                if (w == 0) {
#pragma unroll
                    for (int m = 0; m < 16; m++) {
                        const int y = t + TY * m;
                        if (y < nmy) src_buf[y] = unew[m];
                    }
                }
                team_pair_sync<NY>(pair, tid);
                if (w == 1) {
#pragma unroll
                    for (int m = 0; m < 16; m++) {
                        const int y = t + TY * m;
                        if (y < nmy) {
                            const float2 s_ = src_buf[y];
                            img[m] += factor * (unew[m].x * s_.x + unew[m].y * s_.y);
                        }
                    }
                }
                team_pair_sync<NY>(pair, tid);
            }
        }
        if (w == 1 && a.mode == 0) {
            float2 *part = a.img_parts + ((size_t)ch * a.nz + iz) * n + (size_t)x * nmy;
#pragma unroll
            for (int m = 0; m < 16; m++) {
                const int y = t + TY * m;
                if (y < nmy) part[y] = make_float2(img[m], 0.f);
            }
        }
    }
}

// ---------------------------------------------------------------- exact adjoint (mode 4)
// The receiver of the exact modelling goes up with the adjoint of the migration step:
// y = IFFT2( sum_r conj(P_r) FFT2( W_r^T u ) ), W_r the transposed selection / interpolation
// weights of reference r (the real-part projection where the nearest-lower mode keeps Re).
// Pass A': m * smig injected, then per reference in use the weighted row's y transform into
// C plane r; pass B': per column the x transforms of the references' planes times conj(P_r),
// summed, transformed back into the Y plane; pass C (mode 4) transforms that plane back in y.
template <int NY, int INTERP>
__global__ void __launch_bounds__(256) wem3d_rows_fwd_adj_kernel(const Mig3dArgs a)
{
    constexpr int TY = NY / 16, TEAMS = 256 / TY;
    constexpr int TW = fft_tw_size<NY>(), TWP = (TW + 1) & ~1;
    extern __shared__ float4 smem_raw[];
    float2 *s_tw = reinterpret_cast<float2 *>(smem_raw);
    float2 *s_x = s_tw + TWP;
    const int tid = threadIdx.x, team = tid / TY, t = tid - team * TY;
    float2 *xbuf = s_x + (size_t)team * pad16(NY);
    const unsigned sync = team_sync_handle<NY>(tid);
    for (int i = tid; i < TW; i += 256) s_tw[i] = a.twy[i];
    __syncthreads();
    const int iz = a.iz, n = a.nmx * a.nmy, nmy = a.nmy;
    if (!(a.zflag[iz] & Z_REC)) return;  // the receiver does not step here: nothing to transform
    const unsigned long long used = a.refmask ? a.refmask[iz] : ~0ull;
    const long long njobs = (long long)a.nitems * a.nmx;
    for (long long job = (long long)blockIdx.x * TEAMS + team; job < njobs; job += (long long)gridDim.x * TEAMS) {
        const int item = (int)(job / a.nmx), x = (int)(job - (long long)item * a.nmx);
        const size_t zrow = (size_t)iz * n + (size_t)x * nmy;
        const float2 *urow = a.U + ((size_t)item * 2 + 1) * n + (size_t)x * nmy;
        const float2 *sm = a.smig + ((size_t)item * a.nz + iz) * n + (size_t)x * nmy;
        float2 v[16];
        uint32_t selp[4] = { 0, 0, 0, 0 };
        float wl[16];
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const int y = t + TY * m;
            float2 q = make_float2(0.f, 0.f);
            uint32_t b = 0x7fu;
            wl[m] = 0.f;
            if (y < nmy) {
                q = urow[y];
                const float mv = a.mimg[zrow + y];
                const float2 s_ = sm[y];
                q.x += mv * s_.x;  // injection (wem.c:270-272)
                q.y += mv * s_.y;
                b = a.selb[zrow + y];
                if (INTERP == 1) wl[m] = a.wlin[zrow + y];
            }
            v[m] = q;
            selp[m >> 2] |= b << (8 * (m & 3));
        }
        for (int r = 0; r < a.nref; r++) {
            if (!((used >> r) & 1ull)) continue;  // team-uniform
            float2 u[16];
#pragma unroll
            for (int m = 0; m < 16; m++) {
                bool re_only;
                const float g = sel_weight<INTERP>(selp, wl, m, r, re_only);
                u[m] = make_float2(v[m].x * g, re_only ? 0.f : v[m].y * g);
            }
            fft_row<NY, -1>(u, xbuf, s_tw, t, sync);
            float2 *crow = a.C + ((((size_t)item * 2 + 1) * a.nref + r) * a.nmx + x) * NY;
#pragma unroll
            for (int m = 0; m < 16; m++) crow[t + TY * m] = u[m];
        }
    }
}

template <int NX>
__global__ void __launch_bounds__(ColShape<NX>::NT) wem3d_cols_adj_kernel(const Mig3dArgs a)
{
    using CS = ColShape<NX>;
    constexpr int TX = CS::TX, CW = CS::CW, NT = CS::NT, HALF = CS::HALF;
    extern __shared__ float4 smem_raw[];
    float2 *s_tw = reinterpret_cast<float2 *>(smem_raw);
    float2 *s_ph = s_tw + CS::TWP;                    // [ROWS][HALF] phase table of one reference
    float2 *s_x = s_ph + (size_t)2 * CS::ROWS * HALF;  // exchange buffers (the layout of pass B)
    const int pitch = tile_pitch(a.nmx);
    float2 *s_tile = s_x + (size_t)2 * CW * pad16(NX);  // [2][CW][pitch]: the receiver half is used
    const int tid = threadIdx.x, team = tid / TX, t = tid - team * TX;
    const int w = team / CW, c = team - w * CW;
    float2 *xbuf = s_x + (size_t)team * pad16(NX);
    const unsigned sync = team_sync_handle<NX>(tid);
    for (int i = tid; i < CS::TW; i += NT) s_tw[i] = a.twx[i];
    const int iz = a.iz, nmx = a.nmx, nky = a.nky, nblk = nky / CW;
    const bool active = w == 1 && (a.zflag[iz] & Z_REC);
    const bool step = (a.zflag[iz] & Z_REC) != 0;  // CTA-uniform
    const unsigned long long used = a.refmask ? a.refmask[iz] : ~0ull;
    constexpr int H = CW / 2;
    for (int job = blockIdx.x; step && job < a.nitems * nblk; job += gridDim.x) {
        const int item = job / nblk, blk = job - item * nblk;
        const int ky_c = col_ky(blk, c, H, nky);
        const int row_c = c < H ? c : (ky_c == 0 ? H : c - H);
        const bool zero_col = col_ky(blk, CW - 1, H, nky) == 0;
        const float wv = __fmul_rn((float)(a.ifmin + a.item_iwi[item]), a.dw);
        const float w2 = __fmul_rn(wv, wv);
        float2 acc[16];
#pragma unroll
        for (int m = 0; m < 16; m++) acc[m] = make_float2(0.f, 0.f);
        for (int r = 0; r < a.nref; r++) {
            if (!((used >> r) & 1ull)) continue;
            __syncthreads();  // the previous reference's table and tile are no longer read
            const float2 *src = a.C + (((size_t)item * 2 + 1) * a.nref + r) * nmx * nky;
            for (int e = tid; e < nmx * CW; e += NT) {
                const int x = e / CW, cc = e - x * CW;
                s_tile[((size_t)CW + cc) * pitch + x] = src[(size_t)x * nky + col_ky(blk, cc, H, nky)];
            }
            const float slow2 = a.slow2[(size_t)iz * a.nref + r];
            for (int e = tid; e < (zero_col ? H + 1 : H) * HALF; e += NT) {
                const int rr = e / HALF, kk = e - rr * HALF;
                const int kyi = rr < H ? col_ky(blk, rr, H, nky) : 0;
                const float ky = __fmul_rn(a.dky, (float)kyi);
                const float kx = __fmul_rn(a.dkx, (float)kk);
                const float s2 = __fsub_rn(__fsub_rn(__fmul_rn(w2, slow2), __fmul_rn(kx, kx)), __fmul_rn(ky, ky));
                float2 P;
                if (s2 >= 0.f) {
                    float sn, cs;
                    sincosf(__fmul_rn(__fsqrt_rn(s2), a.dz), &sn, &cs);
                    P = make_float2(cs, sn);
                } else {
                    P = make_float2(expf(-__fmul_rn(__fmul_rn(0.2f, __fsqrt_rn(-s2)), fabsf(a.dz))), 0.f);
                }
                s_ph[e] = make_float2(P.x * a.inv_n, P.y * a.inv_n);
            }
            __syncthreads();
            if (active) {
                float2 v[16];
#pragma unroll
                for (int m = 0; m < 16; m++) {
                    const int x = t + TX * m;
                    v[m] = x < nmx ? s_tile[((size_t)CW + c) * pitch + x] : make_float2(0.f, 0.f);
                }
                fft_row<NX, -1>(v, xbuf, s_tw, t, sync);
#pragma unroll
                for (int m = 0; m < 16; m++) {
                    const int k = t + TX * m;
                    const float2 q = cmulc(v[m], s_ph[(size_t)row_c * HALF + (k <= NX / 2 ? k : NX - k)]);
                    acc[m].x += q.x;
                    acc[m].y += q.y;
                }
            }
        }
        if (active) fft_row<NX, +1>(acc, xbuf, s_tw, t, sync);
        __syncthreads();  // every team is past its last tile read
        if (active) {
#pragma unroll
            for (int m = 0; m < 16; m++) {
                const int x = t + TX * m;
                if (x < nmx) s_tile[((size_t)CW + c) * pitch + x] = acc[m];
            }
        }
        __syncthreads();
        float2 *dst = a.Y + ((size_t)item * 2 + 1) * nmx * nky;
        for (int e = tid; e < nmx * CW; e += NT) {
            const int x = e / CW, cc = e - x * CW;
            dst[(size_t)x * nky + col_ky(blk, cc, H, nky)] = s_tile[((size_t)CW + cc) * pitch + x];
        }
    }
}

// initial planes: source spike at (igx, igy), receiver spectra (wem.c:230-233)
__global__ void wem3d_init_kernel(const Mig3dArgs a)
{
    const int n = a.nmx * a.nmy;
    const long long total = (long long)a.nitems * 2 * n;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int item = (int)(e / (2 * n));
        const int rem = (int)(e - (long long)item * 2 * n);
        const int w = rem / n, cell = rem - w * n;
        const int shot = a.item_shot[item], iwi = a.item_iwi[item];
        float2 v;
        if (w == 0) v = cell == a.src_cell[shot] ? a.srcw[iwi] : make_float2(0.f, 0.f);
        else v = a.mode == 0 ? a.recv[((size_t)shot * a.nwf + iwi) * n + cell] : make_float2(0.f, 0.f);
        a.U[e] = v;
    }
}

// ---------------------------------------------------------------- host side
template <int NY> static int rows_fwd(const Mig3dArgs &a, int grid, cudaStream_t st)
{
    constexpr int TW = fft_tw_size<NY>(), TWP = (TW + 1) & ~1;
    const size_t smem = sizeof(float2) * ((size_t)TWP + (size_t)(256 / (NY / 16)) * pad16(NY));
    auto k = wem3d_rows_fwd_kernel<NY>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return -1;
    k<<<grid, 256, smem, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <int NY, bool PSPI, int INTERP> static int rows_inv(const Mig3dArgs &a, int grid, cudaStream_t st)
{
    constexpr int TW = fft_tw_size<NY>(), TWP = (TW + 1) & ~1;
    const size_t smem = sizeof(float2) * ((size_t)TWP + (size_t)(256 / (NY / 16)) * pad16(NY));
    auto k = wem3d_rows_inv_kernel<NY, PSPI, INTERP>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return -1;
    k<<<grid, 256, smem, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <int NX, bool PSPI> static int cols(const Mig3dArgs &a, int grid, cudaStream_t st, size_t *smem_out)
{
    using CS = ColShape<NX>;
    const size_t smem = col_smem_bytes(CS::TWP, CS::HALF, CS::CW, 2 * CS::CW, pad16(NX), a.nmx, NX, PSPI && a.plan);
    if (smem_out) { *smem_out = smem; return 0; }
    auto k = wem3d_cols_kernel<NX, PSPI>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return -1;
    k<<<grid, CS::NT, smem, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

#define W3_SWITCH(n, CALL)              \
    switch (n) {                        \
    case 64: return CALL(64);           \
    case 128: return CALL(128);         \
    case 256: return CALL(256);         \
    case 512: return CALL(512);         \
    case 1024: return CALL(1024);       \
    default: return -1;                 \
    }

int m3d_supported(int nkx, int nky)
{
    auto ok = [](int n) { return n == 64 || n == 128 || n == 256 || n == 512 || n == 1024; };
    return ok(nkx) && ok(nky);
}

int m3d_cols_block(int nkx)
{
#define CALL(N) ColShape<N>::CW
    W3_SWITCH(nkx, CALL)
#undef CALL
}

int m3d_cols_smem(int nkx, int pspi, const Mig3dArgs &a, size_t *smem)
{
#define CALL(N) (pspi ? cols<N, true>(a, 0, 0, smem) : cols<N, false>(a, 0, 0, smem))
    W3_SWITCH(nkx, CALL)
#undef CALL
}

template <int NY, int INTERP> static int rows_fwd_adj(const Mig3dArgs &a, int grid, cudaStream_t st)
{
    constexpr int TW = fft_tw_size<NY>(), TWP = (TW + 1) & ~1;
    const size_t smem = sizeof(float2) * ((size_t)TWP + (size_t)(256 / (NY / 16)) * pad16(NY));
    auto k = wem3d_rows_fwd_adj_kernel<NY, INTERP>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return -1;
    k<<<grid, 256, smem, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <int NX> static int cols_adj(const Mig3dArgs &a, int grid, cudaStream_t st)
{
    using CS = ColShape<NX>;
    const size_t smem = col_smem_bytes(CS::TWP, CS::HALF, CS::CW, 2 * CS::CW, pad16(NX), a.nmx);
    auto k = wem3d_cols_adj_kernel<NX>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return -1;
    k<<<grid, CS::NT, smem, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int m3d_launch_step(int nkx, int nky, int pspi, int interp, const Mig3dArgs &a, int nsm, cudaStream_t st)
{
    int rc;
    if (a.mode == 4) {  // the exact adjoint's receiver step (PSPI)
        if (!pspi) return -1;
#define CALL(N) (interp == 0 ? rows_fwd_adj<N, 0>(a, nsm * 4, st) : rows_fwd_adj<N, 1>(a, nsm * 4, st))
        rc = [&]() { W3_SWITCH(nky, CALL) }();
#undef CALL
        if (rc) return rc;
#define CALL(N) cols_adj<N>(a, nsm * 2, st)
        rc = [&]() { W3_SWITCH(nkx, CALL) }();
#undef CALL
        if (rc) return rc;
#define CALL(N) (interp == 0 ? rows_inv<N, true, 0>(a, nsm * 4, st) : rows_inv<N, true, 1>(a, nsm * 4, st))
        rc = [&]() { W3_SWITCH(nky, CALL) }();
#undef CALL
        return rc;
    }
#define CALL(N) rows_fwd<N>(a, nsm * 4, st)
    rc = [&]() { W3_SWITCH(nky, CALL) }();
#undef CALL
    if (rc) return rc;
#define CALL(N) (pspi ? cols<N, true>(a, nsm * 2, st, nullptr) : cols<N, false>(a, nsm * 2, st, nullptr))
    rc = [&]() { W3_SWITCH(nkx, CALL) }();
#undef CALL
    if (rc) return rc;
#define CALL(N) (!pspi ? rows_inv<N, false, 0>(a, nsm * 4, st) : interp == 0 ? rows_inv<N, true, 0>(a, nsm * 4, st) : rows_inv<N, true, 1>(a, nsm * 4, st))
    rc = [&]() { W3_SWITCH(nky, CALL) }();
#undef CALL
    return rc;
}

int m3d_launch_init(const Mig3dArgs &a, cudaStream_t st)
{
    wem3d_init_kernel<<<1024, 256, 0, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// the modelled receiver planes at the surface (wem.c:278-280)
__global__ void wem3d_collect_kernel(const Mig3dArgs a, float2 *dg, float scale)
{
    const int n = a.nmx * a.nmy;
    const long long total = (long long)a.nitems * n;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int item = (int)(e / n), cell = (int)(e - (long long)item * n);
        const float2 u = a.U[((size_t)item * 2 + 1) * n + cell];
        dg[((size_t)a.item_shot[item] * a.nwf + a.item_iwi[item]) * n + cell] = make_float2(u.x * scale, u.y * scale);
    }
}

int m3d_launch_collect(const Mig3dArgs &a, float2 *dg, float scale, cudaStream_t st)
{
    wem3d_collect_kernel<<<1024, 256, 0, st>>>(a, dg, scale);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace gbwem
