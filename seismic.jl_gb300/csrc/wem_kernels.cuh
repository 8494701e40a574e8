// wem_kernels.cuh -- the depth-recursion kernels as templates over the row length N
// (migration and Born modelling) and their per-N launch helpers. Each N is
// instantiated in its own translation unit (wem_n<N>.cu) so that the build
// compiles them in parallel.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "wem_fft.cuh"
#include "wem_internal.h"
#include "wem_step.cuh"

namespace gbwem {

// ------------------------------------------------------------------ migration
// TC (split16 mode, N = 2048): the FFTs' DFT stages run on the tensor cores; each
// team gets 32 TMEM columns for its accumulators and an mbarrier.
// PAIR (PSPI nearest-lower mode, FP32): the step of step_mig_paired, with an N-sample
// spectrum buffer per team in place of the selection accumulator.
// BLU (FP32): transforms of length a.nlog (not a power of two) on rows of N samples,
// N >= 2 a.nlog - 1, in Bluestein's chirp form (xform in wem_step.cuh).
// GT (PSPI FP32, one transform per reference): the depth's phase tables are read from the
// precomputed tables in device memory (through L2) instead of being copied into shared
// memory, for reference counts whose tables do not fit there (a.ptab required).
template <int N, bool PSPI, int INTERP, int S, bool TC = false, bool PAIR = false, bool BLU = false, bool GT = false>
__global__ void __launch_bounds__(2 * S * (N / 16), 1) wem_migrate_kernel(const MigArgs a)
{
    static_assert(!PAIR || (PSPI && INTERP == 0 && !TC), "paired transforms: PSPI nearest-lower mode, FP32");
    static_assert(!BLU || (!PAIR && !TC), "Bluestein rows: FP32, one transform per reference");
    static_assert(!GT || (PSPI && !PAIR && !TC && !BLU), "tables in device memory: PSPI FP32, one transform per reference");
    using SH = MigShape<N>;
    constexpr int T = SH::T, PADN = SH::PADN;
    constexpr int NT = 2 * S * T;
    extern __shared__ float4 smem_raw[];
    const Smem<N, PSPI, BLU> sm(smem_raw, GT ? 0 : a.nref, a.nmx, 2 * S, PAIR);
    if (GT && !a.ptab) return;  // the host launches this form only with the tables in place

    const int tid = threadIdx.x;
    const int team = tid / T, t = tid - team * T;
    const bool is_src = team < S;
    const int sg = is_src ? team : team - S;               // shot within the group
    float2 *xbuf = sm.x + (size_t)team * PADN;
    float2 *sacc = sm.acc + (size_t)team * sm.acc_stride;
    const unsigned sync = team_sync_handle<N>(tid);

    for (int i = tid; i < SH::TW; i += NT) sm.tw[i] = a.twid[i];
    if constexpr (PAIR)
        for (int i = tid; i <= N / 2; i += NT) sm.wd[i] = a.wdot[i];

    TcTeam tc{};
    constexpr uint32_t TCOLS = 2 * S * 32 < 32 ? 32 : 2 * S * 32;  // power of two for 2S in {1, 2, 4}
    uint32_t *tslot = nullptr;
    if constexpr (TC) {
        uint4 *w = reinterpret_cast<uint4 *>(sm.tcx);
        for (int i = tid; i < TC_W_BYTES / 16; i += NT) w[i] = a.tcw[i];
        fence_async_smem();  // the W operands become visible to the tensor core
        uint64_t *mb = reinterpret_cast<uint64_t *>(sm.tcx + TC_W_BYTES);
        float *red = reinterpret_cast<float *>(mb + 2 * S);
        tslot = reinterpret_cast<uint32_t *>(red + 4 * 2 * S);
        int *abort = reinterpret_cast<int *>(tslot + 1);
        if (tid == 0) {
            for (int i = 0; i < 2 * S; i++) mbar_init(smem_u32(&mb[i]), 1);
            *abort = 0;
            mbar_init_fence();
        }
        if (tid < 32) tmem_alloc(tslot, TCOLS);
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        tc.red = red + 4 * team;
        tc.a = smem_u32(xbuf);
        tc.w = smem_u32(w);
        tc.d = *tslot + 32u * team;
        tc.dw = tc.d + ((uint32_t)(32 * ((t >> 5) & 3)) << 16);
        tc.mbar = smem_u32(&mb[team]);
        tc.phase = 0;
        tc.abort = abort;
        tc.err = a.err;
    }

    // the bulk-copy path of the precomputed tables: the CTA's mbarrier, its phase, the
    // abort flag of a wait that ran out
    __shared__ __align__(8) uint64_t s_tbar;
    __shared__ int s_tabort;
    const bool tma = PSPI && a.ptab && a.tma;
    uint32_t tphase = 0;
    if (tma) {
        if (tid == 0) {
            mbar_init(smem_u32(&s_tbar), 1);
            s_tabort = 0;
            mbar_init_fence();
        }
        __syncthreads();
    }

    float2 *slot = a.slots + (size_t)blockIdx.x * a.nz * a.nmx;
    const int nitems = a.ngroups * a.nwf;
    // split-step: a second set of depth tables after the shared-memory layout. Where a shot group
    // is part-filled (a one-shot survey leaves all but one slot empty), the empty slots' teams
    // build the next depth's tables into the other set while the live teams run the current
    // depth, so that the table build leaves the depth chain's critical path.
    Smem<N, PSPI, BLU> sm1 = sm;
    if constexpr (!PSPI && !TC) {
        sm1.ph = reinterpret_cast<float2 *>(reinterpret_cast<char *>(smem_raw) +
                                            mig_smem_bytes<N>(false, a.nref, a.nmx, 2 * S, false, false, BLU));
        sm1.corr = sm1.ph + ph_entries<N, BLU>(false, a.nref);
    }
    const int nmx = a.nmx;
    bool tables_free = true;  // no thread still reads the tables of the previous step

    for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
        const int g = item % a.ngroups;
        const int iwi = item / a.ngroups;
        const int shot = g * S + sg;
        const bool shot_ok = shot < a.nshot;
        const int iw = a.ifmin + iwi;
        const float w = __fmul_rn((float)iw, a.dw);        // w = iw*dw, wem.c:228
        const float w2 = __fmul_rn(w, w);
        const float factor = iw == 0 ? 1.f : 2.f;          // wem.c:226-227

        // split-step, part-filled group: the tables of depth 0 by every thread, the later ones by
        // the empty slots' teams (helper index hid of nhelp) one depth ahead
        const int nlive = a.nshot - g * S;  // live slots of the group (CTA-uniform)
        const bool helped = !PSPI && !TC && nlive < S;
        const int nhelp = 2 * (S - nlive) * T;
        const int hid = ((is_src ? 0 : S - nlive) + (sg - nlive)) * T + t;
        if constexpr (!PSPI && !TC) {
            if (helped) {
                if (!tables_free) __syncthreads();
                build_tables<N, PSPI, INTERP, BLU, TC>(a, sm, w, w2, 0, tid, NT);
                __syncthreads();
            }
        }

        // initial rows (wem.c:230-233): source spike at igx, receiver spectra
        float2 v[16];
        const int igx = shot_ok ? a.igx[shot] : -1;
        const float2 sw = a.srcw[iwi];
        const float2 *rrow = a.recv + ((size_t)(shot_ok ? shot : 0) * (a.recv_nwf ? a.recv_nwf : a.nwf) + iwi) * nmx;
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const int x = t + T * m;
            float2 u = make_float2(0.f, 0.f);
            if (x < nmx && shot_ok) u = is_src ? (x == igx ? sw : u) : rrow[x];
            v[m] = u;
        }

        for (int iz = 0; iz < a.nz; iz++) {
            const uint8_t zf = a.zflag[iz];
            // split-step: a slot of a part-filled shot group has zero rows and its team skips
            // the arithmetic (a one-shot survey leaves most slots empty; the PSPI forms keep
            // the registers of the full-group code)
            const bool active = (PSPI || shot_ok) && (is_src ? (zf & Z_SRC) : (zf & Z_REC));
            if (zf & Z_REC) {
                // the CTA's image row of this depth to L2 now; it is read and rewritten at the
                // end of the step
                const float2 *srow = slot + (size_t)iz * nmx;
                for (int x = tid * 16; x < nmx; x += NT * 16) asm volatile("prefetch.global.L2 [%0];" ::"l"(srow + x));
            }
            if (PSPI && a.ptab) {
                // precomputed tables: copied while the rows go through their forward
                // transforms (the barrier first: the previous depth's tables and exchange
                // buffers are no longer read); the depth's reference masks are loaded before
                // the barrier, which hides their latency
                const unsigned long long um = ref_mask(a, iz), cm = PAIR ? cx_mask(a, iz) : 0ull;
                const unsigned long long cu = GT ? 0ull : um;  // the phase tables copied (GT: none)
                __syncthreads();
                if constexpr (PSPI) {
                    if (tma) {
                        if (tid == 0 && !s_tabort) copy_tables_bulk<N, INTERP, PAIR>(a, sm, iwi, iz, cu, smem_u32(&s_tbar));
                    } else {
                        copy_tables_async<N, INTERP, PAIR>(a, sm, iwi, iz, tid, NT, cu);
                    }
                    float inv_s = 1.f;
                    if (active) {
                        if constexpr (PAIR) {
                            paired_forward<N>(v, xbuf, sacc, sm.tw, t, sync);
                        } else if constexpr (TC) {
                            // split16: the row enters the transform scaled by a power of two
                            float sc;
                            row_scale<T>(v, tc.red, t, sync, sc, inv_s);
#pragma unroll
                            for (int m = 0; m < 16; m++) v[m] = cscale(v[m], sc);
                            fft_row<N, -1, TC>(v, xbuf, sm.tw, t, sync, &tc);
                        } else {
                            xform<N, -1, false, BLU>(v, xbuf, sm.tw, t, sync, nullptr, a);
                        }
                    }
                    if (tma) tables_bulk_wait(smem_u32(&s_tbar), tphase, &s_tabort, a.err);
                    else cp_async_wait_all();
                    __syncthreads();
                    if (active) {
                        if constexpr (PAIR) {
                            paired_inverse<N>(v, is_src, a, sm, xbuf, sacc, t, sync, um, cm);
                        } else if constexpr (GT) {
                            Smem<N, PSPI, BLU> smg = sm;  // the depth's tables where they lie in device memory
                            smg.ph = const_cast<float2 *>(a.ptab) + ((size_t)iwi * a.nz + iz) * a.nref * SH::PHS;
                            step_mig_tail<N, PSPI, INTERP, TC>(v, is_src, a, smg, xbuf, sacc, t, sync, &tc, um, inv_s);
                        } else {
                            step_mig_tail<N, PSPI, INTERP, TC>(v, is_src, a, sm, xbuf, sacc, t, sync, &tc, um, inv_s);
                        }
                    }
                }
            } else if (!PSPI && !TC && helped) {
                if constexpr (!PSPI && !TC) {
                    // this depth's tables are complete (built one depth ahead), the previous
                    // depth's set and every exchange buffer are free (the image sum of the
                    // previous depth reads the receivers' buffers)
                    __syncthreads();
                    const Smem<N, PSPI, BLU> &cur = (iz & 1) ? sm1 : sm;
                    if (!shot_ok && iz + 1 < a.nz)
                        build_tables<N, PSPI, INTERP, BLU, TC>(a, (iz & 1) ? sm : sm1, w, w2, iz + 1, hid, nhelp);
                    if (active) step_mig<N, PSPI, INTERP, TC>(v, is_src, a, cur, xbuf, sacc, t, sync, &tc, ref_mask(a, iz));
                }
            } else {
                if (!tables_free) __syncthreads();
                build_tables<N, PSPI, INTERP, BLU, TC>(a, sm, w, w2, iz, tid, NT);
                if constexpr (PAIR)
                    if (tid < WPOS_STRIDE) sm.wpos[tid] = a.wpos ? a.wpos[(size_t)iz * WPOS_STRIDE + tid] : 0;
                __syncthreads();
                if (active) {
                    if constexpr (PAIR)
                        step_mig_paired<N>(v, is_src, a, sm, xbuf, sacc, t, sync, ref_mask(a, iz), cx_mask(a, iz));
                    else
                        step_mig<N, PSPI, INTERP, TC>(v, is_src, a, sm, xbuf, sacc, t, sync, &tc, ref_mask(a, iz));
                }
            }

            // ---- imaging condition (wem.c:243-247), summed over the group's shots
            if (zf & Z_REC) {
                // this thread's first two accumulator entries (x = tid, tid + NT), loaded now so
                // that their latency passes behind the two barriers below; only this thread
                // touches them
                float2 *srow = slot + (size_t)iz * nmx;
                const float2 acc0 = tid < nmx ? srow[tid] : make_float2(0.f, 0.f);
                const float2 acc1 = tid + NT < nmx ? srow[tid + NT] : make_float2(0.f, 0.f);
                if (is_src) {
#pragma unroll
                    for (int m = 0; m < 16; m++) {
                        const int x = t + T * m;
                        if (x < nmx) xbuf[x] = v[m];
                    }
                }
                __syncthreads();  // every step done: the tables are free from here on
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
                for (int x = tid, k = 0; x < nmx; x += NT, k++) {
                    float c = 0.f;
#pragma unroll
                    for (int s_ = 0; s_ < S; s_++) c += reinterpret_cast<const float *>(sm.x + (size_t)(S + s_) * PADN)[x];
                    kahan_add(&srow[x], c, k == 0 ? acc0 : (k == 1 ? acc1 : srow[x]));
                }
                tables_free = true;
            } else {
                tables_free = false;
            }
        }
    }
    if (tma && s_tabort && tid == 0) mbar_wait_bounded(smem_u32(&s_tbar), tphase ^ 1u);  // copies still in flight
    if constexpr (TC) {
        // every MMA was waited for, unless a wait ran out: then drain before freeing TMEM
        if (t == 0 && *tc.abort) {
            tc_commit(tc.mbar);
            mbar_wait_bounded(tc.mbar, tc.phase);
        }
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid < 32) tmem_dealloc(*tslot, TCOLS);
    }
}

// ------------------------------------------------------------------ modelling (Born)
// One team per shot. Per (group of S shots, frequency): the source wavefield is
// continued down and kept at every depth in global scratch (smig, wem.c:253-265),
// then the receiver wavefield is continued up from the bottom with the image
// injected at each depth (wem.c:266-276); the surface row, divided by
// sqrt(ntfft) (wem.c:277-279), is the shot's spectrum at this frequency.
// Rows of up to 1024 samples: two CTAs per SM (their shared memory fits twice), so the
// registers are capped at 128 per thread.
template <int N, bool PSPI, int INTERP, int S, bool EXACT, bool BLU = false>
__global__ void __launch_bounds__(S * (N / 16), N <= 1024 ? 2 : 1) wem_model_kernel(const MigArgs a, const BornArgs b)
{
    using SH = MigShape<N>;
    constexpr int T = SH::T, PADN = SH::PADN;
    constexpr int NT = S * T;
    extern __shared__ float4 smem_raw[];
    const Smem<N, PSPI, BLU> sm(smem_raw, a.nref, a.nmx, S);
    const int tid = threadIdx.x;
    const int team = tid / T, t = tid - team * T;
    float2 *xbuf = sm.x + (size_t)team * PADN;
    float2 *sacc = sm.acc + (size_t)team * sm.acc_stride;
    const unsigned sync = team_sync_handle<N>(tid);
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
            const bool act = (PSPI || shot_ok) && (a.zflag[iz] & Z_SRC) != 0;  // split-step: empty slots skip
            __syncthreads();
            if (PSPI && a.ptab) {
                // precomputed tables, copied behind the forward transform
                if constexpr (PSPI) {
                    copy_tables_async<N, INTERP, false>(a, sm, iwi, iz, tid, NT);
                    if (act) xform<N, -1, false, BLU>(v, xbuf, sm.tw, t, sync, nullptr, a);
                    cp_async_wait_all();
                    __syncthreads();
                    if (act) step_mig_tail<N, PSPI, INTERP>(v, true, a, sm, xbuf, sacc, t, sync, nullptr, ref_mask(a, iz), 1.f);
                }
            } else {
                build_tables<N, PSPI, INTERP>(a, sm, w, w2, iz, tid, NT);
                __syncthreads();
                if (act) step_mig<N, PSPI, INTERP>(v, true, a, sm, xbuf, sacc, t, sync, nullptr, ref_mask(a, iz));
            }
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
        // injection of m * smig at depth iz (wem.c:270-272): registers and global memory only
        auto inject = [&](int iz) {
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
        };
        for (int iz = nz - 1; iz >= 0; iz--) {
            const bool rec = (PSPI || shot_ok) && (a.zflag[iz] & Z_REC) != 0;
            if (iz > 0 && 8 * t < nmx) {
                // the next depth's source and image rows to L2 (64 bytes of each per thread)
                asm volatile("prefetch.global.L2 [%0];" ::"l"(smig + (size_t)(iz - 1) * nmx + 8 * t));
                if (16 * t < nmx) asm volatile("prefetch.global.L2 [%0];" ::"l"(b.img + (size_t)(iz - 1) * nmx + 16 * t));
            }
            __syncthreads();
            if (PSPI && a.ptab) {
                if constexpr (PSPI) {
                    // the tables copied while this depth's injection loads its rows
                    copy_tables_async<N, INTERP, false>(a, sm, iwi, iz, tid, NT);
                    if (rec) inject(iz);
                    cp_async_wait_all();
                }
            } else {
                build_tables<N, PSPI, INTERP>(a, sm, w, w2, iz, tid, NT);
            }
            __syncthreads();
            if (rec) {
                if (!(PSPI && a.ptab)) inject(iz);
                step_model<N, PSPI, INTERP, EXACT, BLU>(v, a, sm, xbuf, sacc, t, sync, ref_mask(a, iz));
            }
        }
        if (shot_ok) {
            float2 *out = b.dg + ((size_t)shot * (a.recv_nwf ? a.recv_nwf : a.nwf) + iwi) * nmx;
#pragma unroll
            for (int m = 0; m < 16; m++) {
                const int x = t + T * m;
                if (x < nmx) out[x] = make_float2(v[m].x * b.inv_sqt, v[m].y * b.inv_sqt);
            }
        }
    }
}

// ------------------------------------------------------------------ per-N launch helpers
// Two CTA shapes per row length: "wide" (512 threads, 2S rows sharing one set of phase
// tables) and "narrow" (256 threads); wide is used whenever its shared memory fits.
template <int N> struct Shapes {
    static constexpr int T = N / 16;
    static constexpr int S_WIDE = (2 * T >= 512) ? 1 : (512 / (2 * T) > 16 ? 16 : 512 / (2 * T));
    static constexpr int S_NARROW = (2 * T >= 256) ? 1 : (256 / (2 * T) > 16 ? 16 : 256 / (2 * T));
    // modelling: one team per shot, 256 threads
    static constexpr int S_MODEL = (T >= 256) ? 1 : (256 / T > 16 ? 16 : 256 / T);
};

template <int N, bool PSPI, int INTERP, int S, bool TC, bool PAIR = false, bool BLU = false, bool GT = false>
int mig_run(const MigArgs *a, int grid, size_t smem, cudaStream_t st, int *bps)
{
    auto k = wem_migrate_kernel<N, PSPI, INTERP, S, TC, PAIR, BLU, GT>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return -1;
    if (bps) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, k, 2 * S * (N / 16), smem) == cudaSuccess ? 0 : -1;
    k<<<grid, 2 * S * (N / 16), smem, st>>>(*a);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <int N, int S, bool TC, bool BLU = false>
int mig_sel(int pspi, int interp, const MigArgs *a, int grid, size_t smem, cudaStream_t st, int *bps)
{
    if (!pspi) return mig_run<N, false, 0, S, TC, false, BLU>(a, grid, smem, st, bps);
    if (interp == 0) return mig_run<N, true, 0, S, TC, false, BLU>(a, grid, smem, st, bps);
    return mig_run<N, true, 1, S, TC, false, BLU>(a, grid, smem, st, bps);
}

// wide = 1 selects the 512-thread shape. form: MIG_FORM_FP32; MIG_FORM_SPLIT16, the
// tensor-core form, built for N = 2048 only (-2 otherwise); MIG_FORM_PAIRED, the paired
// inverse transforms of the PSPI nearest-lower mode (-2 for other modes); MIG_FORM_BLU,
// transforms of a length that is not a power of two on N-sample rows (wide shape only).
// Fills *S/*threads/*smem; launches when a != nullptr and bps == nullptr, queries
// occupancy when bps != nullptr.
template <int N>
int mig_launch(int wide, int pspi, int interp, int nref, int nmx, const MigArgs *a, int grid, cudaStream_t st,
               int *S, int *threads, size_t *smem, int *bps, int form)
{
    using SH = Shapes<N>;
    const int s_ = wide ? SH::S_WIDE : SH::S_NARROW;
    const int tc = form == MIG_FORM_SPLIT16;
    *S = s_;
    *threads = 2 * s_ * SH::T;
    *smem = mig_smem_bytes<N>(pspi != 0, nref, nmx, 2 * s_, tc != 0, form == MIG_FORM_PAIRED, form == MIG_FORM_BLU);
    if (!pspi && !tc)  // split-step: the second set of depth tables (wem_migrate_kernel)
        *smem += sizeof(float2) * ((size_t)(form == MIG_FORM_BLU ? ph_entries<N, true>(false, nref) : ph_entries<N>(false, nref)) +
                                   (size_t)((nmx + 1) & ~1));
    if (form == MIG_FORM_BLU) {
        if (!wide) return -2;
        if (!a && !bps) return 0;
        return mig_sel<N, SH::S_WIDE, false, true>(pspi, interp, a, grid, *smem, st, bps);
    }
    if (form == MIG_FORM_GT) {
        if constexpr (N >= 1024) {
            if (!pspi) return -2;
            *smem = mig_smem_bytes<N>(true, 0, nmx, 2 * s_);  // no phase tables in shared memory
            if (!a && !bps) return 0;
            if (interp == 0) {
                if (wide) return mig_run<N, true, 0, SH::S_WIDE, false, false, false, true>(a, grid, *smem, st, bps);
                return mig_run<N, true, 0, SH::S_NARROW, false, false, false, true>(a, grid, *smem, st, bps);
            }
            if (wide) return mig_run<N, true, 1, SH::S_WIDE, false, false, false, true>(a, grid, *smem, st, bps);
            return mig_run<N, true, 1, SH::S_NARROW, false, false, false, true>(a, grid, *smem, st, bps);
        } else {
            return -2;
        }
    }
    if (form == MIG_FORM_PAIRED) {
        if (!pspi || interp != 0) return -2;
        if (!a && !bps) return 0;
        if (wide) return mig_run<N, true, 0, SH::S_WIDE, false, true>(a, grid, *smem, st, bps);
        return mig_run<N, true, 0, SH::S_NARROW, false, true>(a, grid, *smem, st, bps);
    }
    if (tc) {
        if constexpr (N == 2048) {
            if (!a && !bps) return 0;
            if (wide) return mig_sel<N, SH::S_WIDE, true>(pspi, interp, a, grid, *smem, st, bps);
            return mig_sel<N, SH::S_NARROW, true>(pspi, interp, a, grid, *smem, st, bps);
        } else {
            return -2;
        }
    }
    if (!a && !bps) return 0;
    if (wide) return mig_sel<N, SH::S_WIDE, false>(pspi, interp, a, grid, *smem, st, bps);
    return mig_sel<N, SH::S_NARROW, false>(pspi, interp, a, grid, *smem, st, bps);
}

template <int N, bool PSPI, int INTERP, bool EXACT, bool BLU = false>
int model_run(const MigArgs *a, const BornArgs *b, int grid, size_t smem, cudaStream_t st, int *bps)
{
    constexpr int S = Shapes<N>::S_MODEL;
    auto k = wem_model_kernel<N, PSPI, INTERP, S, EXACT, BLU>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return -1;
    if (bps) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, k, S * (N / 16), smem) == cudaSuccess ? 0 : -1;
    k<<<grid, S * (N / 16), smem, st>>>(*a, *b);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <int N, bool BLU>
int model_sel(int pspi, int interp, int exact, const MigArgs *a, const BornArgs *b, int grid, size_t smem,
              cudaStream_t st, int *bps)
{
    if (!pspi) return model_run<N, false, 0, false, BLU>(a, b, grid, smem, st, bps);
    if (exact) {
        if (interp == 0) return model_run<N, true, 0, true, BLU>(a, b, grid, smem, st, bps);
        return model_run<N, true, 1, true, BLU>(a, b, grid, smem, st, bps);
    }
    if (interp == 0) return model_run<N, true, 0, false, BLU>(a, b, grid, smem, st, bps);
    return model_run<N, true, 1, false, BLU>(a, b, grid, smem, st, bps);
}

// blu = 1: transforms of a length that is not a power of two on N-sample rows
template <int N>
int model_launch(int pspi, int interp, int exact, int nref, int nmx, const MigArgs *a, const BornArgs *b, int grid,
                 cudaStream_t st, int *S, int *threads, size_t *smem, int *bps, int blu)
{
    using SH = Shapes<N>;
    *S = SH::S_MODEL;
    *threads = SH::S_MODEL * SH::T;
    *smem = mig_smem_bytes<N>(pspi != 0, nref, nmx, SH::S_MODEL, false, false, blu != 0);
    if (!a && !bps) return 0;
    if (blu) return model_sel<N, true>(pspi, interp, exact, a, b, grid, *smem, st, bps);
    return model_sel<N, false>(pspi, interp, exact, a, b, grid, *smem, st, bps);
}

// defined in wem_n<N>.cu
#define WEM_DECLARE_N(N)                                                                                          \
    extern template int mig_launch<N>(int, int, int, int, int, const MigArgs *, int, cudaStream_t, int *, int *, \
                                      size_t *, int *, int);                                                      \
    extern template int model_launch<N>(int, int, int, int, int, const MigArgs *, const BornArgs *, int,         \
                                        cudaStream_t, int *, int *, size_t *, int *, int);
WEM_DECLARE_N(32)
WEM_DECLARE_N(64)
WEM_DECLARE_N(128)
WEM_DECLARE_N(256)
WEM_DECLARE_N(512)
WEM_DECLARE_N(1024)
WEM_DECLARE_N(2048)
WEM_DECLARE_N(4096)
#undef WEM_DECLARE_N

}  // namespace gbwem
