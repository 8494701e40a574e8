// wem_tc.cuh -- the DFT stages of the row FFT on the tensor cores (tcgen05), with
// split-FP16 operands and FP32 accumulation ("split16" precision mode).
//
// A team of 128 threads (one warpgroup) holds a row of N = 2048 samples; in each
// Stockham pass of wem_fft.cuh thread t owns butterfly group t: 16 complex values
// (radix 16) or two groups of 8 (the radix-8 pass). The DFT of all 128 groups of a
// team is one matrix product per group slot
//
//     D[128 x 2R] = A[128 x 2R] * W[2R x 2R]     (real form, (re, im) interleaved)
//
// with row t of A the values of thread t and W the real form of the complex DFT
// matrix (W[2r][2q] = W[2r+1][2q+1] = c, W[2r+1][2q] = -s, W[2r][2q+1] = s for
// c + i s = e^{DIR 2 pi i r q / R}). Every FP32 operand x is split into
// hi = fp16(x) and lo = fp16(x - hi), and so is W (built in FP64 on the host), and
// D = A_hi W_hi + A_lo W_hi + A_hi W_lo accumulates in FP32 in tensor memory; the
// dropped A_lo W_lo term is below 2^-22 of the result. Thread t writes its row of
// A_hi and A_lo to shared memory (the team's exchange buffer, free at that point of
// the pass), one thread issues the tcgen05.mma instructions and commits them to the
// team's mbarrier, and after the wait thread t reads row t of D back with
// tcgen05.ld: accumulator row t lives in TMEM lane t, which belongs to warp t/32 of
// the warpgroup.
//
// Range: fp16 holds |x| <= 65504. Rows enter the forward transform scaled by a power
// of two so that every |re|, |im| < 2^7; a radix-16 pass grows the bound 16x, so all
// pass inputs stay below 2^15, and the inverse transforms start from spectra times
// phase / N (bounded by the same 2^7). The caller undoes the scale exactly.
//
// Shared operand layout (no swizzle, K-major, the canonical tcgen05 layout): core
// matrices of 8 rows x 16 bytes (8 fp16 along K) stored as 128 contiguous bytes;
// core matrices adjacent along K are 128 B apart (leading byte offset) and groups
// of 8 rows are 16*K bytes apart (stride byte offset, K in fp16 elements).
//
// The issuing thread alone waits on the mbarrier, the rest of the team at a named
// barrier behind it. Every mbarrier wait is bounded (about a second of clock cycles); a
// wait that runs out sets the CTA's abort flag and the launch's error word, after which
// the CTA issues no more tensor-core work and waits no more, so it runs to its end
// (results are garbage, the host reports WEM_ERR_TIMEOUT).
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "wem_fft.cuh"

namespace gbwem {

// bytes of the W operands in shared memory: W16 fwd hi/lo, inv hi/lo (2048 B each),
// then W8 fwd hi/lo, inv hi/lo (512 B each)
constexpr int TC_W_BYTES = 4 * 2048 + 4 * 512;
constexpr int TC_W8_OFF = 4 * 2048;
// bytes of a team's A operands (they alias its exchange buffer)
constexpr int TC_A_BYTES = 16384;
constexpr long long TC_WAIT_CYCLES = 2000000000LL;  // ~1 s at 2 GHz

struct TcTeam {
    float *red;      // 4 floats of reduction scratch of the team (row_scale)
    uint32_t a;      // shared address of the team's A operands (its exchange buffer)
    uint32_t w;      // shared address of the W operands
    uint32_t d;      // TMEM address of the team's accumulator columns (lane 0)
    uint32_t dw;     // TMEM address of this warp's lane quarter of them
    uint32_t mbar;   // shared address of the team's mbarrier
    uint32_t phase;  // parity of the next completion to wait for
    volatile int *abort;  // CTA-wide: set once any wait ran out
    int *err;             // launch-wide error word (global)
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: no swizzle, base offset 0, version 1 (bit 46)
__device__ __forceinline__ uint64_t tc_sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);
}

// instruction descriptor of kind::f16: A, B fp16 (K-major), D fp32, M = 128, N = NCOL
template <int NCOL> __device__ __forceinline__ constexpr uint32_t tc_idesc()
{
    return (1u << 4) | ((uint32_t)(NCOL >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d_tmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void tc_commit(uint32_t mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ bool mbar_try_wait(uint32_t mbar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(mbar), "r"(parity)
        : "memory");
    return ok != 0;
}

// bounded wait for the phase of the given parity; false when it ran out
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t mbar, uint32_t parity)
{
    const long long t0 = clock64();
    while (!mbar_try_wait(mbar, parity))
        if (clock64() - t0 > TC_WAIT_CYCLES) return false;
    return true;
}

// TMEM allocation by one whole warp; the base address lands in *slot
__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// 32 consecutive accumulator columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&r)[32])
{
    uint32_t q[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(q[0]), "=r"(q[1]), "=r"(q[2]), "=r"(q[3]), "=r"(q[4]), "=r"(q[5]), "=r"(q[6]), "=r"(q[7]), "=r"(q[8]),
          "=r"(q[9]), "=r"(q[10]), "=r"(q[11]), "=r"(q[12]), "=r"(q[13]), "=r"(q[14]), "=r"(q[15]), "=r"(q[16]),
          "=r"(q[17]), "=r"(q[18]), "=r"(q[19]), "=r"(q[20]), "=r"(q[21]), "=r"(q[22]), "=r"(q[23]), "=r"(q[24]),
          "=r"(q[25]), "=r"(q[26]), "=r"(q[27]), "=r"(q[28]), "=r"(q[29]), "=r"(q[30]), "=r"(q[31])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) r[i] = __uint_as_float(q[i]);
}

// hi/lo fp16 pair of a complex value, as two packed half2 words
__device__ __forceinline__ void split_c(float2 v, uint32_t &hi, uint32_t &lo)
{
    const __half2 h = __floats2half2_rn(v.x, v.y);
    const float2 hf = __half22float2(h);
    const __half2 l = __floats2half2_rn(v.x - hf.x, v.y - hf.y);
    hi = *reinterpret_cast<const uint32_t *>(&h);
    lo = *reinterpret_cast<const uint32_t *>(&l);
}

// Store group values u[0..C-1] (C = 8 or 16 complex) as row t of an A operand pair
// (hi at a, lo at a + 128*4*C bytes), K = 2C fp16 per row.
template <int C> __device__ __forceinline__ void tc_store_row(const float2 *u, char *a_gen, int t)
{
    constexpr int ROWB = 4 * C;        // bytes of one row (2C fp16)
    constexpr int TILE = 128 * ROWB;   // bytes of one 128-row operand
    constexpr int GSTR = 8 * ROWB;     // stride byte offset: 8 rows
    char *rowbase = a_gen + (t >> 3) * GSTR + (t & 7) * 16;
#pragma unroll
    for (int c = 0; c < C / 4; c++) {
        uint32_t h[4], l[4];
#pragma unroll
        for (int j = 0; j < 4; j++) split_c(u[4 * c + j], h[j], l[j]);
        *reinterpret_cast<uint4 *>(rowbase + c * 128) = make_uint4(h[0], h[1], h[2], h[3]);
        *reinterpret_cast<uint4 *>(rowbase + TILE + c * 128) = make_uint4(l[0], l[1], l[2], l[3]);
    }
}

// One DFT stage of radix R (16, or 8 with two groups per thread) on the team's rows.
// u[16]: in and out, natural order within each group (as dft<R, DIR> in wem_fft.cuh).
template <int R, int DIR, int T>
__device__ __forceinline__ void tc_dft(float2 (&u)[16], TcTeam &tc, char *a_gen, int t, unsigned bar_id)
{
    // thread t stores row t; the A operand pair(s) fill 16 KB of the exchange buffer
    static_assert(T == 128, "the tensor-core stage needs teams of one warpgroup");
    static_assert(R == 16 || R == 8, "radix 16 or 8");
    if constexpr (R == 16) {
        tc_store_row<16>(u, a_gen, t);
    } else {
        tc_store_row<8>(u, a_gen, t);
        tc_store_row<8>(u + 8, a_gen + 8192, t);
    }
    fence_async_smem();  // the generic-proxy stores become visible to the tensor core
    team_sync<T>(bar_id);
    const bool live = *tc.abort == 0;
    if (t == 0 && live) {
        tc_fence_after();
        const int dsel = DIR < 0 ? 0 : 2;
        if constexpr (R == 16) {
            const uint32_t ahi = tc.a, alo = tc.a + 8192;
            const uint32_t whi = tc.w + dsel * 2048, wlo = whi + 2048;
            constexpr uint32_t id = tc_idesc<32>();
#pragma unroll
            for (int k = 0; k < 2; k++)
                tc_mma(tc.d, tc_sdesc(ahi + k * 256, 128, 512), tc_sdesc(whi + k * 256, 128, 512), id, k);
#pragma unroll
            for (int k = 0; k < 2; k++)
                tc_mma(tc.d, tc_sdesc(alo + k * 256, 128, 512), tc_sdesc(whi + k * 256, 128, 512), id, 1);
#pragma unroll
            for (int k = 0; k < 2; k++)
                tc_mma(tc.d, tc_sdesc(ahi + k * 256, 128, 512), tc_sdesc(wlo + k * 256, 128, 512), id, 1);
        } else {
            const uint32_t whi = tc.w + TC_W8_OFF + dsel * 512, wlo = whi + 512;
            constexpr uint32_t id = tc_idesc<16>();
#pragma unroll
            for (int b = 0; b < 2; b++) {
                const uint32_t ahi = tc.a + b * 8192, alo = ahi + 4096, d = tc.d + 16 * b;
                tc_mma(d, tc_sdesc(ahi, 128, 256), tc_sdesc(whi, 128, 256), id, 0);
                tc_mma(d, tc_sdesc(alo, 128, 256), tc_sdesc(whi, 128, 256), id, 1);
                tc_mma(d, tc_sdesc(ahi, 128, 256), tc_sdesc(wlo, 128, 256), id, 1);
            }
        }
        tc_commit(tc.mbar);
        // the issuing thread alone polls the mbarrier; the team waits at the barrier below
        if (!mbar_wait_bounded(tc.mbar, tc.phase)) {
            *tc.abort = 1;
            atomicExch(tc.err, 1);
        }
    }
    tc.phase ^= 1u;
    team_sync<T>(bar_id);  // the team's MMAs have completed
    tc_fence_after();
    float r[32];
    tmem_ld32(tc.dw, r);
#pragma unroll
    for (int j = 0; j < 16; j++) u[j] = make_float2(r[2 * j], r[2 * j + 1]);
    tc_fence_before();  // the reads are ordered before the team barrier that precedes the next MMA
}

// Power-of-two scale that brings the team's row below 2^7 in every component
// (1 for a zero row), and its inverse. red: 4 floats of scratch per team.
template <int T>
__device__ __forceinline__ void row_scale(const float2 (&v)[16], float *red, int t, unsigned bar_id, float &s,
                                          float &inv_s)
{
    float m = 0.f;
#pragma unroll
    for (int i = 0; i < 16; i++) m = fmaxf(m, fmaxf(fabsf(v[i].x), fabsf(v[i].y)));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((t & 31) == 0) red[t >> 5] = m;
    team_sync<T>(bar_id);
    m = fmaxf(fmaxf(red[0], red[1]), fmaxf(red[2], red[3]));
    team_sync<T>(bar_id);  // red is reused by the next call
    // 2^k > m >= 2^(k-1) for normal m: k = unbiased exponent + 1
    const int k = m > 0.f ? (int)((__float_as_uint(m) >> 23) & 0xffu) - 126 : 0;
    int e = 7 - k;
    e = e < -126 ? -126 : (e > 126 ? 126 : e);
    s = __uint_as_float((uint32_t)(127 + e) << 23);
    inv_s = __uint_as_float((uint32_t)(127 - e) << 23);
}

}  // namespace gbwem
