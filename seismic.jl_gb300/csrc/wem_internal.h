// wem_internal.h -- structures shared by the host runtime (wem_api.cu) and the
// kernels (wem_kernels.cu). Not part of the public ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gbwem {

// Per-depth selection byte of the PSPI interpolation, one per (iz, ix): bits 0-6
// iref1, bit 7 set when vref2 - vref1 > 10 (wem.c:454: interpolate between iref1
// and iref2 = iref1 + 1; otherwise the nearest-lower wavefield is taken whole).
constexpr uint8_t SEL_INTERP = 0x80;

// Per-depth activity flags (wem.c:235-242): source continued when z >= sz,
// receiver continued and image formed when z >= gz.
constexpr uint8_t Z_SRC = 1, Z_REC = 2;

struct MigArgs {
    int nmx;        // live samples per row (grid cells along x)
    int nz;
    int nref;       // PSPI reference velocities (1 for split-step)
    int nwf;        // frequencies in the band [ifmin, ifmax)
    int ifmin;
    int nshot;
    int ngroups;    // ceil(nshot / shots per CTA)
    float dw;       // angular frequency step (float, wem.c:85)
    float dz;
    float dkx;      // wavenumber step (float, wem.c:83)
    float inv_n;    // 1/nkx, folds the two 1/sqrt(nkx) of wem.c:437,445
    const float2 *recv;    // [nshot][nwf][nmx] receiver spectra, w^2/sqrt(ntfft) applied
    const float2 *srcw;    // [nwf] wavelet spectrum / sqrt(ntfft)
    const int *igx;        // [nshot] source cell
    const float *vref;     // [nz][nref]
    const float *slow2;    // [nz][nref] 1/(vref*vref) in float (wem.c:434)
    const float *po;       // [nz] mean slowness
    const float *pd;       // [nz][nmx] slowness perturbation
    const uint8_t *selb;   // [nz][nmx] selection bytes
    const float *wlin;     // [nz][nmx] linear-interpolation weight of iref2
    const float *taper;    // [nmx] boundary taper (split-step)
    const uint8_t *zflag;  // [nz]
    const float2 *twid;    // FFT twiddle table of the row length
    float2 *slots;         // [gridDim.x][nz][nmx] (sum, compensation) image accumulators
    const uint4 *tcw;      // split16 mode: the W operands of the tensor-core DFT stages (10240 B)
    int *err;              // split16 mode: set when a tensor-core wait ran out
    const unsigned long long *refmask;  // [nz] references in use at each depth (nullptr: all)
    const unsigned long long *cxmask;   // [nz] references some point takes whole (nullptr: all)
    // paired form: per depth the count (0 .. WHOLE_MAX) and positions of the points that take
    // their wavefield whole when they are that few ([nz][WPOS_STRIDE]; nullptr: none)
    const int *wpos;
    const float2 *wdot;    // paired form: e^{+2 pi i e / nkx}, e = 0 .. nkx/2
    // paired form: the phase tables of every (frequency, depth), [nwf][nz][nref][nkx/2 + 2]
    // (nullptr: each CTA builds its own), and the selection rows padded to 16 bytes
    const float2 *ptab;
    const uint8_t *selbp;  // [nz][(nmx + 15) / 16 * 16]
    const float *wlinp;    // [nz][(nmx + 3) / 4 * 4] linear weights, rows padded to 16 bytes
    // rows whose transform length nkx is not a power of two (Bluestein's chirp form): the
    // transform length L = nkx (the kernels' row length N is a power of two >= 2L - 1), the
    // chirp b[n] = e^{i pi n^2 / L} (n < L) and G/N, G the N-point FFT of b placed at n and
    // N - n (see xform in wem_step.cuh)
    int nlog;
    const float2 *chirp;
    const float2 *bfft;
    // split16 PSPI: phase tables built in FP64 -- the reference velocities in double
    // ([nz][nref], vmin + r (vmax - vmin)/(nref - 1) from the float extremes) and the
    // wavenumber step 2 pi / (nkx dmx) in double
    const double *vref64;
    double dkx64;
    // 1: the precomputed tables reach shared memory by bulk copies (TMA engine) completing on
    // an mbarrier; 0: per-thread 16-byte cp.async
    int tma;
    // frequencies between the rows of one shot in recv (migration) and dg (modelling) when a
    // launch covers a band [ifmin, ifmin + nwf) of a longer spectrum; 0: nwf
    int recv_nwf;
};
// points per depth whose imaginary part the paired form takes from a direct sum
constexpr int WHOLE_MAX = 4;
constexpr int WPOS_STRIDE = 8;  // ints per depth in wpos (count, positions, padding to 32 bytes)

struct SpectraArgs {
    const float *d;        // [ntr][ld] (ld = 0: nt)
    int ntr, nt, ntfft;    // nt: samples transformed, at most ntfft (f_op's r2c reads ntfft samples, wem.c:490-493)
    int ld;                // row stride of d in samples
    int ifmin, nwf;
    const int64_t *out_base;  // [ntr] element offset of (row, iwi = 0) in out
    int64_t out_fstride;      // element stride between consecutive frequencies
    const float2 *wtab;       // [ntfft] e^{-2 pi i k / ntfft}
    const float *scale;       // [nwf]
    float2 *out;
};

struct BornArgs {
    const float *img;   // [nz][nmx] image (depth-major)
    float2 *smig;       // [gridDim.x * shots per CTA][nz][nmx] source wavefield scratch
    float2 *dg;         // [nshot][nwf][nmx] modelled spectra (already / sqrt(ntfft))
    float inv_sqt;      // 1/sqrtf(ntfft)
};

struct SynthArgs {
    const float2 *dg;         // [nshot][nwf][nmx]
    int nwf, ifmin, nt, nf;   // nf: length of the real transform, (nw-1)*2 (wem.c:487)
    int ntr;
    const int64_t *in_base;   // [ntr] element offset of (shot, iwi = 0, cell) in dg
    int64_t in_fstride;       // nmx
    const float2 *wtab;       // [nf] e^{-2 pi i k / nf}
    const float *scale;       // [nwf] w^2 times the half-spectrum weight
    float *out;               // [ntr][nt]
};

// 3-D depth recursion (wem_3d.cu): state of every item (shot, frequency) in flight.
struct Mig3dArgs {
    int nmx, nmy, nkx, nky, nz, nref, nwf, ifmin, nitems, chunk, iz;
    float dw, dz, dkx, dky, inv_n;
    const float *vref, *slow2, *po, *pd, *wlin, *taper, *tapery;
    const uint8_t *selb, *zflag;
    const float2 *twx, *twy;
    const int *item_iwi, *item_shot, *src_cell;
    const float2 *srcw, *recv;
    float2 *U;          // [item][2][nmx][nmy]
    float2 *Y;          // [item][2][nmx][nky]
    float2 *C;          // [item][2][nref][nmx][nky]
    float2 *img_parts;  // [chunk][nz][nmx*nmy] (sum, 0)
    // modelling (wem.c:252-281): mode 1 continues the source down and keeps it in smig;
    // mode 2 continues the receiver up (-dz, adj=false) with m * smig injected first;
    // mode 4 continues it up with the exact adjoint of the migration step (PSPI);
    // mode 3 continues the source down as the angle computation does (ssop_source: the
    // split-step correction before the transform) and keeps it in smig
    int mode, pspi;     // mode 0: migration
    float2 *smig;       // [item][nz][nmx*nmy]
    const float *mimg;  // [nz][nmx*nmy] image, depth-major
    // PSPI nearest-lower mode: per depth the planes of pass B/C, [nz][PLAN3_STRIDE] = count,
    // then (r1, r2) per plane: the real parts of r1 and r2 in one plane, or r2 = -1 for a
    // reference of its own (nullptr: one plane per reference)
    const int *plan;
    // with a plan: per depth the count (<= WHOLE_MAX) and cells (x * nmy + y) of the points
    // that take their wavefield whole (their references are paired; the imaginary parts are
    // direct sums: pass B sums each column over kx into dsum, pass C sums over ky)
    const int *wpos;    // [nz][WPOS_STRIDE]
    float2 *dsum;       // [item][2][WHOLE_MAX][nky]
    // mode 4, the exact adjoint's receiver going up: the references in use per depth (bit r;
    // nullptr: all)
    const unsigned long long *refmask;
};
constexpr int PLAN3_MAX = 16, PLAN3_STRIDE = 1 + 2 * PLAN3_MAX;
int m3d_supported(int nkx, int nky);
int m3d_cols_block(int nkx);
int m3d_cols_smem(int nkx, int pspi, const Mig3dArgs &a, size_t *smem);
int m3d_launch_step(int nkx, int nky, int pspi, int interp, const Mig3dArgs &a, int nsm, cudaStream_t st);
int m3d_launch_init(const Mig3dArgs &a, cudaStream_t st);
// dg[(shot * nwf + iwi) * n + cell] = receiver plane of each item * scale
int m3d_launch_collect(const Mig3dArgs &a, float2 *dg, float scale, cudaStream_t st);

// host-side launchers (wem_kernels.cu). `wide` selects the 512-thread CTA shape of
// the migration kernel (2S rows sharing the phase tables) over the 256-thread one.
// source-side incidence angles (wem_angles.cu), 2-D
struct AngleArgs {
    int nmx, nz, nwf, ifmin, igx;
    int nshot;             // shots of the batch (blockIdx.y); igxs[s] their source cells (nullptr: igx)
    const int *igxs;
    float dw, dz, oz, sz, dkx, inv_sqrt_n;  // inv_sqrt_n = 1/sqrtf(nkx)
    const float *po;       // [nz] mean slowness
    const float *pd;       // [nz][nmx] slowness perturbation
    const float *taper;    // [nmx] boundary_condition weights
    const float2 *srcw;    // [nwf] source spectrum / sqrt(ntfft) over the band
    const float2 *twx;     // [nmx] e^{-2 pi i k / nmx}
    float2 *u;             // [shot][nwf][nz][nmx] source wavefield
};
struct AngleAccumArgs {
    int nmx, nz, nwf, nw, nfreq_div;
    const float2 *u, *ux, *uz, *ul, *ur;  // [nwf][nz][nmx]
    const float *uzp;                     // u_z in planes instead: [nwf][re, im][nz][nmx] (nullptr: uz)
    float *angx, *angy;                   // [nmx][nz]
};
// interleaved complex entries of `entry` samples -> [re plane, im plane] per entry
int launch_planar(const float2 *in, float *out, long long entry, long long nentries, cudaStream_t st);
// 3-D: running sums over batches of frequencies, one point per thread
struct AngleAccum3Args {
    int n, nz, nwf, nw, nfreq_div, last;  // n = nmx*nmy; last: write the angles after this batch
    const float2 *u, *ux, *uy, *uz, *lx, *rx, *ly, *ry;  // [nwf][nz][n]
    float *sum;                                          // [4][n][nz]: ang x, sign x, ang y, sign y
    float *angx, *angy;                                  // [n][nz]
};
int launch_angles_accum3(const AngleAccum3Args &a, cudaStream_t st);
struct AngleXArgs {
    long long nlines;                  // rows of nmx samples (frequency, depth)
    float dkx;
    const float2 *twx;                 // FFT twiddle table of the row length
    const float2 *u;                   // [nlines][nmx]
    float2 *ux, *ul, *ur;              // [nlines][nmx]
};
// Derivatives along one axis as circular convolutions on power-of-two rows (wem_angles.cu):
// nlines lines of L samples; cols == 1: contiguous lines ([line][L]); cols > 1: column c of
// plane p ([p][L][cols], nlines = planes * cols). H: nout transfer functions of the row
// length M = angles_conv_length(L) (G/M of the convolution kernel), out[o] like u.
struct AngleConvArgs {
    int L, cols, nout;
    long long nlines;
    const float2 *tw;   // FFT twiddle table of M
    const float2 *H;    // [nout][M]
    const float2 *u;
    float2 *out[3];
};
// M for an axis of L samples: the power of two >= max(32, 2L - 1); 0 above L = 2048
int angles_conv_length(int L);
int launch_angles_conv(const AngleConvArgs &a, int nsm, cudaStream_t st);
int launch_angles_extrap(const AngleArgs &a, cudaStream_t st);
// power-of-two nmx in [32, 2048]: which = 0 extrapolation, 1 x derivatives on the row FFT
bool angles_fft_supported(int nmx);
int launch_angles_fft(const AngleArgs &a, const AngleXArgs &x, int which, cudaStream_t st);
int launch_angles_accum(const AngleAccumArgs &a, cudaStream_t st);

// Forms of the 2-D depth kernel: FP32; split16 (tensor-core DFT stages, nkx = 2048 only);
// paired (FP32, PSPI nearest-lower mode: two references' real parts per inverse transform);
// Bluestein (FP32, transform length nkx not a power of two, on rows of the power of two
// N >= 2 nkx - 1; the nkx argument of the dispatch functions below is that N).
// MIG_FORM_GT: PSPI FP32 with the phase tables read from device memory (nkx >= 1024), for
// reference counts whose tables do not fit in shared memory
constexpr int MIG_FORM_FP32 = 0, MIG_FORM_SPLIT16 = 1, MIG_FORM_PAIRED = 2, MIG_FORM_BLU = 3, MIG_FORM_GT = 4;
int migrate_config(int nkx, int wide, int pspi, int interp, int nmx, int nref, int *shots_per_cta, int *threads,
                   size_t *smem, int form = MIG_FORM_FP32);
int migrate_max_grid(int nkx, int wide, int pspi, int interp, int nmx, int nref, int *blocks_per_sm,
                     int form = MIG_FORM_FP32);
int launch_migrate(int nkx, int wide, int pspi, int interp, const MigArgs &a, int grid, cudaStream_t st,
                   int form = MIG_FORM_FP32);
// one bounded mbarrier wait that nothing completes; *timed_out (device) = 1 when it gave up
int launch_wait_probe(int *timed_out, cudaStream_t st);
// FP32 FMA probe: grid CTAs of 512 threads, each thread 64 x iters FMAs
int launch_fma_probe(float *out, int iters, int grid, cudaStream_t st);
// the precomputed phase tables (a.ptab layout: `half` entries of every reference in use at a
// stride of `phs` float2) into out
int launch_phase_tables(int half, int phs, const MigArgs &a, float2 *out, cudaStream_t st, int f64 = 0);
// the 10240-byte W operand image of the split16 DFT stages
void tc_w_table_host(uint16_t *out);
// blu = 1: the Bluestein rows (MIG_FORM_BLU), nkx the row length N
int model_config(int nkx, int pspi, int nmx, int nref, int *shots_per_cta, int *threads, size_t *smem, int blu = 0);
int model_max_grid(int nkx, int pspi, int interp, int exact, int nmx, int nref, int *blocks_per_sm, int blu = 0);
int launch_model(int nkx, int pspi, int interp, int exact, const MigArgs &a, const BornArgs &b, int grid,
                 cudaStream_t st, int blu = 0);
int launch_spectra(const SpectraArgs &a, cudaStream_t st);
int launch_image_reduce(const float2 *slots, int nslots, int nz, int nmx, float *m, cudaStream_t st);
int launch_synth(const SynthArgs &a, cudaStream_t st);
int launch_transpose(const float *in, int rows, int cols, float *out, cudaStream_t st);
int twiddle_table_size(int nkx);
void twiddle_table_host(int nkx, float2 *out);

}  // namespace gbwem
