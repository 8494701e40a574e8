/*
 * shotwem_gb300.h -- C ABI of the GB300 shot-profile wave-equation migration library
 * (shotwem.so). Plain pointers and sizes only; every entry returns an int status.
 *
 * Drop-in entry points (same names and argument meaning as the reference's C core):
 *   main(argc, argv)   replaces src/Imaging/c/shotwem.c:12 (the symbol the Julia
 *                      wrapper binds: src/Imaging/ShotProfileWEM.jl:347
 *                      ccall((:main,"shotwem"), Int32, (Int32, Ptr{Ptr{UInt8}}), ...));
 *                      exported by the library, also available as shotwem_main.
 *   wem(...)           replaces src/Imaging/c/wem.h:3-11 / wem.c:3-204.
 * Batched entry points (no reference counterpart; they let one call migrate or
 * model every shot of a survey on one GPU instead of one process per shot,
 * src/Imaging/ShotProfileWEM.jl:104-106 and :288-290):
 *   wem_ctx_create / wem_prepare / wem_migrate / wem_model / wem_ctx_destroy.
 *
 * Array layouts follow the reference's float** arrays (first index slowest, n1
 * fastest): vel[ix][iz], m[ix][iz], d[ix][it], ix = imx*nmy + imy.
 */
#ifndef SHOTWEM_GB300_H
#define SHOTWEM_GB300_H
#include <stdbool.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Only the functions below are exported from shotwem.so. */
#if defined(__GNUC__)
#define WEM_API __attribute__((visibility("default")))
#else
#define WEM_API
#endif

/* Status codes. The reference has none: wem() is void (wem.c:3), main() calls
   exit(1) on a missing argument (shotwem.c:30-33) and SeisRead/SeisWrite only
   printf on I/O failure (seismic.c:277-289, 323-337). */
#define WEM_OK 0
#define WEM_ERR_ARG (-1)      /* invalid or missing argument */
#define WEM_ERR_SIZE (-2)     /* size the library does not support (e.g. a 3-D plane side not a power of two) */
#define WEM_ERR_CUDA (-3)     /* a CUDA runtime call failed */
#define WEM_ERR_TIMEOUT (-4)  /* a bounded device-side wait ran out */
#define WEM_ERR_IO (-5)       /* seis file could not be read or written */
#define WEM_ERR_NOMEM (-6)    /* host or device allocation failed */
#define WEM_ERR_NODEV (-7)    /* no CUDA device */

/* PSPI interpolation between reference wavefields */
#define WEM_INTERP_REF 0     /* the reference's arithmetic: wem.c:450-460 with linear_interp
                                (wem.c:473-478) returning float -> real part of the
                                nearest-lower reference wavefield */
#define WEM_INTERP_LINEAR 1  /* complex linear interpolation, the formula of wem.c:476 */

/* arithmetic of the depth-extrapolation FFTs */
#define WEM_PREC_FP32 0      /* complex FP32 */
#define WEM_PREC_SPLIT16 1   /* no counterpart in the reference: the DFT stages of the migration's
                                FFTs on the tensor cores with split fp16 (hi + lo) operands and
                                FP32 accumulation; 2-D rows of padx*nmx = 2048 only (other
                                geometries return WEM_ERR_SIZE). Modelling (wem_model*) computes
                                in FP32 in this mode. */

typedef struct wem_ctx wem_ctx;

/* Survey geometry and operator options; names and meaning as the arguments of
   wem() (wem.h:3-11) and the key=value options of main() (shotwem.c:27-42). */
typedef struct wem_params {
    int nt;         /* time samples per trace (and of the wavelet) */
    float ot, dt;
    int nmx;        /* image/receiver grid, x */
    float omx, dmx;
    int nmy;        /* image/receiver grid, y (1 for 2-D) */
    float omy, dmy;
    int nz;         /* depth steps */
    float oz, dz;
    float gz, sz;   /* receiver and source depth */
    int nref;       /* PSPI reference velocities per depth step (>= 2) */
    float fmin, fmax;
    int padt, padx; /* FFT padding factors for t and x/y */
    int pspi;       /* 1: PSPI (wem.c:380), 0: split-step (wem.c:289) */
    int interp;     /* WEM_INTERP_* */
    int precision;  /* WEM_PREC_* */
    int verbose;
} wem_params;

/* Last error message of the calling thread ("" if none). */
WEM_API const char *wem_last_error(void);
/* Library version, major*10000 + minor*100 + patch. */
WEM_API int wem_version(void);

/* A context owns a CUDA stream and the device buffers it reuses from call to call
   (tables, spectra, image accumulators); device = CUDA ordinal. */
WEM_API int wem_ctx_create(wem_ctx **ctx, int device);
WEM_API int wem_ctx_destroy(wem_ctx *ctx);

/* Build the per-velocity-model tables on the device: slowness split (wem.c:28-36),
   reference velocities and interpolation indices (wem.c:40-70), frequency and
   wavenumber grids (wem.c:79-89), wavelet spectrum (wem.c:112-119).
   vel: [nmx*nmy][nz]; wav: [nt]. Later wem_migrate / wem_model calls with the
   same ctx reuse them until the next wem_prepare. */
WEM_API int wem_prepare(wem_ctx *ctx, const wem_params *p, const float *vel, const float *wav);

/* Migration (adjoint, wem.c adj=true) of nshot shots, stacked into one image.
   Shot s has sources at (sx[s], sy[s]) and traces trace_offset[s] ..
   trace_offset[s+1]-1 of d ([ntrace][nt], host memory); trace i lies on grid
   cell trace_cell[i] (= imx*nmy + imy). Grid cells without a trace carry zero
   data, as the reference migrates the full grid for every shot (wem.c:122-133).
   m: [nmx*nmy][nz] host memory, overwritten. sy may be NULL (all 0). */
WEM_API int wem_migrate(wem_ctx *ctx, int nshot, const float *sx, const float *sy,
                const int64_t *trace_offset, const int32_t *trace_cell,
                const float *d, float *m);

/* Same, with every array already in device memory (ctx's device), ordered on
   ctx's stream; returns after enqueueing when sync == 0. */
WEM_API int wem_migrate_device(wem_ctx *ctx, int nshot, const float *sx, const float *sy,
                       const int64_t *trace_offset, const int32_t *trace_cell,
                       const float *d_dev, float *m_dev, int sync);

/* Modelling (wem.c adj=false, wem.c:252-281 and 177-188): the data the image m
   ([nmx*nmy][nz], host) produces for each of nshot shots, at the traces given by
   trace_offset / trace_cell (as in wem_migrate); d: [ntrace][nt] host, overwritten.
   exact = 0: the reference's operator (its PSPI interpolation after the inverse FFTs,
   the half-spectrum weights of its real inverse transform); exact = 1: the exact
   adjoint of wem_migrate with the same parameters, for least-squares migration
   (the two differ only for PSPI in laterally varying velocity and at the Nyquist
   frequency). On 3-D grids (nmy > 1) exact = 1 continues the receiver up with the adjoint of
   the 3-D migration step (PSPI; for split-step the reference's operator already is it). */
WEM_API int wem_model(wem_ctx *ctx, int nshot, const float *sx, const float *sy,
                      const int64_t *trace_offset, const int32_t *trace_cell,
                      const float *m, float *d, int exact);

/* Same, with m and d in device memory, ordered on ctx's stream. */
WEM_API int wem_model_device(wem_ctx *ctx, int nshot, const float *sx, const float *sy,
                             const int64_t *trace_offset, const int32_t *trace_cell,
                             const float *m_dev, float *d_dev, int exact, int sync);

/* One-call convenience: wem_prepare + wem_migrate. */
WEM_API int wem_migrate_survey(wem_ctx *ctx, const wem_params *p, const float *vel, const float *wav,
                       int nshot, const float *sx, const float *sy, const int64_t *trace_offset,
                       const int32_t *trace_cell, const float *d, float *m);

/* Source-side incidence angles of nshot shots: compute_angles (wem.c:566-684, and its
   file-level main in compute_angles.c), the operator behind Seismic.jl's ComputeAngles.
   For each shot the source wavefield of every frequency in [fmin, fmax] of the unpadded
   time axis is continued down with ssop_source's split-step operator on the unpadded
   grid, and angx = mean over frequency of (180/pi) atan(|du/dx| / (|du/dz| + 1e-10)),
   signed by the side the energy arrives from. Uses nt, dt, the grid, sz, fmin and fmax of
   p (padt, padx, pspi, nref, interp are not used; any nmx and nz). vel [nmx][nz], wav [nt];
   angx, angy: host [nshot][nmx][nz] (angy may be NULL; it is 0 in 2-D). Needs a context
   (wem_ctx_create), not wem_prepare. 2-D: nmx <= 4096; the shots run in batches whose
   wavefield volumes fit in half the free device memory, and the context keeps those buffers
   for its next call (wem_ctx_destroy frees them). 3-D (nmy > 1): nmx and nmy powers of
   two in [64, 1024] (WEM_ERR_SIZE otherwise); angy is then the y-axis angle. */
WEM_API int wem_angles(wem_ctx *ctx, const wem_params *p, const float *vel, const float *wav, int nshot,
                       const float *sx, const float *sy, float *angx, float *angy);

/* Elapsed device time (ms) of the last wem_migrate* call's GPU work, from CUDA
   events on ctx's stream; and how many kernels it launched. */
WEM_API int wem_last_timing(wem_ctx *ctx, float *ms, int *kernels);

/* Device time (ms) of each kernel of the last call: trace spectra, depth
   recursion, image reduction (CUDA events around each launch). */
WEM_API int wem_last_kernel_times(wem_ctx *ctx, float *ms_spectra, float *ms_extrapolate, float *ms_reduce);

/* Self-test of the bounded device-side waits (no counterpart in the reference): the
   tensor-core stages of the split16 form wait on an mbarrier with a time limit (about a
   second) and report WEM_ERR_TIMEOUT instead of hanging. This launches one such wait that
   nothing completes on `device` and returns in *timed_out whether it gave up (1), and in
   *ms how long the launch took; the context of the device stays usable. */
WEM_API int wem_selftest_wait_timeout(int device, int *timed_out, float *ms);

/* Measured FP32 FMA throughput of `device` in TFLOP/s (no counterpart in the reference):
   the best of three ~40 ms launches of a kernel of independent FMA chains, 2 FLOPs per
   FMA. The denominator of the CUDA-core roofline of the depth kernels. */
WEM_API int wem_measure_fp32_peak(int device, double *tflops);

/* How the last 2-D wem_migrate* call ran its depth recursion (no counterpart in the
   reference): threads per CTA, shots sharing one CTA's phase tables, CTAs launched,
   whether the call replayed a captured CUDA graph of the whole launch sequence (1) or
   launched it (0), and whether it timed the CTA shapes on this geometry first (1). */
WEM_API int wem_last_launch(wem_ctx *ctx, int *threads, int *shots_per_cta, int *grid, int *replayed,
                            int *tuned);

/* The form of the depth kernel the last 2-D wem_migrate* call ran (no counterpart in the
   reference; the autotuner's choice): *form 0 FP32 with one inverse transform per
   reference velocity, 1 split16 (tensor-core DFT stages), 2 FP32 paired (two references'
   real parts per inverse transform, PSPI nearest-lower mode), 3 FP32 on power-of-two rows
   carrying a transform length that is not a power of two (Bluestein), 4 FP32 PSPI with the
   phase tables read from device memory (rows of 1024 points and up, chosen only when the
   reference velocities' tables do not fit in shared memory); *bulk_tables 1 when
   the precomputed phase tables reached shared memory by bulk copies (TMA engine), 0 by
   per-thread asynchronous copies or built in each CTA. */
WEM_API int wem_last_launch_form(wem_ctx *ctx, int *form, int *bulk_tables);

/* The cudaStream_t (as void*) on which ctx orders all its work. */
WEM_API int wem_ctx_stream(wem_ctx *ctx, void **stream);

/* Migration of nshot shots that allocates nothing -- no counterpart in the reference.
   For callers that cannot call cudaMalloc/cudaFree while they run (an application that
   gives all device memory to its own pool at start-up, or a loop with a fixed memory
   budget): the caller passes device buffers for every input and the output, and all
   working memory comes from one fixed 24 MiB device array inside the library. CUDA
   loads that array (and the code of the kernels the call launches) on a device when
   the library's module is first used there (lazy module loading, CUDA's default), and
   the device keeps it until the process exits: make one small call on each device
   before handing the rest of its memory to a pool of your own, or run with
   CUDA_MODULE_LOADING=EAGER.
   vel_dev [nmx][nz], wav_dev [nt], d_dev [nshot][nmx][nt] (every shot on the full
   grid), m_dev [nmx][nz] (overwritten); sx, sy: host arrays of nshot source
   positions (sy may be NULL); stream: a cudaStream_t or NULL; the call returns when
   the result is in m_dev. 2-D only; padx*nmx in {256, 512, 1024, 2048}; nmx, nz <= 1024;
   nref <= 16; nshot <= 64; and the tables (12*nz*nmx bytes), trace spectra
   (8*nshot*nfreq*nmx bytes) and image (4*nz*nmx bytes) must fit the 24 MiB together --
   larger surveys return WEM_ERR_SIZE. Every call looks up the array's device address on
   the current device (the first call on a device also loads it there); make that first
   call before any stream capture. Each call waits for its stream (cudaStreamSynchronize)
   before it returns. Calls share the array: calls that overlap on the GPU (other
   streams, other host threads) race and corrupt each other. The image is summed with
   atomic additions, so its last bits can vary from run to run. */
WEM_API int wem_migrate_noalloc(const wem_params *p, const float *vel_dev, const float *wav_dev, int nshot,
                                const float *sx, const float *sy, const float *d_dev, float *m_dev, void *stream);

/* Elastic shot-profile migration (adj = 1) or its forward operator (adj = 0) on `device`:
   the reference's ewem() (ewem.c:3-253, ewem.h:3-16) for nshot shots at once, on 2-D
   (nmy = 1) and 3-D (nmy > 1) grids. With n = nmx*nmy cells (cell = imx*nmy + imy):
   vp, vs [n][nz]; wav [nt]; ux, uz [nshot][n][nt], the x and z components recorded on every
   grid cell (adj: read; forward: written); mpp, mps2 [n][nz], the P and S images (adj:
   written, stacked over the shots; forward: read); sy is read on 3-D grids (it may be NULL
   in 2-D). The y component and the S1 image take no part, as in the reference's separation
   (ewem.c:553-741). 2-D: padx*nmx a power of two in [64, 2048] or another length in
   [33, 1024]; 3-D: padx*nmx and padx*nmy powers of two in [64, 1024]. Allocates its device
   memory per call. */
WEM_API int wem_elastic(int device, const wem_params *p, const float *vp, const float *vs, const float *wav,
                        int nshot, const float *sx, const float *sy, float *ux, float *uz, float *mpp,
                        float *mps2, int adj);

/* Device time in ms of the calling thread's last wem_elastic call (spectra, tables, depth
   kernel, reduction or synthesis; CUDA events), no counterpart in the reference. */
WEM_API float wem_elastic_last_ms(void);

/* Drop-in for the reference's ewem() (ewem.h:3-16): the same arguments, float** rows as
   alloc2float builds them (seismic.c:92-106), one shot; adj: (ux, uz) -> (mpp, mps2), mps1
   zeroed; forward: (mpp, mps2) -> (ux, uz), uy zeroed. Returns a status instead of void. */
WEM_API int ewem(float **ux, float **uy, float **uz, float **mpp, float **mps1, float **mps2, float **wav, int nt,
                 float ot, float dt, int nmx, float omx, float dmx, int nmy, float omy, float dmy, float sx, float sy,
                 int nz, float oz, float dz, float gz, float sz, float **vp, float **vs, float fmin, float fmax,
                 int padt, int padx, bool adj, bool verbose);

/* Drop-in for the reference's wem() (wem.h:3-11). Same arguments, float** rows as
   alloc2float builds them (seismic.c:92-106). Returns a status instead of void.
   adj=true: d -> m (m overwritten); adj=false: m -> d (d overwritten). */
WEM_API int wem(float **d, float **m, float **wav, int nt, float ot, float dt, int nmx, float omx,
        float dmx, int nmy, float omy, float dmy, float sx, float sy, int nz, float oz, float dz,
        float gz, float sz, float **vel, int nref, float fmin, float fmax, int padt, int padx,
        bool adj, bool pspi, bool verbose);

/* Drop-in for shotwem.c:12 main(): argv holds key=value strings (argv[0] ignored):
   adj= pspi= nref= d= m= vel= wav= sx= sy= sz= gz= fmin= fmax= padt= padx= verbose=
   (y/n booleans, seismic.c:41-55), plus interp=ref|linear. Reads and writes seis
   files; returns a WEM_* status instead of calling exit(). */
WEM_API int shotwem_main(int argc, char **argv);

#ifdef __cplusplus
}
#endif
#endif
