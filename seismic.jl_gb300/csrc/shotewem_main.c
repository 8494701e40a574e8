/* shotewem_main.c -- the file-level drop-in for the reference's shotewem.so: main(argc, argv)
 * of src/Imaging/c/shotewem.c:13, which Seismic.jl's ShotProfileEWEM binds by name
 * (src/Imaging/ShotProfileEWEM.jl:416-430), computing on the GPU through wem_elastic
 * (include/shotwem_gb300.h).
 *
 * Same keys, defaults and files as shotewem.c:35-120: ux= uy= uz= mpp= mps1= mps2= vp= vs=
 * wav= required; adj (y), verbose, sz, gz, sx, sy (0), fmin (0), fmax (80), padt, padx (1).
 * nt from the wavelet's n1 with ot/dt from its text header; nz from vp's n1; the grid from
 * vp's trace headers (nx, ny from the imx/imy span, ox/dx from the first two mx, oy from the
 * first my, dy = dx); oz/dz from the text header of the last model file read (vs), as there.
 * Migration writes mpp (trid 1), mps1 and mps2 (trid 2) with vp's headers, mx/my from the
 * ux traces' gx/gy and imx/imy recomputed (shotewem.c:175-198); mps1 is zero because the
 * separation leaves S1 out (ewem.c:553-741). The forward operator writes ux, uy, uz with
 * mpp's headers, n1/o1/d1 of the wavelet, gx/gy = mx/my and hx/hy the offsets (shotewem.c:
 * 120-150); uy is zero. Differences, on error paths only: a missing key returns WEM_ERR_ARG
 * instead of exit(1), an unreadable file WEM_ERR_IO, a data file with more traces than the
 * grid is read only up to the grid size. 3-D grids (ny > 1) run on the x-y plane passes when
 * padx*nx and padx*ny are powers of two in [64, 1024], and return WEM_ERR_SIZE otherwise.
 */
#include <math.h>
#include <stdbool.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/shotwem_gb300.h"
#include "cli_args.h"
#include "seis_io.h"

enum { UX, UY, UZ, MPP, MPS1, MPS2, NFILES };

static int run(int argc, char **argv)
{
    static const char *keys[NFILES] = { "ux", "uy", "uz", "mpp", "mps1", "mps2" };
    bool adj = true, verbose = false;
    arg_bool(argc, argv, "adj", &adj);
    arg_bool(argc, argv, "verbose", &verbose);
    const char *name[NFILES];
    for (int k = 0; k < NFILES; k++) name[k] = arg_value(argc, argv, keys[k]);
    const char *vp_name = arg_value(argc, argv, "vp"), *vs_name = arg_value(argc, argv, "vs");
    const char *wav_name = arg_value(argc, argv, "wav");
    bool missing = !vp_name || !vs_name || !wav_name;
    for (int k = 0; k < NFILES; k++) missing = missing || !name[k];
    if (missing) {
        fprintf(stderr, "shotewem: required keys ux= uy= uz= mpp= mps1= mps2= vp= vs= wav= "
                        "(common-shot elastic wave-equation migration)\n");
        return WEM_ERR_ARG;
    }
    float sz = 0, gz = 0, sx = 0, sy = 0, fmin = 0, fmax = 80;
    int padt = 1, padx = 1;
    arg_float(argc, argv, "sz", &sz);
    arg_float(argc, argv, "gz", &gz);
    arg_float(argc, argv, "sx", &sx);
    arg_float(argc, argv, "sy", &sy);
    arg_float(argc, argv, "fmin", &fmin);
    arg_float(argc, argv, "fmax", &fmax);
    arg_int(argc, argv, "padt", &padt);
    arg_int(argc, argv, "padx", &padx);

    seis_file_header fh;
    seis_init_file_header(&fh);
    if (seis_read_file_header(wav_name, &fh)) return WEM_ERR_IO;
    const int nt = fh.n[0];
    seis_init_file_header(&fh);
    if (seis_read_file_header(vp_name, &fh)) return WEM_ERR_IO;
    const int nz = fh.n[0];
    const int ntraces = fh.n[1] * fh.n[2] * fh.n[3] * fh.n[4];
    if (nt < 2 || nz < 1 || ntraces < 2) return WEM_ERR_ARG;

    int rc = WEM_OK, got = 0;
    float *wav = (float *)calloc((size_t)nt, sizeof(float));
    float *vp = (float *)calloc((size_t)ntraces * nz, sizeof(float));
    float *vs = (float *)calloc((size_t)ntraces * nz, sizeof(float));
    seis_trace_header *h_vp = (seis_trace_header *)calloc((size_t)ntraces, sizeof(seis_trace_header));
    seis_trace_header *h_vs = (seis_trace_header *)calloc((size_t)ntraces, sizeof(seis_trace_header));
    seis_trace_header *h_wav = (seis_trace_header *)calloc(1, sizeof(seis_trace_header));
    float *f[NFILES] = { 0 };
    seis_trace_header *h[NFILES] = { 0 };
    if (!wav || !vp || !vs || !h_vp || !h_vs || !h_wav) { rc = WEM_ERR_NOMEM; goto out; }
    if (seis_read(wav_name, wav, h_wav, 1, &fh, &got)) { rc = WEM_ERR_IO; goto out; }
    const float ot = fh.o[0], dt = fh.d[0];
    if (seis_read(vp_name, vp, h_vp, ntraces, &fh, &got)) { rc = WEM_ERR_IO; goto out; }
    if (seis_read(vs_name, vs, h_vs, ntraces, &fh, &got)) { rc = WEM_ERR_IO; goto out; }
    /* shotewem.c:74-82 */
    const int nx = h_vp[ntraces - 1].imx - h_vp[0].imx + 1;
    const int ny = h_vp[ntraces - 1].imy - h_vp[0].imy + 1;
    const float oz = fh.o[0], dz = fh.d[0];
    const float ox = h_vp[0].mx, dx = h_vp[1].mx - h_vp[0].mx;
    const float oy = h_vp[0].my, dy = dx;
    const int n = nx * ny;
    if (nx < 1 || ny < 1 || n > ntraces) { rc = WEM_ERR_ARG; goto out; }
    for (int k = 0; k < NFILES; k++) {
        const int n1 = k < MPP ? nt : nz;
        f[k] = (float *)calloc((size_t)n * n1, sizeof(float));
        h[k] = (seis_trace_header *)calloc((size_t)n, sizeof(seis_trace_header));
        if (!f[k] || !h[k]) { rc = WEM_ERR_NOMEM; goto out; }
    }
    seis_file_header fio;
    /* inputs: the three components (migration) or the three images (forward), shotewem.c:84-104;
       uy and mps1 are read as there although the 2-D operator does not use them */
    for (int k = adj ? UX : MPP; k < (adj ? MPP : NFILES); k++)
        if (seis_read(name[k], f[k], h[k], n, &fio, &got)) { rc = WEM_ERR_IO; goto out; }

    wem_params p;
    memset(&p, 0, sizeof(p));
    p.nt = nt; p.ot = ot; p.dt = dt; p.nmx = nx; p.omx = ox; p.dmx = dx; p.nmy = ny; p.omy = oy; p.dmy = dy;
    p.nz = nz; p.oz = oz; p.dz = dz; p.gz = gz; p.sz = sz; p.fmin = fmin; p.fmax = fmax;
    p.padt = padt; p.padx = padx; p.verbose = verbose;
    if ((rc = wem_elastic(0, &p, vp, vs, wav, 1, &sx, &sy, f[UX], f[UZ], f[MPP], f[MPS2], adj ? 1 : 0))) goto out;

    seis_file_header fo;
    seis_init_file_header(&fo);
    if (adj) { /* shotewem.c:171-198 */
        static const int trid[3] = { 1, 2, 2 };
        memset(f[MPS1], 0, sizeof(float) * (size_t)n * nz);
        fo.n[0] = nz; fo.o[0] = oz; fo.d[0] = dz;
        fo.n[1] = nx; fo.o[1] = ox; fo.d[1] = dx;
        fo.n[2] = ny; fo.o[2] = oy; fo.d[2] = dy;
        for (int k = MPP; k < NFILES; k++) {
            for (int i = 0; i < n; i++) {
                h[k][i] = h_vp[i];
                h[k][i].trid = trid[k - MPP];
                h[k][i].mx = h[UX][i].gx;
                h[k][i].my = h[UX][i].gy;
                h[k][i].imx = (int)truncf((h[k][i].mx - ox) / dx);
                h[k][i].imy = (int)truncf((h[k][i].my - oy) / dy);
            }
            if (seis_write(name[k], f[k], h[k], &fo)) { rc = WEM_ERR_IO; goto out; }
        }
    } else { /* shotewem.c:120-150, 199-206 */
        memset(f[UY], 0, sizeof(float) * (size_t)n * nt);
        fo.n[0] = nt; fo.o[0] = ot; fo.d[0] = dt;
        fo.n[1] = nx; fo.o[1] = ox; fo.d[1] = dx;
        fo.n[2] = ny; fo.o[2] = oy; fo.d[2] = dy;
        for (int k = UX; k < MPP; k++) {
            for (int i = 0; i < n; i++) {
                h[k][i] = h[MPP][i];
                h[k][i].n1 = nt;
                h[k][i].d1 = dt;
                h[k][i].o1 = ot;
                h[k][i].gx = h[MPP][i].mx;
                h[k][i].gy = h[MPP][i].my;
                h[k][i].hx = h[MPP][i].mx - sx;
                h[k][i].hy = h[MPP][i].my - sy;
            }
            if (seis_write(name[k], f[k], h[k], &fo)) { rc = WEM_ERR_IO; goto out; }
        }
    }
out:
    for (int k = 0; k < NFILES; k++) { free(f[k]); free(h[k]); }
    free(wav); free(vp); free(vs); free(h_vp); free(h_vs); free(h_wav);
    if (rc && verbose) fprintf(stderr, "shotewem: status %d: %s\n", rc, wem_last_error());
    return rc;
}

/* The symbol ShotProfileEWEM calls: ccall((:main, "shotewem"), ...). */
WEM_API int main(int argc, char **argv) { return run(argc, argv); }
WEM_API int shotewem_main(int argc, char **argv) { return run(argc, argv); }
