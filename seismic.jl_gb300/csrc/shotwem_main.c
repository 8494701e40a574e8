/* shotwem_main.c -- the file-level drop-in: main(argc, argv) of src/Imaging/c/shotwem.c:12,
 * which the Julia wrapper binds by name (src/Imaging/ShotProfileWEM.jl:347).
 *
 * Same keys, defaults and file conventions as shotwem.c:27-130; differences, all
 * on error paths: a missing required key returns WEM_ERR_ARG instead of exit(1)
 * (shotwem.c:30-33), unreadable files return WEM_ERR_IO instead of a printf
 * (seismic.c:277-289), and a data file with more traces than the grid is read
 * only up to the grid size (the reference would overrun its buffer).
 * New key: interp=ref|linear (PSPI interpolation, default ref = reference arithmetic).
 */
#include <math.h>
#include <stdbool.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/shotwem_gb300.h"
#include "cli_args.h"
#include "seis_io.h"

static int run(int argc, char **argv)
{
    bool adj = true, pspi = true, verbose = false;
    arg_bool(argc, argv, "adj", &adj);
    arg_bool(argc, argv, "pspi", &pspi);
    arg_bool(argc, argv, "verbose", &verbose);
    const char *d_name = arg_value(argc, argv, "d"), *m_name = arg_value(argc, argv, "m");
    const char *vel_name = arg_value(argc, argv, "vel"), *wav_name = arg_value(argc, argv, "wav");
    if (!d_name || !m_name || !vel_name || !wav_name) {
        fprintf(stderr, "shotwem: required keys d= m= vel= wav= (common-shot wave-equation migration)\n");
        return WEM_ERR_ARG;
    }
    float sz = 0, gz = 0, sx = 0, sy = 0, fmin = 0, fmax = 80;
    int padt = 1, padx = 1, nref = 5;
    arg_float(argc, argv, "sz", &sz);
    arg_float(argc, argv, "gz", &gz);
    arg_float(argc, argv, "sx", &sx);
    arg_float(argc, argv, "sy", &sy);
    arg_float(argc, argv, "fmin", &fmin);
    arg_float(argc, argv, "fmax", &fmax);
    arg_int(argc, argv, "padt", &padt);
    arg_int(argc, argv, "padx", &padx);
    arg_int(argc, argv, "nref", &nref);
    const char *interp = arg_value(argc, argv, "interp");
    const int interp_mode = (interp && !strcmp(interp, "linear")) ? WEM_INTERP_LINEAR : WEM_INTERP_REF;

    seis_file_header fh;
    seis_init_file_header(&fh);
    if (seis_read_file_header(wav_name, &fh)) return WEM_ERR_IO;
    const int nt = fh.n[0];
    seis_init_file_header(&fh);
    if (seis_read_file_header(vel_name, &fh)) return WEM_ERR_IO;
    const int nz = fh.n[0];
    const int ntraces = fh.n[1] * fh.n[2] * fh.n[3] * fh.n[4];
    if (nt < 1 || nz < 1 || ntraces < 2) return WEM_ERR_ARG;

    int rc = WEM_OK, got = 0;
    float *wav = (float *)calloc((size_t)nt, sizeof(float));
    float *vel = (float *)calloc((size_t)ntraces * nz, sizeof(float));
    seis_trace_header *h_wav = (seis_trace_header *)calloc(1, sizeof(seis_trace_header));
    seis_trace_header *h_vel = (seis_trace_header *)calloc((size_t)ntraces, sizeof(seis_trace_header));
    float *d = NULL, *m = NULL;
    seis_trace_header *h_d = NULL, *h_m = NULL;
    float **dr = NULL, **mr = NULL, **vr = NULL;
    if (!wav || !vel || !h_wav || !h_vel) { rc = WEM_ERR_NOMEM; goto out; }
    if (seis_read(wav_name, wav, h_wav, 1, &fh, &got)) { rc = WEM_ERR_IO; goto out; }
    const float ot = fh.o[0], dt = fh.d[0];
    if (seis_read(vel_name, vel, h_vel, ntraces, &fh, &got)) { rc = WEM_ERR_IO; goto out; }
    /* grid from the velocity headers, shotwem.c:61-68 (dy is set to dx) */
    const int nx = h_vel[ntraces - 1].imx - h_vel[0].imx + 1;
    const int ny = h_vel[ntraces - 1].imy - h_vel[0].imy + 1;
    const float oz = fh.o[0], dz = fh.d[0];
    const float ox = h_vel[0].mx, dx = h_vel[1].mx - h_vel[0].mx;
    const float oy = h_vel[0].my, dy = dx;
    const int n = nx * ny;
    if (nx < 1 || ny < 1 || n > ntraces) { rc = WEM_ERR_ARG; goto out; }

    d = (float *)calloc((size_t)n * nt, sizeof(float));
    m = (float *)calloc((size_t)n * nz, sizeof(float));
    h_d = (seis_trace_header *)calloc((size_t)n, sizeof(seis_trace_header));
    h_m = (seis_trace_header *)calloc((size_t)n, sizeof(seis_trace_header));
    dr = (float **)malloc(sizeof(float *) * n);
    mr = (float **)malloc(sizeof(float *) * n);
    vr = (float **)malloc(sizeof(float *) * n);
    float *wr[1] = { wav };
    if (!d || !m || !h_d || !h_m || !dr || !mr || !vr) { rc = WEM_ERR_NOMEM; goto out; }
    for (int i = 0; i < n; i++) { dr[i] = d + (size_t)i * nt; mr[i] = m + (size_t)i * nz; vr[i] = vel + (size_t)i * nz; }
    seis_file_header fio;
    if (adj) {
        if (seis_read(d_name, d, h_d, n, &fio, &got)) { rc = WEM_ERR_IO; goto out; }
        memcpy(h_m, h_vel, sizeof(seis_trace_header) * n);
    } else {
        if (seis_read(m_name, m, h_m, n, &fio, &got)) { rc = WEM_ERR_IO; goto out; }
        for (int i = 0; i < n; i++) {
            h_d[i] = h_m[i];
            h_d[i].n1 = nt;
            h_d[i].d1 = dt;
            h_d[i].o1 = ot;
            h_d[i].gx = h_m[i].mx;
            h_d[i].gy = h_m[i].my;
            h_d[i].hx = h_m[i].mx - sx;
            h_d[i].hy = h_m[i].my - sy;
        }
    }
    if (interp_mode == WEM_INTERP_REF) {
        rc = wem(dr, mr, wr, nt, ot, dt, nx, ox, dx, ny, oy, dy, sx, sy, nz, oz, dz, gz, sz, vr, nref, fmin, fmax, padt,
                 padx, adj, pspi, verbose);
    } else {
        wem_ctx *ctx = NULL;
        wem_params p;
        memset(&p, 0, sizeof(p));
        p.nt = nt; p.ot = ot; p.dt = dt; p.nmx = nx; p.omx = ox; p.dmx = dx; p.nmy = ny; p.omy = oy; p.dmy = dy;
        p.nz = nz; p.oz = oz; p.dz = dz; p.gz = gz; p.sz = sz; p.nref = nref; p.fmin = fmin; p.fmax = fmax;
        p.padt = padt; p.padx = padx; p.pspi = pspi; p.interp = interp_mode; p.precision = WEM_PREC_FP32;
        p.verbose = verbose;
        if (!adj) { rc = WEM_ERR_SIZE; goto out; }
        rc = wem_ctx_create(&ctx, 0);
        if (!rc) {
            int64_t off[2] = { 0, n };
            int32_t *cell = (int32_t *)malloc(sizeof(int32_t) * n);
            if (!cell) rc = WEM_ERR_NOMEM;
            else {
                for (int i = 0; i < n; i++) cell[i] = i;
                rc = wem_migrate_survey(ctx, &p, vel, wav, 1, &sx, &sy, off, cell, d, m);
                free(cell);
            }
            wem_ctx_destroy(ctx);
        }
    }
    if (rc) goto out;
    if (adj) {
        /* image headers from the data headers, shotwem.c:114-122 */
        for (int i = 0; i < n; i++) {
            h_m[i].mx = h_d[i].gx;
            h_m[i].my = h_d[i].gy;
            h_m[i].imx = (int)truncf((h_m[i].mx - ox) / dx);
            h_m[i].imy = (int)truncf((h_m[i].my - oy) / dy);
        }
        seis_init_file_header(&fio);
        fio.n[0] = nz; fio.o[0] = oz; fio.d[0] = dz;
        fio.n[1] = nx; fio.o[1] = ox; fio.d[1] = dx;
        fio.n[2] = ny; fio.o[2] = oy; fio.d[2] = dy;
        if (seis_write(m_name, m, h_m, &fio)) rc = WEM_ERR_IO;
    } else {
        seis_init_file_header(&fio);
        fio.n[0] = nt; fio.o[0] = ot; fio.d[0] = dt;
        fio.n[1] = nx; fio.o[1] = ox; fio.d[1] = dx;
        fio.n[2] = ny; fio.o[2] = oy; fio.d[2] = dy;
        if (seis_write(d_name, d, h_d, &fio)) rc = WEM_ERR_IO;
    }
out:
    free(wav); free(vel); free(h_wav); free(h_vel); free(d); free(m); free(h_d); free(h_m);
    free(dr); free(mr); free(vr);
    if (rc && verbose) fprintf(stderr, "shotwem: status %d: %s\n", rc, wem_last_error());
    return rc;
}

int shotwem_main(int argc, char **argv) { return run(argc, argv); }

/* The symbol the Julia wrapper calls: ccall((:main, "shotwem"), ...). */
WEM_API int main(int argc, char **argv) { return run(argc, argv); }
