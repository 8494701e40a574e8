/* compute_angles_main.c -- the file-level drop-in for the reference's compute_angles.so:
 * main(argc, argv) of src/Imaging/c/compute_angles.c:12, which Seismic.jl's
 * ComputeAngles binds by name (src/Imaging/ComputeAngles.jl:126-140), computing on the
 * GPU through wem_angles (include/shotwem_gb300.h).
 *
 * Same keys, defaults and files as compute_angles.c:27-120: angx= angy= vel= dipx= dipy=
 * wav= required; sz, sx, sy, fmin (0), fmax (80), dip_flag, verbose. The grid comes from
 * the velocity's trace headers (nx, ny from the imx/imy span, dx from the first two mx,
 * dy from the y step or dx); ot/dt from the wavelet's first trace header. The output
 * sections carry the velocity's trace headers with sx set. Differences, on error paths
 * only: a missing key returns WEM_ERR_ARG instead of exit(1), an unreadable file
 * WEM_ERR_IO.
 */
#include <stdbool.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/shotwem_gb300.h"
#include "cli_args.h"
#include "seis_io.h"

static int run(int argc, char **argv)
{
    bool verbose = false, dip_flag = false;
    arg_bool(argc, argv, "verbose", &verbose);
    arg_bool(argc, argv, "dip_flag", &dip_flag);
    const char *angx_name = arg_value(argc, argv, "angx"), *angy_name = arg_value(argc, argv, "angy");
    const char *vel_name = arg_value(argc, argv, "vel"), *wav_name = arg_value(argc, argv, "wav");
    const char *dipx_name = arg_value(argc, argv, "dipx"), *dipy_name = arg_value(argc, argv, "dipy");
    if (!angx_name || !angy_name || !vel_name || !dipx_name || !dipy_name || !wav_name) {
        fprintf(stderr, "compute_angles: required keys angx= angy= vel= dipx= dipy= wav=\n");
        return WEM_ERR_ARG;
    }
    float sz = 0, sx = 0, sy = 0, fmin = 0, fmax = 80;
    arg_float(argc, argv, "sz", &sz);
    arg_float(argc, argv, "sx", &sx);
    arg_float(argc, argv, "sy", &sy);
    arg_float(argc, argv, "fmin", &fmin);
    arg_float(argc, argv, "fmax", &fmax);

    seis_file_header fh;
    seis_init_file_header(&fh);
    if (seis_read_file_header(wav_name, &fh)) return WEM_ERR_IO;
    const int nt = fh.n[0];
    seis_init_file_header(&fh);
    if (seis_read_file_header(vel_name, &fh)) return WEM_ERR_IO;
    const int nz = fh.n[0];
    const int ntraces = fh.n[1] * fh.n[2] * fh.n[3] * fh.n[4];
    if (nt < 2 || nz < 1 || ntraces < 2) return WEM_ERR_ARG;

    int rc = WEM_OK, got = 0;
    float *wav = (float *)calloc((size_t)nt, sizeof(float));
    float *vel = (float *)calloc((size_t)ntraces * nz, sizeof(float));
    seis_trace_header *h_wav = (seis_trace_header *)calloc(1, sizeof(seis_trace_header));
    seis_trace_header *h_vel = (seis_trace_header *)calloc((size_t)ntraces, sizeof(seis_trace_header));
    float *ax = NULL, *ay = NULL, *dip = NULL;
    seis_trace_header *h_out = NULL, *h_dip = NULL;
    wem_ctx *ctx = NULL;
    if (!wav || !vel || !h_wav || !h_vel) { rc = WEM_ERR_NOMEM; goto out; }
    if (seis_read(wav_name, wav, h_wav, 1, &fh, &got)) { rc = WEM_ERR_IO; goto out; }
    const float ot = h_wav[0].o1, dt = h_wav[0].d1;
    if (seis_read(vel_name, vel, h_vel, ntraces, &fh, &got)) { rc = WEM_ERR_IO; goto out; }
    /* compute_angles.c:56-63 */
    const int nx = h_vel[ntraces - 1].imx - h_vel[0].imx + 1;
    const int ny = h_vel[ntraces - 1].imy - h_vel[0].imy + 1;
    const float oz = h_vel[0].o1, dz = h_vel[0].d1;
    const float ox = h_vel[0].mx, dx = h_vel[1].mx - h_vel[0].mx;
    const float oy = h_vel[0].my;
    const float dy = ntraces > nx ? h_vel[nx].my - h_vel[nx - 1].my : dx;
    const int n = nx * ny;
    if (nx < 1 || ny < 1 || n > ntraces) { rc = WEM_ERR_ARG; goto out; }

    ax = (float *)calloc((size_t)n * nz, sizeof(float));
    ay = (float *)calloc((size_t)n * nz, sizeof(float));
    h_out = (seis_trace_header *)calloc((size_t)n, sizeof(seis_trace_header));
    if (!ax || !ay || !h_out) { rc = WEM_ERR_NOMEM; goto out; }
    wem_params p;
    memset(&p, 0, sizeof(p));
    p.nt = nt; p.ot = ot; p.dt = dt; p.nmx = nx; p.omx = ox; p.dmx = dx; p.nmy = ny; p.omy = oy; p.dmy = dy;
    p.nz = nz; p.oz = oz; p.dz = dz; p.sz = sz; p.fmin = fmin; p.fmax = fmax; p.padt = 1; p.padx = 1;
    p.verbose = verbose;
    if ((rc = wem_ctx_create(&ctx, 0))) goto out;
    if ((rc = wem_angles(ctx, &p, vel, wav, 1, &sx, &sy, ax, ay))) goto out;
    if (dip_flag) { /* compute_angles.c:83-96 */
        dip = (float *)calloc((size_t)ntraces * nz, sizeof(float));
        h_dip = (seis_trace_header *)calloc((size_t)ntraces, sizeof(seis_trace_header));
        if (!dip || !h_dip) { rc = WEM_ERR_NOMEM; goto out; }
        if (seis_read(dipx_name, dip, h_dip, ntraces, &fh, &got)) { rc = WEM_ERR_IO; goto out; }
        for (size_t i = 0; i < (size_t)n * nz; i++) ax[i] += dip[i];
        if (seis_read(dipy_name, dip, h_dip, ntraces, &fh, &got)) { rc = WEM_ERR_IO; goto out; }
        for (size_t i = 0; i < (size_t)n * nz; i++) ay[i] += dip[i];
    }
    for (int i = 0; i < n; i++) {
        h_out[i] = h_vel[i];
        h_out[i].sx = sx;
    }
    seis_file_header fo;
    seis_init_file_header(&fo);
    fo.n[0] = nz; fo.o[0] = oz; fo.d[0] = dz;
    fo.n[1] = nx; fo.o[1] = ox; fo.d[1] = dx;
    fo.n[2] = ny; fo.o[2] = oy; fo.d[2] = dy;
    if (seis_write(angx_name, ax, h_out, &fo) || seis_write(angy_name, ay, h_out, &fo)) rc = WEM_ERR_IO;
out:
    if (ctx) wem_ctx_destroy(ctx);
    free(wav); free(vel); free(h_wav); free(h_vel); free(ax); free(ay); free(h_out); free(dip); free(h_dip);
    if (rc && verbose) fprintf(stderr, "compute_angles: status %d: %s\n", rc, wem_last_error());
    return rc;
}

/* The symbol ComputeAngles calls: ccall((:main, "compute_angles"), ...). */
WEM_API int main(int argc, char **argv) { return run(argc, argv); }
WEM_API int compute_angles_main(int argc, char **argv) { return run(argc, argv); }
