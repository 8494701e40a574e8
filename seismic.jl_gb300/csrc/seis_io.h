/* seis_io.h -- the seis file format the reference's C core and Julia package share
 * (C: src/API/c/seismic.h:20-86, seismic.c:270-461; Julia: src/ReadWrite/Header.jl,
 * SeisRead.jl, SeisWrite.jl):
 *   <name>            text header, lines "\t<key>=<value>" (n1..n5, o1..o5, d1..d5,
 *                     label/unit/title strings, data_format, esize, in, headers);
 *                     a later line overrides an earlier one;
 *   <in> (@data@)     ntraces x n1 native float32, trace after trace;
 *   <headers>         ntraces x 124-byte trace headers (31 four-byte fields).
 * The structs keep the reference's field order because the header file is binary.
 */
#ifndef WEM_SEIS_IO_H
#define WEM_SEIS_IO_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct seis_trace_header {
    int tracenum;
    float o1;
    int n1;
    float d1;
    float sx, sy, gx, gy, mx, my, hx, hy, h, az, ang;
    int isx, isy, igx, igy, imx, imy, ihx, ihy, ih, iaz, iang;
    float selev, gelev, sstat, gstat;
    int trid;
} seis_trace_header;

typedef struct seis_file_header {
    int n[5];
    float o[5];
    float d[5];
    char label[5][100];
    char unit[5][100];
    char title[100];
    char data_format[100];
    int esize;
    char dname[512];
    char hname[512];
} seis_file_header;

void seis_init_file_header(seis_file_header *fh);
/* 0 on success, nonzero when the text header cannot be opened */
int seis_read_file_header(const char *name, seis_file_header *fh);
/* Reads up to max_traces traces (rows of n1 floats at d + i*n1) and their headers.
   *ntraces receives the number of traces in the file. */
int seis_read(const char *name, float *d, seis_trace_header *h, int max_traces, seis_file_header *fh, int *ntraces);
/* Writes name, name@data@ and name@headers@ (prefixed by $DATAPATH when set, as
   seismic.c:306-318); the trace count is n2*n3*n4*n5 of fh. */
int seis_write(const char *name, const float *d, const seis_trace_header *h, seis_file_header *fh);

#ifdef __cplusplus
}
#endif
#endif
