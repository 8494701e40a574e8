/* seis_io.c -- reader and writer of the seis format (see seis_io.h). */
#include "seis_io.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

void seis_init_file_header(seis_file_header *fh)
{
    /* defaults of seismic.c:346-378 */
    memset(fh, 0, sizeof(*fh));
    for (int i = 0; i < 5; i++) { fh->n[i] = 1; fh->o[i] = 1.f; fh->d[i] = 1.f; }
    fh->o[0] = 0.f;
    fh->d[0] = 0.f;
    strcpy(fh->data_format, "native_float");
    fh->esize = 4;
    strcpy(fh->dname, "NULL");
    strcpy(fh->hname, "NULL");
}

/* value of a quoted string field: key="value" */
static void quoted(const char *p, char *out, size_t cap)
{
    const char *q = strchr(p, '"');
    if (!q) { snprintf(out, cap, "%s", p); return; }
    q++;
    const char *e = strchr(q, '"');
    size_t n = e ? (size_t)(e - q) : strlen(q);
    if (n >= cap) n = cap - 1;
    memcpy(out, q, n);
    out[n] = '\0';
}

int seis_read_file_header(const char *name, seis_file_header *fh)
{
    FILE *fp = fopen(name, "r");
    if (!fp) return 1;
    char line[1024];
    while (fgets(line, sizeof(line), fp)) {
        char *s = line;
        while (*s == ' ' || *s == '\t') s++;
        char *eq = strchr(s, '=');
        if (!eq) continue;
        *eq = '\0';
        const char *key = s, *val = eq + 1;
        char *nl = strchr(eq + 1, '\n');
        if (nl) *nl = '\0';
        if (key[0] && key[1] && !key[2] && (key[0] == 'n' || key[0] == 'o' || key[0] == 'd') && key[1] >= '1' &&
            key[1] <= '5') {
            const int i = key[1] - '1';
            if (key[0] == 'n') fh->n[i] = atoi(val);
            else if (key[0] == 'o') fh->o[i] = (float)atof(val);
            else fh->d[i] = (float)atof(val);
        } else if (!strcmp(key, "in")) quoted(val, fh->dname, sizeof(fh->dname));
        else if (!strcmp(key, "headers")) quoted(val, fh->hname, sizeof(fh->hname));
        else if (!strcmp(key, "title")) quoted(val, fh->title, sizeof(fh->title));
        else if (!strcmp(key, "data_format")) quoted(val, fh->data_format, sizeof(fh->data_format));
        else if (!strcmp(key, "esize")) fh->esize = atoi(val);
        else if (!strncmp(key, "label", 5) && key[5] >= '1' && key[5] <= '5' && !key[6])
            quoted(val, fh->label[key[5] - '1'], sizeof(fh->label[0]));
        else if (!strncmp(key, "unit", 4) && key[4] >= '1' && key[4] <= '5' && !key[5])
            quoted(val, fh->unit[key[4] - '1'], sizeof(fh->unit[0]));
    }
    fclose(fp);
    return 0;
}

int seis_read(const char *name, float *d, seis_trace_header *h, int max_traces, seis_file_header *fh, int *ntraces)
{
    seis_init_file_header(fh);
    if (seis_read_file_header(name, fh)) return 1;
    const long long ntr = (long long)fh->n[1] * fh->n[2] * fh->n[3] * fh->n[4];
    if (ntraces) *ntraces = (int)ntr;
    const int nread = ntr < max_traces ? (int)ntr : max_traces;
    if (h) {
        FILE *fp = fopen(fh->hname, "rb");
        if (!fp) return 2;
        size_t got = fread(h, sizeof(seis_trace_header), (size_t)nread, fp);
        fclose(fp);
        if (got != (size_t)nread) return 3;
    }
    if (d) {
        FILE *fp = fopen(fh->dname, "rb");
        if (!fp) return 4;
        size_t got = fread(d, sizeof(float) * (size_t)fh->n[0], (size_t)nread, fp);
        fclose(fp);
        if (got != (size_t)nread) return 5;
    }
    return 0;
}

int seis_write(const char *name, const float *d, const seis_trace_header *h, seis_file_header *fh)
{
    const char *dp = getenv("DATAPATH");
    snprintf(fh->dname, sizeof(fh->dname), "%s%s@data@", dp ? dp : "", name);
    snprintf(fh->hname, sizeof(fh->hname), "%s%s@headers@", dp ? dp : "", name);
    FILE *fp = fopen(name, "w");
    if (!fp) return 1;
    for (int i = 0; i < 5; i++) fprintf(fp, "\tn%d=%d\n", i + 1, fh->n[i]);
    for (int i = 0; i < 5; i++) fprintf(fp, "\to%d=%f\n", i + 1, fh->o[i]);
    for (int i = 0; i < 5; i++) fprintf(fp, "\td%d=%f\n", i + 1, fh->d[i]);
    for (int i = 0; i < 5; i++) fprintf(fp, "\tlabel%d=\"%s\"\n", i + 1, fh->label[i]);
    for (int i = 0; i < 5; i++) fprintf(fp, "\tunit%d=\"%s\"\n", i + 1, fh->unit[i]);
    fprintf(fp, "\ttitle=\"%s\"\n", fh->title);
    fprintf(fp, "\tdata_format=\"%s\"\n", fh->data_format);
    fprintf(fp, "\tesize=%d\n", fh->esize);
    fprintf(fp, "\tin=\"%s\"\n", fh->dname);
    fprintf(fp, "\theaders=\"%s\"\n", fh->hname);
    if (fclose(fp)) return 1;
    const size_t ntr = (size_t)fh->n[1] * fh->n[2] * fh->n[3] * fh->n[4];
    fp = fopen(fh->hname, "wb");
    if (!fp) return 2;
    size_t put = fwrite(h, sizeof(seis_trace_header), ntr, fp);
    if (fclose(fp) || put != ntr) return 3;
    fp = fopen(fh->dname, "wb");
    if (!fp) return 4;
    put = fwrite(d, sizeof(float) * (size_t)fh->n[0], ntr, fp);
    if (fclose(fp) || put != ntr) return 5;
    return 0;
}
