/* cli_args.h -- the key=value argument lookup of the main() drop-ins (shotwem, compute_angles,
 * shotewem), with the semantics of the reference's par_read_* (src/API/c/seismic.c:2-71): the
 * first argument from argv[1] on whose name matches wins; booleans are true when the value
 * starts with 'y' (seismic.c:50); a missing key leaves the default.
 */
#ifndef WEM_CLI_ARGS_H
#define WEM_CLI_ARGS_H
#include <stdbool.h>
#include <stdlib.h>
#include <string.h>

static inline const char *arg_value(int argc, char **argv, const char *key)
{
    const size_t n = strlen(key);
    for (int i = 1; i < argc; i++) {
        if (!argv[i]) continue;
        if (!strncmp(argv[i], key, n) && argv[i][n] == '=') return argv[i] + n + 1;
    }
    return NULL;
}
static inline void arg_bool(int argc, char **argv, const char *k, bool *v)
{
    const char *s = arg_value(argc, argv, k);
    if (s) *v = (s[0] == 'y');
}
static inline void arg_int(int argc, char **argv, const char *k, int *v)
{
    const char *s = arg_value(argc, argv, k);
    if (s) *v = atoi(s);
}
static inline void arg_float(int argc, char **argv, const char *k, float *v)
{
    const char *s = arg_value(argc, argv, k);
    if (s) *v = (float)atof(s);
}

#endif
