/* compute_angles_gb300.h -- entry points of compute_angles.so, the GPU drop-in for the
 * reference's compute_angles library (src/Imaging/c/compute_angles.c), which
 * Seismic.jl's ComputeAngles calls by name (src/Imaging/ComputeAngles.jl:126-140).
 * The computation is wem_angles of shotwem.so (include/shotwem_gb300.h), which
 * compute_angles.so links.
 */
#ifndef COMPUTE_ANGLES_GB300_H
#define COMPUTE_ANGLES_GB300_H

#include "shotwem_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* main(argc, argv) of compute_angles.c:12 -- same keys (angx= angy= vel= dipx= dipy= wav=
   required; sz sx sy fmin fmax dip_flag verbose), same seis files; returns 0 or a
   WEM_ERR_* status instead of exit(1). Replaces compute_angles.c:12-120. */
WEM_API int compute_angles_main(int argc, char **argv);

#ifdef __cplusplus
}
#endif
#endif
