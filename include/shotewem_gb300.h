/* shotewem_gb300.h -- entry points of shotewem.so, the GPU drop-in for the reference's
 * shotewem library (src/Imaging/c/shotewem.c), which Seismic.jl's ShotProfileEWEM calls by
 * name (src/Imaging/ShotProfileEWEM.jl:416-430). The computation is wem_elastic of
 * shotwem.so (include/shotwem_gb300.h), which shotewem.so links.
 */
#ifndef SHOTEWEM_GB300_H
#define SHOTEWEM_GB300_H

#include "shotwem_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* main(argc, argv) of shotewem.c:13 -- same keys (ux= uy= uz= mpp= mps1= mps2= vp= vs= wav=
   required; adj verbose sz gz sx sy fmin fmax padt padx), same seis files; 2-D grids;
   returns 0 or a WEM_ERR_* status instead of exit(1). Replaces shotewem.c:13-222. */
WEM_API int shotewem_main(int argc, char **argv);

#ifdef __cplusplus
}
#endif
#endif
