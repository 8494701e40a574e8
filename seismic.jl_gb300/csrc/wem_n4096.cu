// wem_n4096.cu -- instantiates the depth-recursion kernels for rows of 4096 samples.
#include "wem_kernels.cuh"

namespace gbwem {
template int mig_launch<4096>(int, int, int, int, int, const MigArgs *, int, cudaStream_t, int *, int *, size_t *, int *, int);
template int model_launch<4096>(int, int, int, int, int, const MigArgs *, const BornArgs *, int, cudaStream_t, int *,
                               int *, size_t *, int *, int);
}  // namespace gbwem
