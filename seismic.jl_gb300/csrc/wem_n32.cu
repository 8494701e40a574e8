// wem_n32.cu -- instantiates the depth-recursion kernels for rows of 32 samples.
#include "wem_kernels.cuh"

namespace gbwem {
template int mig_launch<32>(int, int, int, int, int, const MigArgs *, int, cudaStream_t, int *, int *, size_t *, int *, int);
template int model_launch<32>(int, int, int, int, int, const MigArgs *, const BornArgs *, int, cudaStream_t, int *,
                               int *, size_t *, int *, int);
}  // namespace gbwem
