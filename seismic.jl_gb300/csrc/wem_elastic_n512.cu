// wem_elastic_n512.cu -- instantiates the elastic depth kernels for rows of 512 samples.
#include "wem_elastic.cuh"

namespace gbwem {
template int ewem_launch_n<512>(int, int, const EwemArgs *, int, int, cudaStream_t, int *, size_t *);
}  // namespace gbwem
