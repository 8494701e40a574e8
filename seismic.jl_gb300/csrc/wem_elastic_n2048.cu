// wem_elastic_n2048.cu -- instantiates the elastic depth kernels for rows of 2048 samples.
#include "wem_elastic.cuh"

namespace gbwem {
template int ewem_launch_n<2048>(int, int, const EwemArgs *, int, int, cudaStream_t, int *, size_t *);
}  // namespace gbwem
