// wem_elastic_n1024.cu -- instantiates the elastic depth kernels for rows of 1024 samples.
#include "wem_elastic.cuh"

namespace gbwem {
template int ewem_launch_n<1024>(int, int, const EwemArgs *, int, int, cudaStream_t, int *, size_t *);
}  // namespace gbwem
