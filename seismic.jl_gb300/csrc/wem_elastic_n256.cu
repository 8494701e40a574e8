// wem_elastic_n256.cu -- instantiates the elastic depth kernels for rows of 256 samples.
#include "wem_elastic.cuh"

namespace gbwem {
template int ewem_launch_n<256>(int, int, const EwemArgs *, int, int, cudaStream_t, int *, size_t *);
}  // namespace gbwem
