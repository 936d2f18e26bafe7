// persist kernels of the engine for float: explicit instantiations of the
// launch wrappers in device_kernels.cuh.
#include "device_kernels.cuh"

namespace tb {

template cudaError_t launch_persistent<float>(unsigned, int, cudaStream_t, const ItemDev<float>*, const Group*, const Chunk*,
                                              int64_t, int*, unsigned long long*, int*, float*, const float*, int64_t);
template cudaError_t occupancy_persistent<float>(int*, int);

}  // namespace tb
