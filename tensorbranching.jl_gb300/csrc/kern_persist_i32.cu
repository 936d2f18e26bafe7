// persist kernels of the engine for int32_t: explicit instantiations of the
// launch wrappers in device_kernels.cuh.
#include "device_kernels.cuh"

namespace tb {

template cudaError_t launch_persistent<int32_t>(unsigned, int, cudaStream_t, const ItemDev<int32_t>*, const Group*, const Chunk*,
                                              int64_t, int*, unsigned long long*, int*, float*, const float*, int64_t);
template cudaError_t occupancy_persistent<int32_t>(int*, int);

}  // namespace tb
