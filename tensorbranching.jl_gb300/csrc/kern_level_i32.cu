// level kernels of the engine for int32_t: explicit instantiations of the
// launch wrappers in device_kernels.cuh.
#include "device_kernels.cuh"

namespace tb {

template cudaError_t launch_level<int32_t, 1>(unsigned, int, cudaStream_t, const ItemDev<int32_t>*, const Group*, int,
                                             const LevelSpan&, float*, const float*, int*);
template cudaError_t occupancy_level<int32_t, 1>(int*, int);
template cudaError_t launch_level<int32_t, 2>(unsigned, int, cudaStream_t, const ItemDev<int32_t>*, const Group*, int,
                                             const LevelSpan&, float*, const float*, int*);
template cudaError_t occupancy_level<int32_t, 2>(int*, int);
template cudaError_t launch_level<int32_t, 5>(unsigned, int, cudaStream_t, const ItemDev<int32_t>*, const Group*, int,
                                             const LevelSpan&, float*, const float*, int*);
template cudaError_t occupancy_level<int32_t, 5>(int*, int);

}  // namespace tb
