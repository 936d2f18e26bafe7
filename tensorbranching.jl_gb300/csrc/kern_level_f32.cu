// level kernels of the engine for float: explicit instantiations of the
// launch wrappers in device_kernels.cuh.
#include "device_kernels.cuh"

namespace tb {

template cudaError_t launch_level<float, 1>(unsigned, int, cudaStream_t, const ItemDev<float>*, const Group*, int,
                                             const LevelSpan&, float*, const float*, int*);
template cudaError_t occupancy_level<float, 1>(int*, int);
template cudaError_t launch_level<float, 2>(unsigned, int, cudaStream_t, const ItemDev<float>*, const Group*, int,
                                             const LevelSpan&, float*, const float*, int*);
template cudaError_t occupancy_level<float, 2>(int*, int);
template cudaError_t launch_level<float, 5>(unsigned, int, cudaStream_t, const ItemDev<float>*, const Group*, int,
                                             const LevelSpan&, float*, const float*, int*);
template cudaError_t occupancy_level<float, 5>(int*, int);

}  // namespace tb
