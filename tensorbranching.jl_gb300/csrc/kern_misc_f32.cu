// misc kernels of the engine for float: explicit instantiations of the
// launch wrappers in device_kernels.cuh.
#include "device_kernels.cuh"

namespace tb {

template cudaError_t launch_leaves<float>(unsigned, cudaStream_t, const LeafDesc*, int, const int8_t*, float*, const float*);
template cudaError_t launch_tile<float>(unsigned, int, cudaStream_t, const TileDesc&, float*, int64_t);
template cudaError_t launch_final<float>(cudaStream_t, const FinalDesc&, const float*, float, float*);
template cudaError_t launch_small<float>(unsigned, int, cudaStream_t, const ItemDev<float>*, const int32_t*, int,
                                             float*, const float*);
template cudaError_t launch_k1_any<float>(const float*, const float*, float*, int64_t, int64_t, int64_t, int64_t,
                                           cudaStream_t);

}  // namespace tb
