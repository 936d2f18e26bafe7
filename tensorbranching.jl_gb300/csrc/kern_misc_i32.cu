// misc kernels of the engine for int32_t: explicit instantiations of the
// launch wrappers in device_kernels.cuh.
#include "device_kernels.cuh"

namespace tb {

template cudaError_t launch_leaves<int32_t>(unsigned, cudaStream_t, const LeafDesc*, int, const int8_t*, int32_t*, const float*);
template cudaError_t launch_tile<int32_t>(unsigned, int, cudaStream_t, const TileDesc&, int32_t*, int64_t);
template cudaError_t launch_final<int32_t>(cudaStream_t, const FinalDesc&, const int32_t*, float, float*);
template cudaError_t launch_small<int32_t>(unsigned, int, cudaStream_t, const ItemDev<int32_t>*, const int32_t*, int,
                                             float*, const float*);
template cudaError_t launch_k1_any<int32_t>(const int32_t*, const int32_t*, int32_t*, int64_t, int64_t, int64_t, int64_t,
                                           cudaStream_t);

}  // namespace tb
