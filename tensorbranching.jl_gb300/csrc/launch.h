// Host-side launch wrappers of the engine's kernels.  They are defined in
// device_kernels.cuh and instantiated for f32 and int32 by the kern_*.cu
// translation units, so the host code of engine.cu compiles without the
// device code.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "tb_internal.h"

namespace tb {

// Opt kernel `fn` in to `bytes` of dynamic shared memory on the current
// device.  The attribute is per device, so the state is kept per (kernel,
// device) and raised when a launch asks for more; thread-safe (engine.cu).
cudaError_t smem_optin(const void* fn, int bytes);

template <typename T>
cudaError_t launch_leaves(unsigned grid, cudaStream_t s, const LeafDesc* leaves, int n, const int8_t* sv, T* arena,
                          const float* w);
template <typename T>
cudaError_t launch_tile(unsigned grid, int smem, cudaStream_t s, const TileDesc& d, T* arena, int64_t chunk);
template <typename T>
cudaError_t launch_final(cudaStream_t s, const FinalDesc& f, const T* arena, float r, float* out);
// fused small form: one block per item; block b runs item order[b] (b < n)
template <typename T>
cudaError_t launch_small(unsigned grid, int smem, cudaStream_t s, const ItemDev<T>* items, const int32_t* order,
                         int n, float* out_item, const float* r);
template <typename T>
cudaError_t launch_k1_any(const T* A, const T* B, T* C, int64_t M, int64_t N, int64_t K, int64_t batch,
                          cudaStream_t s);
template <typename T, int KINDS>
cudaError_t launch_level(unsigned grid, int smem, cudaStream_t s, const ItemDev<T>* items, const Group* groups,
                         int n_groups, const LevelSpan& span, float* out_item, const float* r, int* err);
template <typename T, int KINDS>
cudaError_t occupancy_level(int* per_sm, int smem);
template <typename T>
cudaError_t launch_persistent(unsigned ctas, int smem, cudaStream_t s, const ItemDev<T>* items, const Group* groups,
                              const Chunk* chunks, int64_t n_chunks, int* done, unsigned long long* ticket, int* err,
                              float* out_item, const float* r, int64_t timeout_ns);
template <typename T>
cudaError_t occupancy_persistent(int* per_sm, int smem);

// Complexities and peak memory of many contraction trees of one network
// (csrc/score.cu): one warp per tree.
cudaError_t launch_score_trees(int warps, cudaStream_t s, int n_trees, int T, int W, const uint32_t* leaf_bits,
                               const uint32_t* iy_bits, const int32_t* children, uint32_t* scratch, double* out);

}  // namespace tb
