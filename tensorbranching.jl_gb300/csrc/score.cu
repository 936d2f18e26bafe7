// Scoring many contraction trees of one network on the device: the space,
// time and read-write complexity and the peak memory of a post-order
// evaluation of each tree (contraction_complexity as used at
// src/types.jl:115-121 and src/branch.jl:132-147, contraction_peak_memory
// src/utils.jl:197-219), the step before the contraction when a slicer
// compares candidate trees.
//
// One warp per tree.  Label sets are bitsets of W 32-bit words.  A
// bottom-up pass forms U(x), the labels of the leaves under x; a top-down
// pass forms O(x), the labels needed outside x (the open labels at the
// root, then O(parent) | U(sibling)); the output labels of x are
// S(x) = U(x) & O(x) (leaves keep their own labels).  Node n with children
// a, b then has |L(n)| = |S(a) | S(b)| and tensor size 2^|S(n)|.
#include <cuda_runtime.h>
#include <stdint.h>

#include "launch.h"

namespace tb {

namespace {

__device__ __forceinline__ double exp2i(int k) { return ldexp(1.0, k); }

__global__ void __launch_bounds__(256) k_score_trees(int n_trees, int T, int W, const uint32_t* __restrict__ leaf_bits,
                                                     const uint32_t* __restrict__ iy_bits,
                                                     const int32_t* __restrict__ children, uint32_t* __restrict__ scratch,
                                                     double* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int n_warps = (gridDim.x * blockDim.x) >> 5;
  const int nn = 2 * T - 1, nodes = T - 1;
  const size_t per_warp = (size_t)2 * nn * W + nn;
  uint32_t* U = scratch + (size_t)warp * per_warp;
  uint32_t* O = U + (size_t)nn * W;
  int32_t* sz = reinterpret_cast<int32_t*>(O + (size_t)nn * W);
  for (int tr = warp; tr < n_trees; tr += n_warps) {
    const int32_t* ch = children + (size_t)tr * 2 * nodes;
    // leaves
    for (int i = 0; i < T; i++) {
      int c = 0;
      for (int k = lane; k < W; k += 32) {
        const uint32_t v = leaf_bits[(size_t)i * W + k];
        U[(size_t)i * W + k] = v;
        c += __popc(v);
      }
      for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
      if (lane == 0) sz[i] = c;
    }
    // bottom-up unions (post-order: children precede parents)
    for (int j = 0; j < nodes; j++) {
      const int a = ch[2 * j], b = ch[2 * j + 1], n = T + j;
      for (int k = lane; k < W; k += 32) U[(size_t)n * W + k] = U[(size_t)a * W + k] | U[(size_t)b * W + k];
      __syncwarp();
    }
    // top-down outside sets, output sizes and per-node costs
    double tc = 0.0, rw = 0.0;
    int sc = 0;
    for (int i = 0; i < T; i++) sc = max(sc, sz[i]);
    const int root = nn - 1;
    if (nodes > 0) {
      for (int k = lane; k < W; k += 32) O[(size_t)root * W + k] = iy_bits[k];
      __syncwarp();
    }
    for (int j = nodes - 1; j >= 0; j--) {
      const int a = ch[2 * j], b = ch[2 * j + 1], n = T + j;
      int cn = 0, ca = 0, cb = 0, cl = 0;
      for (int k = lane; k < W; k += 32) {
        const uint32_t on = O[(size_t)n * W + k];
        const uint32_t ua = U[(size_t)a * W + k], ub = U[(size_t)b * W + k];
        const uint32_t oa = on | ub, ob = on | ua;
        if (a >= T) O[(size_t)a * W + k] = oa;
        if (b >= T) O[(size_t)b * W + k] = ob;
        const uint32_t sa = a >= T ? ua & oa : ua;  // a leaf keeps its labels
        const uint32_t sb = b >= T ? ub & ob : ub;
        cn += __popc(U[(size_t)n * W + k] & on);
        ca += __popc(sa);
        cb += __popc(sb);
        cl += __popc(sa | sb);
      }
      for (int o = 16; o > 0; o >>= 1) {
        cn += __shfl_xor_sync(0xffffffffu, cn, o);
        ca += __shfl_xor_sync(0xffffffffu, ca, o);
        cb += __shfl_xor_sync(0xffffffffu, cb, o);
        cl += __shfl_xor_sync(0xffffffffu, cl, o);
      }
      if (lane == 0) {
        sz[n] = cn;
        tc += exp2i(cl);
        rw += exp2i(ca) + exp2i(cb) + exp2i(cn);
      }
      sc = max(sc, cn);
      __syncwarp();
    }
    if (lane == 0) {
      // post-order evaluation: every leaf live at the start, each step
      // allocates its output and frees its operands
      double cur = 0.0;
      for (int i = 0; i < T; i++) cur += exp2i(sz[i]);
      double peak = cur;
      for (int j = 0; j < nodes; j++) {
        cur += exp2i(sz[T + j]) - exp2i(sz[ch[2 * j]]) - exp2i(sz[ch[2 * j + 1]]);
        peak = fmax(peak, cur);
      }
      double* o = out + (size_t)tr * 4;
      o[0] = nodes > 0 ? log2(tc) : (double)sz[0];
      o[1] = (double)sc;
      o[2] = nodes > 0 ? log2(rw) : (double)sz[0];
      o[3] = log2(peak);
    }
    __syncwarp();
  }
}

}  // namespace

cudaError_t launch_score_trees(int warps, cudaStream_t s, int n_trees, int T, int W, const uint32_t* leaf_bits,
                               const uint32_t* iy_bits, const int32_t* children, uint32_t* scratch, double* out) {
  const int blocks = (warps + 7) / 8;
  k_score_trees<<<blocks, 256, 0, s>>>(n_trees, T, W, leaf_bits, iy_bits, children, scratch, out);
  return cudaGetLastError();
}

}  // namespace tb
