// Kernels of the engine: thin __global__ wrappers over the device routines
// of kernels.cuh, and the host-side launch wrappers of launch.h.  Each
// kern_*.cu translation unit instantiates a share of them so the device code
// compiles in parallel.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>

#include "../../include/tb.h"
#include "kernels.cuh"
#include "launch.h"

namespace tb {

// ---------------------------------------------------------------------------
// kernels (thin __global__ wrappers over the device routines)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(kThreads) k_leaves(const LeafDesc* leaves, int n, const int8_t* sv, T* arena,
                                                     const float* w) {
  leaves_tile<T>(leaves, n, sv, arena, blockIdx.x, w);
}

// A stream-tile node: CTA b runs tiles [b * chunk, (b + 1) * chunk).
template <typename T>
__global__ void __launch_bounds__(kThreads, 2) k_tile(const TileDesc d, T* arena, int64_t chunk) {
  extern __shared__ int tb_smem[];
  const int64_t t0 = (int64_t)blockIdx.x * chunk;
  const int64_t t1 = t0 + chunk < d.n_tiles ? t0 + chunk : d.n_tiles;
  stream_tiles<T, true>(d, t0, t1, arena, tb_smem);
}

template <typename T>
__global__ void __launch_bounds__(kThreads) k_final(const FinalDesc f, const T* arena, float r, float* out) {
  final_tile<T>(f, arena, r, out);
}

// Leaves and final steps (stream and GEMM steps run as runs of tiles).
template <typename T>
__device__ __forceinline__ void run_small_step(const ItemDev<T>& it, const Step& st, int64_t tile, float* out_item,
                                               const float* r, int item) {
  if (st.kind == STEP_LEAVES) leaves_tile<T>(it.leaves, it.n_leaves, it.slice_vals, it.arena, (int)tile, it.w);
  else if (st.kind == STEP_FINAL) final_tile<T>(it.fin, it.arena, r ? r[item] : 0.0f, out_item + item);
  else if (st.kind == STEP_FILL && (it.flags & 2)) fill_tile<T>(it.gemms[st.desc], it.arena, tile);
  // STEP_FILL without bit 1 and STEP_KRED with it have nothing to do
}

__device__ __forceinline__ int find_group(const Group* groups, int n_groups, int64_t tk) {
  int lo = 0, hi = n_groups - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (groups[mid].first <= tk) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// One launch per tree level: block b runs ticket first_ticket + b.  No
// waiting: the previous launch on the stream finished every dependency.
// KINDS bit 0: stream-like steps, bit 1: GEMM steps; 5 is the stream form
// with two resident CTAs per SM (128 registers a thread instead of 80),
// which the autotuner may choose.
template <typename T, int KINDS>
__global__ void __launch_bounds__(kThreads, KINDS == 1 ? 3 : 2) k_level(const ItemDev<T>* items, const Group* groups, int n_groups,
                                                   const LevelSpan span, float* out_item, const float* r, int* err) {
  extern __shared__ int tb_smem[];
  __shared__ int s_g;
  {
    // CTA b runs one run of tickets of this level (LevelSpan), a run of
    // tiles per group: each stream tile builds its tables once, each GEMM run
    // keeps one copy pipeline across its tiles
    const int b = (int)blockIdx.x;
    int64_t tk, end;
    if (b < span.split_cta) {
      tk = span.first + (int64_t)b * span.chunk;
      end = tk + span.chunk < span.mid ? tk + span.chunk : span.mid;
    } else {
      tk = span.mid + (int64_t)(b - span.split_cta) * span.chunk2;
      end = tk + span.chunk2 < span.last ? tk + span.chunk2 : span.last;
    }
    // launched with programmatic stream serialization (launch_level): the
    // next level may launch once every CTA of this one has started; each
    // path below waits for the previous grid's completion (dep_wait) before
    // its first access to the arena or the outputs, after the setup that
    // reads only host-written groups and descriptors
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    if (tk >= end) return;
    // the first group by binary search, then the following ones in order
    // (the index lives in shared memory, not across the tile code's registers)
    if (threadIdx.x == 0) s_g = find_group(groups, n_groups, tk);
    __syncthreads();
    while (tk < end) {
      const int gi = s_g;
      const Group& g = groups[gi];
      int next = gi + 1;
      if ((KINDS & 1) && g.tiny) {
        // a run of tiny steps (one tile, so one ticket, each; listed first
        // in their level) up to the CTA's last ticket or the level's last
        // tiny step: warp w takes the run's steps w, w + 8, ...
        const int n = (int)(g.run < end - tk ? g.run : end - tk);
        dep_wait();
        for (int q = threadIdx.x >> 5; q < n; q += kThreads / 32) {
          const Group& gq = groups[gi + q];
          tiny_node<T>(gq.tile, reinterpret_cast<T*>(gq.arena));
        }
        next = gi + n;
        tk = next < n_groups && groups[next].first < end ? groups[next].first : end;
      } else {
        const int64_t g_end = gi + 1 < n_groups && groups[gi + 1].first < end ? groups[gi + 1].first : end;
        const ItemDev<T>& it = items[g.item];
        const Step& st = it.steps[g.step];
        const int64_t g_first = g.first;
        if ((KINDS & 1) && (st.kind == STEP_TILE || (st.kind == STEP_KRED && !(it.flags & 2)))) {
          stream_tiles<T, KINDS == 5>(it.tiles[st.desc], tk - g_first, g_end - g_first, it.arena, tb_smem, err);
        } else if ((KINDS & 2) && st.kind == STEP_GEMM) {
          // a timed-out copy wait (err set) may leave copies in flight into
          // this CTA's shared memory: use it no further
          if (!gemm_tiles_any<T>(it.gemms[st.desc], tk - g_first, g_end - g_first, it.arena, tb_smem, err,
                                 (it.flags & 1) != 0, (it.flags & 2) != 0))
            return;
        } else {
          dep_wait();
          for (int64_t x = tk; x < g_end; x++) run_small_step<T>(it, st, x - g_first, out_item, r, g.item);
        }
        tk = g_end;
      }
      __syncthreads();  // every thread has read s_g
      if (threadIdx.x == 0) s_g = next;
      __syncthreads();
    }
  }
}

// Persistent executor.  Chunks of tiles are handed out in dependency order,
// so a chunk only waits on chunks already held by running CTAs; every wait is
// bounded by timeout_ns and ends with err set instead of hanging.
template <typename T>
__global__ void __launch_bounds__(kThreads, 2) k_persistent(const ItemDev<T>* items, const Group* groups,
                                                           const Chunk* chunks, int64_t n_chunks, int* done,
                                                           unsigned long long* ticket, int* err, float* out_item,
                                                           const float* r, int64_t timeout_ns) {
  extern __shared__ int tb_smem[];
  __shared__ long long s_c;
  __shared__ int s_stop;
  for (;;) {
    if (threadIdx.x == 0) {
      long long c = (long long)atomicAdd(ticket, 1ull);
      int stop = (c >= n_chunks) || (*(volatile int*)err != 0);
      if (!stop) {
        const Group g = groups[chunks[c].group];
        const ItemDev<T>& it = items[g.item];
        const Step st = it.steps[g.step];
        const int deps[2] = {st.dep0, st.dep1};
        uint64_t t0 = globaltimer();
        for (int d = 0; d < 2 && !stop; d++) {
          if (deps[d] < 0) continue;
          const int need = it.steps[deps[d]].n_tiles;
          const int* cnt = done + it.done_base + deps[d];
          while (ld_acquire(cnt) < need) {
            if (*(volatile int*)err != 0) { stop = 1; break; }
            if (globaltimer() - t0 > (uint64_t)timeout_ns) {
              atomicExch(err, TB_ERR_TIMEOUT);
              stop = 1;
              break;
            }
            __nanosleep(128);
          }
        }
      }
      s_c = c;
      s_stop = stop;
    }
    __syncthreads();
    if (s_stop) break;
    const Chunk ch = chunks[s_c];
    const Group g = groups[ch.group];
    const ItemDev<T>& it = items[g.item];
    const Step& st = it.steps[g.step];
    if (st.kind == STEP_TILE || (st.kind == STEP_KRED && !(it.flags & 2))) {
      stream_tiles<T, false>(it.tiles[st.desc], ch.t0, ch.t1, it.arena, tb_smem, err);
    } else if (st.kind == STEP_GEMM) {
      if (!gemm_tiles_any<T>(it.gemms[st.desc], ch.t0, ch.t1, it.arena, tb_smem, err, (it.flags & 1) != 0,
                             (it.flags & 2) != 0))
        return;  // err is set; copies may still be landing in this CTA's shared memory
    } else {
      for (int64_t x = ch.t0; x < ch.t1; x++) run_small_step<T>(it, st, x, out_item, r, g.item);
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(done + it.done_base + g.step, (int)(ch.t1 - ch.t0));
  }
}

// Fused small form: block b contracts item order[b]'s whole network in
// shared memory (leaves, every node in post-order with a block barrier
// between nodes, the root max) and writes one value.  Node j: thread t
// computes outputs o = t, t + kSmallThreads, ...; the addresses of A and B
// follow from the bits of o (and of the reduced index k) through the node's
// 4-bit label positions.
__device__ __forceinline__ int small_stride(uint32_t p0, uint32_t p1, int i) {
  const uint32_t q = ((i < 8 ? p0 : p1) >> (4 * (i & 7))) & 15u;
  return (int)((1u << q) & 0x7fffu);  // position 15: not in this operand
}

template <typename T>
__global__ void __launch_bounds__(kSmallThreads) k_small(const ItemDev<T>* items, const int32_t* order, int n_items,
                                                         float* out_item, const float* r) {
  extern __shared__ int tb_smem[];
  __shared__ float s_max[kSmallThreads / 32];
  T* sm = reinterpret_cast<T*>(tb_smem);
  const int tid = threadIdx.x;
  if ((int)blockIdx.x >= n_items) return;
  const int item = order[blockIdx.x];
  const ItemDev<T>& it = items[item];
  for (int i = tid; i < it.n_leaves; i += kSmallThreads) {
    const LeafDesc ld = it.leaves[i];
    const T w = Trop<T>::from_w(it.w && ld.label >= 0 ? it.w[ld.label] : ld.w);
    T* dst = sm + it.small_leaf[i];
    for (int e = 0; e < (1 << ld.n_out); e++) {
      T best = Trop<T>::neg();
      for (int raw = 0; raw < (1 << ld.nraw); raw++) {
        bool ok = true;
        for (int k = 0; k < ld.nraw; k++) {
          const int x = (raw >> k) & 1;
          if (ld.slice_idx[k] >= 0) {
            if (x != (int)it.slice_vals[ld.slice_idx[k]]) ok = false;
          } else if (((e >> ld.out_bit[k]) & 1) != x) {
            ok = false;
          }
        }
        if (!ok) continue;
        const T v = ld.nraw == 1 ? ((raw & 1) ? w : T(0)) : (raw == 3 ? Trop<T>::neg() : T(0));
        best = Trop<T>::mx(best, v);
      }
      dst[e] = best;
    }
  }
  __syncthreads();
  // node records come from global memory (L1/L2); the next one is loaded
  // while this one runs
  SmallNode nxt;
  if (it.n_small > 0) nxt = it.small[0];
  for (int j = 0; j < it.n_small; j++) {
    const SmallNode nd = nxt;
    if (j + 1 < it.n_small) nxt = it.small[j + 1];
    const int nc = nd.nc_nk & 0xff, nk = (nd.nc_nk >> 8) & 0xff;
    const T* A = sm + nd.a_off;
    const T* B = sm + nd.b_off;
    T* C = sm + nd.c_off;
    for (int o = tid; o < (1 << nc); o += kSmallThreads) {
      int ao = 0, bo = 0;
      for (int i = 0; i < nc; i++) {
        if ((o >> i) & 1) {
          ao += small_stride(nd.pa[0], nd.pa[1], i);
          bo += small_stride(nd.pb[0], nd.pb[1], i);
        }
      }
      T acc = Trop<T>::neg();
      for (int k = 0; k < (1 << nk); k++) {
        int ak = ao, bk = bo;
        for (int i = 0; i < nk; i++) {
          if ((k >> i) & 1) {
            ak += small_stride(nd.pa[0], nd.pa[1], nc + i);
            bk += small_stride(nd.pb[0], nd.pb[1], nc + i);
          }
        }
        acc = Trop<T>::mac(acc, A[ak], B[bk]);
      }
      C[o] = acc;
    }
    __syncthreads();
  }
  T m = Trop<T>::neg();
  for (int i = tid; i < (1 << it.small_root_log2); i += kSmallThreads) m = Trop<T>::mx(m, sm[it.small_root + i]);
  float v = Trop<T>::to_f(m);
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((tid & 31) == 0) s_max[tid >> 5] = v;
  __syncthreads();
  if (tid == 0) {
    float b = s_max[0];
    for (int w = 1; w < kSmallThreads / 32; w++) b = fmaxf(b, s_max[w]);
    out_item[item] = b + (r ? r[item] : 0.0f);
  }
}

template <typename T, int BM, int BN>
inline cudaError_t launch_k1(const T* A, const T* B, T* C, int64_t M, int64_t N, int64_t K, int64_t batch,
                             cudaStream_t s) {
  using Cfg = K1Cfg<T, BM, BN>;
  cudaError_t e = smem_optin(reinterpret_cast<const void*>(gemm_k1<T, BM, BN>), Cfg::SMEM_BYTES);
  if (e != cudaSuccess) return e;
  int64_t tiles_mn = (M / BM) * (N / BN);
  int64_t grid = tiles_mn * batch;
  if (grid > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  gemm_k1<T, BM, BN><<<(unsigned)grid, 256, Cfg::SMEM_BYTES, s>>>(A, B, C, (int)M, (int)N, (int)K, tiles_mn);
  return cudaGetLastError();
}

template <typename T>
inline cudaError_t dispatch_k1(const T* A, const T* B, T* C, int64_t M, int64_t N, int64_t K, int64_t batch,
                               cudaStream_t s) {
  int bm = M >= 128 ? 128 : M >= 64 ? 64 : M >= 32 ? 32 : 16;
  int bn = N >= 128 ? 128 : N >= 64 ? 64 : N >= 32 ? 32 : 16;
#define K1_CASE(X, Y) \
  if (bm == X && bn == Y) return launch_k1<T, X, Y>(A, B, C, M, N, K, batch, s);
  K1_CASE(128, 128) K1_CASE(128, 64) K1_CASE(128, 32) K1_CASE(128, 16)
  K1_CASE(64, 128) K1_CASE(64, 64) K1_CASE(64, 32) K1_CASE(64, 16)
  K1_CASE(32, 128) K1_CASE(32, 64) K1_CASE(32, 32) K1_CASE(32, 16)
  K1_CASE(16, 128) K1_CASE(16, 64) K1_CASE(16, 32) K1_CASE(16, 16)
#undef K1_CASE
  return cudaErrorInvalidValue;
}


// ---------------------------------------------------------------------------
// launch wrappers (declared in launch.h)
// ---------------------------------------------------------------------------
template <typename T>
cudaError_t launch_small(unsigned grid, int smem, cudaStream_t s, const ItemDev<T>* items, const int32_t* order,
                         int n, float* out_item, const float* r) {
  cudaError_t e = smem_optin(reinterpret_cast<const void*>(k_small<T>), smem);
  if (e != cudaSuccess) return e;
  k_small<T><<<grid, kSmallThreads, smem, s>>>(items, order, n, out_item, r);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_leaves(unsigned grid, cudaStream_t s, const LeafDesc* leaves, int n, const int8_t* sv, T* arena,
                          const float* w) {
  k_leaves<T><<<grid, kThreads, 0, s>>>(leaves, n, sv, arena, w);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_tile(unsigned grid, int smem, cudaStream_t s, const TileDesc& d, T* arena, int64_t chunk) {
  cudaError_t e = smem_optin(reinterpret_cast<const void*>(k_tile<T>), stream_smem_words_max() * 4);
  if (e != cudaSuccess) return e;
  k_tile<T><<<grid, kThreads, smem, s>>>(d, arena, chunk);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_final(cudaStream_t s, const FinalDesc& f, const T* arena, float r, float* out) {
  k_final<T><<<1, kThreads, 0, s>>>(f, arena, r, out);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_k1_any(const T* A, const T* B, T* C, int64_t M, int64_t N, int64_t K, int64_t batch,
                          cudaStream_t s) {
  return dispatch_k1<T>(A, B, C, M, N, K, batch, s);
}

template <typename T, int KINDS>
static cudaError_t level_attr(int smem) {
  return smem_optin(reinterpret_cast<const void*>(k_level<T, KINDS>), smem);
}

template <typename T, int KINDS>
cudaError_t launch_level(unsigned grid, int smem, cudaStream_t s, const ItemDev<T>* items, const Group* groups,
                         int n_groups, const LevelSpan& span, float* out_item, const float* r, int* err) {
  cudaError_t e = level_attr<T, KINDS>(smem);
  if (e != cudaSuccess) return e;
  // programmatic dependent launch: this level's CTAs may start (and find
  // their first group) while the previous level drains; k_level waits on
  // the previous grid before it touches the arena
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kThreads);
  cfg.dynamicSmemBytes = (size_t)smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  e = cudaLaunchKernelEx(&cfg, k_level<T, KINDS>, items, groups, n_groups, span, out_item, r, err);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

template <typename T, int KINDS>
cudaError_t occupancy_level(int* per_sm, int smem) {
  cudaError_t e = level_attr<T, KINDS>(smem);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_level<T, KINDS>, kThreads, smem);
}

template <typename T>
static cudaError_t persistent_attr(int smem) {
  return smem_optin(reinterpret_cast<const void*>(k_persistent<T>), smem);
}

template <typename T>
cudaError_t launch_persistent(unsigned ctas, int smem, cudaStream_t s, const ItemDev<T>* items, const Group* groups,
                              const Chunk* chunks, int64_t n_chunks, int* done, unsigned long long* ticket, int* err,
                              float* out_item, const float* r, int64_t timeout_ns) {
  cudaError_t e = persistent_attr<T>(smem);
  if (e != cudaSuccess) return e;
  k_persistent<T><<<ctas, kThreads, smem, s>>>(items, groups, chunks, n_chunks, done, ticket, err, out_item, r,
                                               timeout_ns);
  return cudaGetLastError();
}

template <typename T>
cudaError_t occupancy_persistent(int* per_sm, int smem) {
  cudaError_t e = persistent_attr<T>(smem);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_persistent<T>, kThreads, smem);
}

}  // namespace tb
