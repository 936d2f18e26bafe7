// tb_solve_static: one MIS contraction with no device allocation.
//
// Some callers cannot allocate GPU memory: code that runs inside another
// runtime's memory pool or allocator hooks, a host process that is only
// handed a stream, or a context where cudaMalloc is forbidden while a graph or
// a real-time loop is running.  For them this entry point keeps every device
// byte it needs -- the tensor arena, the leaf descriptors and the result -- in
// one file-scope __device__ array of fixed size (kStaticScratchBytes), which
// every GPU that loads the library holds until the process exits.  Calls
// larger than that are refused with TB_ERR_UNSUPPORTED.
//
// The contraction follows the plain path: the leaf builder, then per
// contraction node the permute kernels and the batched max-plus GEMM (K1) of
// kernels.cuh, then the max over the root tensor; everything is enqueued on
// the caller's stream and the call returns after the result is on the host.
//
// Set-up: the first call on a device looks up the array's device address with
// cudaGetSymbolAddress, with that device current, and caches it; make that
// first call before any stream capture begins.  Every call shares the array
// and leaves its contents behind: every tensor a call reads is written by
// the same call first, so nothing needs clearing; calls that overlap on the
// GPU (two streams, or two host threads) race on the array and must be
// serialised by the caller.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/tb.h"
#include "kernels.cuh"
#include "launch.h"
#include "plan.h"

namespace tb {
void set_last_error(const std::string& msg);  // engine.cu
}

using namespace tb;

namespace {

constexpr size_t kStaticScratchBytes = size_t(64) << 20;  // 64 MiB per device
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

std::mutex g_static_mu;
void* g_static_ptr[kMaxDevices] = {nullptr};

tb_status sfail(tb_status s, const std::string& m) {
  tb::set_last_error(m);  // read back with tb_last_error(NULL)
  return s;
}

#define SCU(x)                                                                         \
  do {                                                                                 \
    cudaError_t e_ = (x);                                                              \
    if (e_ != cudaSuccess) return sfail(TB_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
  } while (0)

__global__ void __launch_bounds__(kThreads) ks_leaves(const LeafDesc* leaves, int n, const int8_t* sv, float* arena) {
  leaves_tile<float>(leaves, n, sv, arena, blockIdx.x, nullptr);
}

__global__ void __launch_bounds__(kThreads) ks_tile(const TileDesc d, float* arena) {
  extern __shared__ int ks_smem[];
  stream_tile<float>(d, blockIdx.x, arena, ks_smem);
}

__global__ void __launch_bounds__(kThreads) ks_final(const FinalDesc f, const float* arena, float* out) {
  final_tile<float>(f, arena, 0.0f, out);
}

template <int BM, int BN>
cudaError_t ks_k1(const float* A, const float* B, float* C, int64_t M, int64_t N, int64_t K, int64_t batch,
                  cudaStream_t s) {
  using Cfg = K1Cfg<float, BM, BN>;
  cudaError_t e = smem_optin(reinterpret_cast<const void*>(gemm_k1<float, BM, BN>), Cfg::SMEM_BYTES);
  if (e != cudaSuccess) return e;
  int64_t tiles_mn = (M / BM) * (N / BN);
  int64_t grid = tiles_mn * batch;
  if (grid > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  gemm_k1<float, BM, BN><<<(unsigned)grid, 256, Cfg::SMEM_BYTES, s>>>(A, B, C, (int)M, (int)N, (int)K, tiles_mn);
  return cudaGetLastError();
}

cudaError_t ks_gemm(const float* A, const float* B, float* C, int64_t M, int64_t N, int64_t K, int64_t batch,
                    cudaStream_t s) {
  int bm = M >= 128 ? 128 : M >= 64 ? 64 : M >= 32 ? 32 : 16;
  int bn = N >= 128 ? 128 : N >= 64 ? 64 : N >= 32 ? 32 : 16;
#define KS_CASE(X, Y) \
  if (bm == X && bn == Y) return ks_k1<X, Y>(A, B, C, M, N, K, batch, s);
  KS_CASE(128, 128) KS_CASE(128, 64) KS_CASE(128, 32) KS_CASE(128, 16)
  KS_CASE(64, 128) KS_CASE(64, 64) KS_CASE(64, 32) KS_CASE(64, 16)
  KS_CASE(32, 128) KS_CASE(32, 64) KS_CASE(32, 32) KS_CASE(32, 16)
  KS_CASE(16, 128) KS_CASE(16, 64) KS_CASE(16, 32) KS_CASE(16, 16)
#undef KS_CASE
  return cudaErrorInvalidValue;
}

// Device address of the static array on the current device (set-up once).
tb_status static_scratch(void** out) {
  int dev = 0;
  SCU(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return sfail(TB_ERR_UNSUPPORTED, "device ordinal out of range");
  std::lock_guard<std::mutex> lk(g_static_mu);
  if (!g_static_ptr[dev]) {
    void* p = nullptr;
    SCU(cudaGetSymbolAddress(&p, g_static_scratch));
    g_static_ptr[dev] = p;
  }
  *out = g_static_ptr[dev];
  return TB_OK;
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

extern "C" tb_status tb_solve_static(int32_t n_labels, int32_t n_tensors, const int32_t* ix_off,
                                     const int32_t* ix_lab, int32_t n_nodes, const int32_t* children,
                                     const float* weights, float* out_value, void* stream) {
  if (!ix_off || !ix_lab || !weights || !out_value || (n_nodes > 0 && !children))
    return sfail(TB_ERR_INVALID, "null argument");
  PlanInput in;
  in.n_labels = n_labels;
  in.n_tensors = n_tensors;
  in.ix_off = ix_off;
  in.ix_lab = ix_lab;
  in.n_nodes = n_nodes;
  in.children = children;
  PlanHost h;
  std::string e;
  try {
    e = compile_plan(in, h, 0);
  } catch (const std::exception& ex) {
    e = ex.what();
  }
  if (!e.empty()) return sfail(TB_ERR_INVALID, e);
  for (int i = 0; i < h.n_tensors; i++) {
    LeafDesc& ld = h.leaves[i];
    if (ld.nraw < 1 || ld.nraw > 2)
      return sfail(TB_ERR_INVALID, "independent-set leaves have one (vertex) or two (edge) labels");
    if (ld.nraw == 1) {
      float x = weights[h.leaf_raw[i][0]];
      if (!std::isfinite(x)) return sfail(TB_ERR_INVALID, "weights must be finite");
      ld.w = x;
    }
  }
  // layout of the static array: arena | leaf descriptors | result
  const size_t arena_bytes = align256((size_t)h.plain_elems * sizeof(float));
  const size_t leaf_bytes = align256(h.leaves.size() * sizeof(LeafDesc));
  const size_t need = arena_bytes + leaf_bytes + 256;
  if (need > kStaticScratchBytes)
    return sfail(TB_ERR_UNSUPPORTED, "network needs " + std::to_string(need) +
                                         " bytes of device scratch; tb_solve_static holds " +
                                         std::to_string(kStaticScratchBytes) + " bytes (use tb_solve_batch)");
  void* base = nullptr;
  tb_status st = static_scratch(&base);
  if (st) return st;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  char* b = static_cast<char*>(base);
  float* arena = reinterpret_cast<float*>(b);
  LeafDesc* d_leaves = reinterpret_cast<LeafDesc*>(b + arena_bytes);
  float* d_out = reinterpret_cast<float*>(b + arena_bytes + leaf_bytes);
  SCU(cudaMemcpyAsync(d_leaves, h.leaves.data(), h.leaves.size() * sizeof(LeafDesc), cudaMemcpyHostToDevice, s));
  // every stream tile the plan compiler emits fits stream_smem_words_max()
  SCU(smem_optin(reinterpret_cast<const void*>(ks_tile), stream_smem_words_max() * 4));
  ks_leaves<<<(h.n_tensors + kThreads - 1) / kThreads, kThreads, 0, s>>>(d_leaves, h.n_tensors, nullptr, arena);
  SCU(cudaGetLastError());
  if (h.n_nodes == 0) {
    const TileDesc& d = h.tiles[0];
    ks_tile<<<d.n_tiles, kThreads, stream_smem_words(d) * 4, s>>>(d, arena);
    SCU(cudaGetLastError());
  }
  for (int j = 0; j < h.n_nodes; j++) {
    for (const PlainOp& op : h.plain[j]) {
      if (op.kind == PLAIN_TILE) {
        ks_tile<<<op.tile.n_tiles, kThreads, stream_smem_words(op.tile) * 4, s>>>(op.tile, arena);
        SCU(cudaGetLastError());
      } else {
        SCU(ks_gemm(arena + op.a_off, arena + op.b_off, arena + op.c_off, op.M, op.N, op.K, op.batch, s));
      }
    }
  }
  ks_final<<<1, kThreads, 0, s>>>(h.fin, arena, d_out);
  SCU(cudaGetLastError());
  SCU(cudaMemcpyAsync(out_value, d_out, sizeof(float), cudaMemcpyDeviceToHost, s));
  SCU(cudaStreamSynchronize(s));
  return TB_OK;
}
