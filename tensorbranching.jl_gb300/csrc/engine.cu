// Engine: contexts, plans, execution modes and the C ABI of include/tb.h.
//
// Execution modes of tb_solve_batch (contract_slices, src/dynamic_ob.jl:36-48):
//   PLAIN    one item at a time; per contraction node the OMEinsum lowering
//            (permute kernels + K1 batched max-plus GEMM + permute), result
//            copied to the host after every item -- the reference's
//            one-contraction-at-a-time GPU loop, as a drop-in.
//   LAYERED  fused tile kernels, one launch per tree level covering every
//            item, captured in a CUDA graph.
//   BATCHED  one persistent launch: CTAs take tickets in dependency order
//            from a device work queue, wait (bounded) on per-step completion
//            counters, run fused tiles; captured in a CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <type_traits>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "../../include/tb.h"
#include "kernels.cuh"
#include "launch.h"
#include "plan.h"

using namespace tb;

// ---------------------------------------------------------------------------
// K4: max over per-item results (warp-shuffle tree).
__global__ void __launch_bounds__(kThreads) k_reduce_max(const float* v, int n, float* out) {
  __shared__ float wmax[kThreads / 32];
  float m = __int_as_float(0xff800000);
  for (int i = threadIdx.x; i < n; i += kThreads) m = fmaxf(m, v[i]);
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    float b = wmax[0];
    for (int w = 1; w < kThreads / 32; w++) b = fmaxf(b, wmax[w]);
    *out = b;
  }
}

// ---------------------------------------------------------------------------
// host objects
// ---------------------------------------------------------------------------
namespace {

thread_local std::string g_err;

struct DevBuf {
  void* p = nullptr;
  size_t n = 0;
  ~DevBuf() { if (p) cudaFree(p); }
  cudaError_t ensure(size_t bytes) {
    if (bytes <= n) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e == cudaSuccess) n = bytes;
    return e;
  }
};

struct HostBuf {
  void* p = nullptr;
  size_t n = 0;
  uint64_t gen = 0;  // bumps with every (re)allocation: the contents are gone
  ~HostBuf() { if (p) cudaFreeHost(p); }
  cudaError_t ensure(size_t bytes) {
    if (bytes <= n) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
    gen++;
    cudaError_t e = cudaMallocHost(&p, bytes);
    if (e == cudaSuccess) n = bytes;
    return e;
  }
};

}  // namespace

struct tb_plan {
  tb_ctx* ctx = nullptr;
  PlanHost h;
  std::vector<float> weights;  // bound vertex weights by label
  DevBuf d_steps, d_tiles, d_gemms, d_leaves, d_small, d_small_leaf;
  DevBuf d_steps_merged, d_gemms_merged;  // the split-K GEMMs merged (PlanHost::steps_merged)
  DevBuf d_tiny;                          // TinyDesc of each TileDesc (used for the tiny steps)
  bool structure_uploaded = false;
  bool leaves_dirty = false;   // LeafDesc::w on the device is older than the bound weights
  bool i16_ok = false;         // bound weights are integers >= 0 summing below 8192
  bool nonneg_ok = false;      // bound weights are >= 0: every tensor value is >= 0 or -inf
  bool mis_checked = false;    // leaves checked to be vertex / edge tensors
  std::vector<int> vertex_leaves;
  uint64_t version = 0;        // bumps when device buffers move
  bool vertex_dense = false;   // vertex leaf k has label k
  uint64_t seen_call = 0;      // last solve call that staged this plan's weights
  int64_t seen_off = 0;        // where that call staged them
  uint64_t wgen = 1;           // bumps when the bound weights change
  uint64_t staged_wgen = 0;    // the weights generation in the context's staging buffer
  uint64_t staged_epoch = 0;   // ... as of that staging epoch
};

// One launch of the fused small form: items small_order[first, first + count),
// each block asking for smem bytes.
struct SmallGroup {
  int first, count, smem;
};


struct GraphKey {
  std::vector<const tb_plan*> plans;
  std::vector<uint64_t> versions;
  int mode = 0;
  int sched = 0;  // persistent CTAs and chunk divisor the chunk list was built for,
                  // and the stream kernel form and split-K combine the graph holds
  bool operator==(const GraphKey& o) const {
    return plans == o.plans && versions == o.versions && mode == o.mode && sched == o.sched;
  }
};

struct tb_ctx {
  int device = 0;
  tb_options opt{};
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int sms = 0;
  int persistent_ctas = 0;
  int stream_ctas = 0;  // resident CTAs of the stream-tile kernels
  int stream_ctas_wide = 0;  // the same for the 128-register form of the stream level kernel
  bool stream_wide = true;   // per-level stream launches use that form (measured faster on
                             // every benchmark workload; tb_autotune may choose the other)
  bool kpart_atomic = false; // split-K parts combine by atomic max where values allow (tb_autotune)
  bool kpart_merge = true;   // batches whose items fill the GPU run split-K GEMMs merged (merge_choice)
  int gemm_ctas = 0;    // resident CTAs of the GEMM-tile kernels
  std::vector<int32_t> small_order;   // fused small form: items by shared need, largest first
  std::vector<SmallGroup> small_groups;  // launches over small_order
  DevBuf small_order_dev;
  uint64_t call_counter = 0;  // solve calls (stamps plans seen in a call)
  // the batch whose weights the pinned staging buffer holds: a call with the
  // same plans in the same order and the same layout skips re-staging the
  // weights of plans that were not re-bound since
  std::vector<const tb_plan*> stage_plans;
  size_t stage_wbase = 0;
  uint64_t stage_hin_gen = 0, stage_epoch = 0;
  std::mutex plans_mu;        // guards live_plans
  std::unordered_set<tb_plan*> live_plans;  // plans created on this context and not destroyed
  int tune_fallback = TB_MODE_BATCHED;  // tuned mode for batches the fused form cannot run
  size_t budget = 0;
  DevBuf arena, items, groups, chunks, done, misc, slice_vals, out_item, rvals, wvals;
  HostBuf h_items, h_groups, h_chunks, h_in, h_out;
  // batch state of the last upload (reused when the same plans come again)
  GraphKey key;
  bool have_key = false;
  int64_t n_tickets = 0;
  int n_groups = 0;
  int64_t n_chunks = 0;
  struct LevelRange {
    int64_t first, count;
    int kinds;     // 1 stream-like, 2 GEMM
    int g0, g1;    // its groups [g0, g1) (contiguous: groups are sorted by level and kind)
    int64_t tiny;  // tickets of its tiny steps (listed first)
    double tiny_cost, rest_cost;  // estimated CTA time of its tiny steps and of the rest (us; level_span)
  };
  std::vector<LevelRange> level_ranges;
  size_t sv_bytes = 0;
  int n_items = 0;
  cudaGraphExec_t gexec = nullptr;
  double last_ms = 0;
  int64_t last_launches = 0;
  int64_t launches_graph = 0;
  uint64_t plan_counter = 0;
  std::mutex mu;
  // schedule knobs of the batched executor (tb_autotune sets them)
  int ctas_per_sm_max = 2;  // resident k_persistent CTAs per SM
  int chunk_div = 4;        // a stream step's runs hold >= 1/(chunk_div ctas) of its level
  bool tuned = false;
  tb_tune_result tune{};
};

static tb_status fail(tb_status s, const std::string& msg) {
  g_err = msg;
  return s;
}

namespace tb {
// Lets other translation units of the library report through tb_last_error.
void set_last_error(const std::string& msg) { g_err = msg; }

cudaError_t smem_optin(const void* fn, int bytes) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, int> opted;  // (kernel, device) -> bytes
  std::lock_guard<std::mutex> lk(mu);
  int& have = opted[{fn, dev}];
  if (bytes <= have) return cudaSuccess;
  e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e != cudaSuccess) return e;
  have = bytes;
  return cudaSuccess;
}
}  // namespace tb

#define CU(x)                                                                                   \
  do {                                                                                          \
    cudaError_t e_ = (x);                                                                       \
    if (e_ != cudaSuccess)                                                                      \
      return fail(TB_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_));                \
  } while (0)

static int64_t align_up(int64_t x, int64_t a) { return (x + a - 1) / a * a; }

// A stream step one warp of the level kernel runs from global memory
// (tiny_node): one tile, no reduction loop, small enough (a block would split
// its reduction over threads; a warp does not need to).
static bool tiny_step(const TileDesc& d) {
  return d.n_tiles == 1 && d.n_loop == 0 && d.n_tc <= kTinyOut && d.n_tr <= kTinyRed && d.n_tc + d.n_tr <= 10;
}

// tiny_node's form of a tiny step: tensor positions straight from the tile
// bits (one tile, no grid or loop bits: tile bits cover whole tensors)
static TinyDesc make_tiny(const TileDesc& d) {
  TinyDesc t;
  std::memset(&t, 0xff, sizeof(t));
  t.a_off = d.a_off;
  t.b_off = d.b_off;
  t.c_off = d.c_off;
  t.n_tc = (int8_t)d.n_tc;
  t.n_tr = (int8_t)d.n_tr;
  if (!tiny_step(d)) {
    t.n_tc = t.n_tr = 0;
    return t;
  }
  for (int b = 0; b < d.n_tc; b++) {
    t.oa[b] = d.tc_a[b] >= 0 ? d.ta_pos[d.tc_a[b]] : (int8_t)-1;
    t.ob[b] = d.b_off >= 0 && d.tc_b[b] >= 0 ? d.tb_pos[d.tc_b[b]] : (int8_t)-1;
    t.oc[b] = d.tc_pos[b];
  }
  for (int b = 0; b < d.n_tr; b++) {
    t.ra[b] = d.tr_a[b] >= 0 ? d.ta_pos[d.tr_a[b]] : (int8_t)-1;
    t.rb[b] = d.b_off >= 0 && d.tr_b[b] >= 0 ? d.tb_pos[d.tr_b[b]] : (int8_t)-1;
  }
  return t;
}

template <typename T>
static size_t elem() { return sizeof(T); }

static size_t dtype_size(const tb_ctx*) { return 4; }

// Dynamic shared memory of the kernels: stream tiles (see plan_tile's
// limits), GEMM tiles (pipeline stages), or both for the persistent kernel.
static int stream_smem_bytes() { return stream_smem_words_max() * 4; }
static int smem_bytes(int kinds) {
  int b = 0;
  if (kinds & 1) b = std::max(b, stream_smem_bytes());
  if (kinds & 2) b = std::max(b, gemm_smem_bytes_max());
  return b;
}
static int max_stream_smem_bytes() { return smem_bytes(3); }

// The launch wrappers set each kernel's shared-memory limit on first use.
template <typename T>
static tb_status set_kernel_attrs() {
  return TB_OK;
}

// Descriptors to the device (once, and again after re-tiling).  Paths that
// build leaves from LeafDesc::w (tb_contract, dumps, serving) also need the
// leaves re-sent after a re-bind; the batched and plain solves read the
// weights from a per-call weight array instead.
static tb_status upload_plan(tb_plan* p, bool leaf_weights) {
  auto up = [&](DevBuf& b, const void* src, size_t bytes) -> cudaError_t {
    if (bytes == 0) bytes = 16;
    cudaError_t e = b.ensure(bytes);
    if (e != cudaSuccess) return e;
    if (src) return cudaMemcpy(b.p, src, bytes, cudaMemcpyHostToDevice);
    return cudaSuccess;
  };
  PlanHost& h = p->h;
  // LeafDesc::w matters only to the paths that build leaves from it (the
  // batched and plain solves pass a per-call weight array instead)
  if (!p->structure_uploaded || (leaf_weights && p->leaves_dirty))
    for (int i : p->vertex_leaves) h.leaves[i].w = p->weights[h.leaves[i].label];
  if (!p->structure_uploaded) {
    void* before[9] = {p->d_steps.p, p->d_tiles.p, p->d_gemms.p, p->d_leaves.p, p->d_small.p, p->d_small_leaf.p,
                       p->d_steps_merged.p, p->d_gemms_merged.p, p->d_tiny.p};
    CU(up(p->d_steps, h.steps.data(), h.steps.size() * sizeof(Step)));
    CU(up(p->d_tiles, h.tiles.empty() ? nullptr : h.tiles.data(), h.tiles.size() * sizeof(TileDesc)));
    CU(up(p->d_gemms, h.gemms.empty() ? nullptr : h.gemms.data(), h.gemms.size() * sizeof(GemmDesc)));
    {
      std::vector<TinyDesc> tiny(h.tiles.size());
      for (size_t k = 0; k < h.tiles.size(); k++) tiny[k] = make_tiny(h.tiles[k]);
      CU(up(p->d_tiny, tiny.empty() ? nullptr : tiny.data(), tiny.size() * sizeof(TinyDesc)));
    }
    if (h.has_split) {
      CU(up(p->d_steps_merged, h.steps_merged.data(), h.steps_merged.size() * sizeof(Step)));
      CU(up(p->d_gemms_merged, h.gemms_merged.data(), h.gemms_merged.size() * sizeof(GemmDesc)));
    }
    CU(up(p->d_leaves, h.leaves.data(), h.leaves.size() * sizeof(LeafDesc)));
    if (h.small_ok) {
      CU(up(p->d_small, h.small.empty() ? nullptr : h.small.data(), h.small.size() * sizeof(SmallNode)));
      CU(up(p->d_small_leaf, h.small_leaf.data(), h.small_leaf.size() * sizeof(int32_t)));
    }
    void* after[9] = {p->d_steps.p, p->d_tiles.p, p->d_gemms.p, p->d_leaves.p, p->d_small.p, p->d_small_leaf.p,
                      p->d_steps_merged.p, p->d_gemms_merged.p, p->d_tiny.p};
    // captured graphs hold these device pointers: a move invalidates them
    if (std::memcmp(before, after, sizeof(before)) != 0) p->version = ++p->ctx->plan_counter;
    p->structure_uploaded = true;
    p->leaves_dirty = false;
  } else if (leaf_weights && p->leaves_dirty) {
    CU(up(p->d_leaves, h.leaves.data(), h.leaves.size() * sizeof(LeafDesc)));
    p->leaves_dirty = false;
  }
  return TB_OK;
}

// ---------------------------------------------------------------------------
// plain path (drop-in): one item, per-node launches
// ---------------------------------------------------------------------------
template <typename T>
static tb_status plain_item(tb_ctx* c, tb_plan* p, T* arena, const int8_t* d_sv, bool leaves_from_mis,
                            const float* d_w, int64_t& launches) {
  const PlanHost& h = p->h;
  cudaStream_t s = c->stream;
  if (leaves_from_mis) {
    CU(launch_leaves<T>((h.n_tensors + kThreads - 1) / kThreads, s, 
        reinterpret_cast<const LeafDesc*>(p->d_leaves.p), h.n_tensors, d_sv, arena, d_w));
    CU(cudaGetLastError());
    launches++;
  }
  if (h.n_nodes == 0) {
    const TileDesc& d = h.tiles[0];
    int64_t grid = std::min<int64_t>(d.n_tiles, c->stream_ctas);
    CU(launch_tile<T>((unsigned)grid, stream_smem_words(d) * 4, s, d, arena, (d.n_tiles + grid - 1) / grid));
    CU(cudaGetLastError());
    launches++;
    return TB_OK;
  }
  for (int j = 0; j < h.n_nodes; j++) {
    for (const PlainOp& op : h.plain[j]) {
      if (op.kind == PLAIN_TILE) {
        int64_t grid = std::min<int64_t>(op.tile.n_tiles, c->stream_ctas);
        CU(launch_tile<T>((unsigned)grid, stream_smem_words(op.tile) * 4, s, op.tile, arena,
                                                                                    (op.tile.n_tiles + grid - 1) / grid));
        CU(cudaGetLastError());
      } else {
        CU(launch_k1_any<T>(arena + op.a_off, arena + op.b_off, arena + op.c_off, op.M, op.N, op.K, op.batch, s));
      }
      launches++;
    }
  }
  return TB_OK;
}

// ---------------------------------------------------------------------------
// batched upload: items, groups (dependency order), counters
// ---------------------------------------------------------------------------
// One (item, step) of a batch with its launch-order key.
struct GroupKey {
  int level, kinds, tiny, item, step;
};

// Steps of item i of a batch: the merged split-K form where merged[i].
static const std::vector<Step>& batch_steps(tb_plan* const* plans, const char* merged, int i) {
  const PlanHost& h = plans[i]->h;
  return merged && merged[i] ? h.steps_merged : h.steps;
}

// Which items run their split-K GEMMs merged (one pass over the whole K, no
// partials and no max step): those whose plan, over all the batch's items
// that share it, keeps >= 90% of the GEMM CTA slots of the last wave busy
// without the split at every split GEMM.  The plan compiler split K for one
// item alone; a batch of many items fills the GPU by itself.
static std::vector<char> merge_choice(const tb_ctx* c, int n, tb_plan* const* plans) {
  std::vector<char> m(n, 0);
  if (!c->kpart_merge) return m;
  std::unordered_map<const tb_plan*, int> count;
  for (int i = 0; i < n; i++)
    if (plans[i]->h.has_split) count[plans[i]]++;
  std::unordered_map<const tb_plan*, char> ok;
  const int64_t ctas = std::max(1, c->gemm_ctas);
  for (const auto& kv : count) {
    bool good = true;
    for (const GemmDesc& g : kv.first->h.gemms) {
      if (g.ks_log2 == 0) continue;
      const int64_t units = (int64_t)kv.second * (g.n_tiles >> g.ks_log2);
      good = good && (double)units >= 0.9 * (double)(((units + ctas - 1) / ctas) * ctas);
    }
    ok[kv.first] = good;
  }
  for (int i = 0; i < n; i++) {
    auto f = ok.find(plans[i]);
    m[i] = f != ok.end() && f->second;
  }
  return m;
}

// Estimated CTA time (us) of per-level launch work, for level_span's split
// of a grid between tiny steps and the rest (measured on KSG levels: a warp
// runs a one-pass tiny step in ~2 us and each further four passes add about
// as much, with eight warps a CTA; a stream step builds its tables in ~3 us
// and runs each tile of a run in < 1 us).  The tiny share is counted as if
// six warps shared the tiny steps: the split measured best that way on the
// King's-subgraph batches (ksg32_b20 22.0 -> 21.5 ms against eight).
constexpr double kGroupCostUs = 3.0;
constexpr double kTileCostUs = 0.8;
static double tiny_cost_us(int n_tc, int n_tr) {
  const int passes = std::max(1, 1 << std::max(0, n_tc + n_tr - 5));
  return (2.0 + 1.5 * (double)((passes - 1) / 4)) / 6.0;
}

// The batch's steps in launch order: by tree level, then kind (stream-like
// before GEMM), tiny steps first, then item and step.  Steps without tiles
// (the fill and max steps of a merged split-K GEMM) are left out.
static std::vector<GroupKey> sorted_groups(int n, tb_plan* const* plans, bool skip_leaves, const char* merged) {
  std::vector<GroupKey> gk;
  for (int i = 0; i < n; i++) {
    const PlanHost& h = plans[i]->h;
    const std::vector<Step>& steps = batch_steps(plans, merged, i);
    for (int s = 0; s < (int)steps.size(); s++) {
      const Step& st = steps[s];
      if (skip_leaves && st.kind == STEP_LEAVES) continue;
      if (st.n_tiles == 0) continue;
      gk.push_back({st.level, st.kind == STEP_GEMM ? 2 : 1, st.kind == STEP_TILE && tiny_step(h.tiles[st.desc]),
                    i, s});
    }
  }
  std::stable_sort(gk.begin(), gk.end(), [](const GroupKey& a, const GroupKey& b) {
    if (a.level != b.level) return a.level < b.level;
    if (a.kinds != b.kinds) return a.kinds < b.kinds;
    if (a.tiny != b.tiny) return a.tiny > b.tiny;
    if (a.item != b.item) return a.item < b.item;
    return a.step < b.step;
  });
  return gk;
}

// Groups (host copy, gk.size() entries) and one launch range per (level,
// kind); returns the number of tickets.
static int64_t fill_groups(const std::vector<GroupKey>& gk, tb_plan* const* plans, const char* merged,
                           const std::vector<void*>& arenas, Group* hg, std::vector<tb_ctx::LevelRange>& ranges) {
  int64_t tk = 0;
  ranges.clear();
  int cur_level = -1, cur_kinds = -1;
  for (size_t g = 0; g < gk.size(); g++) {
    const tb_plan* p = plans[gk[g].item];
    hg[g].item = gk[g].item;
    hg[g].step = gk[g].step;
    hg[g].first = tk;
    hg[g].tiny = gk[g].tiny;
    hg[g].run = 0;
    hg[g].tile = gk[g].tiny ? reinterpret_cast<const TinyDesc*>(p->d_tiny.p) + p->h.steps[gk[g].step].desc : nullptr;
    hg[g].arena = gk[g].tiny ? arenas[gk[g].item] : nullptr;
    if (gk[g].level != cur_level || gk[g].kinds != cur_kinds) {
      ranges.push_back({tk, 0, gk[g].kinds, (int)g, (int)g, 0, 0.0, 0.0});
      cur_level = gk[g].level;
      cur_kinds = gk[g].kinds;
    }
    const int64_t nt = batch_steps(plans, merged, gk[g].item)[gk[g].step].n_tiles;
    tk += nt;
    ranges.back().count += nt;
    ranges.back().g1 = (int)g + 1;
    if (gk[g].tiny) {
      const TileDesc& d = p->h.tiles[p->h.steps[gk[g].step].desc];
      ranges.back().tiny += nt;
      ranges.back().tiny_cost += tiny_cost_us(d.n_tc, d.n_tr);
    } else {
      ranges.back().rest_cost += kGroupCostUs + kTileCostUs * (double)nt;
    }
  }
  // run lengths of the tiny groups (listed first in their launch range)
  for (size_t g = gk.size(); g-- > 0;)
    if (gk[g].tiny)
      hg[g].run = 1 + (g + 1 < gk.size() && gk[g + 1].tiny && gk[g + 1].level == gk[g].level &&
                               gk[g + 1].kinds == gk[g].kinds
                           ? hg[g + 1].run
                           : 0);
  return tk;
}
template <typename T>
static tb_status upload_batch(tb_ctx* c, int n, tb_plan* const* plans, const std::vector<int64_t>& arena_off,
                              const std::vector<int64_t>& sv_off, bool skip_leaves,
                              const std::vector<int64_t>* w_off) {
  // items
  CU(c->h_items.ensure(sizeof(ItemDev<T>) * n));
  ItemDev<T>* hi = reinterpret_cast<ItemDev<T>*>(c->h_items.p);
  const std::vector<char> merged = merge_choice(c, n, plans);
  int done_base = 0;
  for (int i = 0; i < n; i++) {
    tb_plan* p = plans[i];
    ItemDev<T> it{};
    it.arena = reinterpret_cast<T*>(c->arena.p) + arena_off[i];
    it.steps = reinterpret_cast<const Step*>(merged[i] ? p->d_steps_merged.p : p->d_steps.p);
    it.tiles = reinterpret_cast<const TileDesc*>(p->d_tiles.p);
    it.gemms = reinterpret_cast<const GemmDesc*>(merged[i] ? p->d_gemms_merged.p : p->d_gemms.p);
    it.leaves = reinterpret_cast<const LeafDesc*>(p->d_leaves.p);
    it.slice_vals = reinterpret_cast<const int8_t*>(c->slice_vals.p) + sv_off[i];
    it.w = w_off ? reinterpret_cast<const float*>(c->wvals.p) + (*w_off)[i] : nullptr;
    // exact packed-int16 GEMM tiles only when the context allows them and
    // the per-call weights are the plan's bound ones (the batched solves)
    it.flags = (c->opt.gemm_i16 && w_off && std::is_same<T, float>::value && p->i16_ok) ? 1 : 0;
    // split-K parts by atomic max where every value is >= 0 or -inf (int32:
    // always), with the plan's bound weights
    if (c->kpart_atomic && w_off && (!std::is_same<T, float>::value || p->nonneg_ok)) it.flags |= 2;
    it.r = 0.0f;
    it.n_leaves = p->h.n_tensors;
    it.done_base = done_base;
    it.n_steps = (int)p->h.steps.size();
    it.fin = p->h.fin;
    if (p->h.small_ok) {
      it.small = reinterpret_cast<const SmallNode*>(p->d_small.p);
      it.small_leaf = reinterpret_cast<const int32_t*>(p->d_small_leaf.p);
      it.n_small = (int32_t)p->h.small.size();
      it.small_root = p->h.small_root;
      it.small_root_log2 = p->h.small_root_log2;
      it.small_words = p->h.small_words;
    }
    done_base += it.n_steps;
    hi[i] = it;
  }
  std::vector<GroupKey> gk = sorted_groups(n, plans, skip_leaves, merged.data());
  CU(c->h_groups.ensure(sizeof(Group) * std::max<size_t>(gk.size(), 1)));
  Group* hg = reinterpret_cast<Group*>(c->h_groups.p);
  std::vector<void*> arenas(n);
  for (int i = 0; i < n; i++) arenas[i] = hi[i].arena;
  const int64_t tk = fill_groups(gk, plans, merged.data(), arenas, hg, c->level_ranges);
  c->n_tickets = tk;
  c->n_groups = (int)gk.size();
  // chunks for the persistent executor: runs of stream tiles (tables are
  // built once per chunk and the copy pipeline stays full along the run),
  // single GEMM tiles, whole leaf / final steps.  A stream step is cut into
  // runs of at least 1/ctas of its tiles and at least 1/(4 ctas) of the
  // stream tiles of its whole level, so many small steps of many items do
  // not turn into as many tiny runs.
  std::vector<int64_t> level_tiles;
  for (const GroupKey& x : gk) {
    const Step& st = batch_steps(plans, merged.data(), x.item)[x.step];
    if (st.kind != STEP_TILE && st.kind != STEP_KRED && st.kind != STEP_FILL) continue;
    if ((int)level_tiles.size() <= x.level) level_tiles.resize(x.level + 1, 0);
    level_tiles[x.level] += st.n_tiles;
  }
  const int64_t ctas = std::max(1, c->persistent_ctas);
  std::vector<Chunk> chs;
  for (size_t g = 0; g < gk.size(); g++) {
    const Step& st = batch_steps(plans, merged.data(), gk[g].item)[gk[g].step];
    const int64_t nt = st.n_tiles;
    int64_t cs = 1;
    if (st.kind == STEP_TILE || st.kind == STEP_KRED || st.kind == STEP_FILL) {
      const int64_t lt = level_tiles[gk[g].level];
      const int64_t div = std::max(1, c->chunk_div) * ctas;
      cs = std::max((nt + ctas - 1) / ctas, (lt + div - 1) / div);
      cs = std::max<int64_t>(1, std::min<int64_t>(cs, 256));
    } else if (st.kind == STEP_GEMM) {
      // runs of GEMM units share one copy pipeline; keep >= 1 run per CTA
      cs = std::max<int64_t>(1, std::min<int64_t>(nt / ctas, 64));
    } else if (st.kind == STEP_LEAVES) {
      cs = nt;
    }
    for (int64_t t0 = 0; t0 < nt; t0 += cs) {
      Chunk ch;
      ch.group = (int32_t)g;
      ch.pad_ = 0;
      ch.t0 = t0;
      ch.t1 = std::min(nt, t0 + cs);
      chs.push_back(ch);
    }
  }
  c->n_chunks = (int64_t)chs.size();
  CU(c->chunks.ensure(sizeof(Chunk) * std::max<size_t>(chs.size(), 1)));
  CU(cudaMemcpyAsync(c->chunks.p, chs.data(), sizeof(Chunk) * chs.size(), cudaMemcpyHostToDevice, c->stream));
  CU(cudaStreamSynchronize(c->stream));
  CU(c->items.ensure(sizeof(ItemDev<T>) * n));
  CU(c->groups.ensure(sizeof(Group) * std::max<size_t>(gk.size(), 1)));
  CU(c->done.ensure(sizeof(int) * std::max(done_base, 1) + 64));
  CU(cudaMemcpyAsync(c->items.p, hi, sizeof(ItemDev<T>) * n, cudaMemcpyHostToDevice, c->stream));
  CU(cudaMemcpyAsync(c->groups.p, hg, sizeof(Group) * gk.size(), cudaMemcpyHostToDevice, c->stream));
  c->misc.ensure(64);
  // leaves of skipped-leaf runs count as done
  if (skip_leaves) {
    std::vector<int> init(done_base, 0);
    for (int i = 0; i < n; i++) init[hi[i].done_base] = plans[i]->h.steps[0].n_tiles;
    CU(cudaMemcpyAsync(c->done.p, init.data(), sizeof(int) * done_base, cudaMemcpyHostToDevice, c->stream));
    CU(cudaStreamSynchronize(c->stream));
  }
  return TB_OK;
}

// Grid and ticket span of one per-level launch on at most max_ctas CTAs.
// A launch whose tiny steps come first gives them and its other tiles CTAs
// in proportion to their estimated cost, so neither part waits on a few
// overloaded CTAs (costs in us of one CTA's time, from fill_groups:
// tiny_cost_us a tiny step, kGroupCostUs + kTileCostUs a tile of the rest).
static LevelSpan level_span(const tb_ctx::LevelRange& lr, int64_t max_ctas, int64_t& grid) {
  LevelSpan sp{};
  sp.first = lr.first;
  sp.last = lr.first + lr.count;
  max_ctas = std::max<int64_t>(1, max_ctas);
  const int64_t tiny = lr.tiny, rest = lr.count - lr.tiny;
  if (tiny == 0 || rest == 0 || max_ctas < 2) {
    grid = std::min<int64_t>(lr.count, max_ctas);
    sp.mid = sp.last;
    sp.chunk = (lr.count + grid - 1) / grid;
    sp.chunk2 = 1;
    sp.split_cta = (int32_t)grid;
    return sp;
  }
  const double wt = std::max(lr.tiny_cost, 1e-3), wr = std::max(lr.rest_cost, 1e-3);
  int64_t gt = (int64_t)std::llround((double)max_ctas * wt / (wt + wr));
  gt = std::max<int64_t>(1, std::min<int64_t>(std::min<int64_t>(gt, max_ctas - 1), tiny));
  const int64_t gr = std::min<int64_t>(max_ctas - gt, rest);
  sp.mid = lr.first + tiny;
  sp.chunk = (tiny + gt - 1) / gt;
  sp.chunk2 = (rest + gr - 1) / gr;
  sp.split_cta = (int32_t)gt;
  grid = gt + gr;
  return sp;
}

// One per-level launch of the ranges' kernel form on stream s.
template <typename T>
static cudaError_t launch_range(const tb_ctx* c, const tb_ctx::LevelRange& lr, cudaStream_t s,
                                const ItemDev<T>* items, const Group* groups, float* out_item, const float* r,
                                int* err) {
  const Group* lg = groups + lr.g0;
  const int ng = lr.g1 - lr.g0;
  int64_t grid = 0;
  if (lr.kinds == 2) {
    const LevelSpan sp = level_span(lr, c->gemm_ctas, grid);
    return launch_level<T, 2>((unsigned)grid, smem_bytes(2), s, items, lg, ng, sp, out_item, r, err);
  }
  if (c->stream_wide) {
    const LevelSpan sp = level_span(lr, c->stream_ctas_wide, grid);
    return launch_level<T, 5>((unsigned)grid, smem_bytes(1), s, items, lg, ng, sp, out_item, r, err);
  }
  const LevelSpan sp = level_span(lr, c->stream_ctas, grid);
  return launch_level<T, 1>((unsigned)grid, smem_bytes(1), s, items, lg, ng, sp, out_item, r, err);
}

// One launch of the per-level schedule: every tile of one (tree level,
// kind) of the uploaded batch.
template <typename T>
static tb_status enqueue_level(tb_ctx* c, const tb_ctx::LevelRange& lr) {
  const ItemDev<T>* items = reinterpret_cast<const ItemDev<T>*>(c->items.p);
  const Group* groups = reinterpret_cast<const Group*>(c->groups.p);
  float* out_item = reinterpret_cast<float*>(c->out_item.p);
  const float* rv = reinterpret_cast<const float*>(c->rvals.p);
  int* err = reinterpret_cast<int*>(reinterpret_cast<char*>(c->misc.p) + 16);
  if (lr.count > 0x7fffffffLL) return fail(TB_ERR_UNSUPPORTED, "level too large for one launch");
  // the kernel searches only this level's groups (their tickets are absolute)
  CU(launch_range<T>(c, lr, c->stream, items, groups, out_item, rv, err));
  return TB_OK;
}

template <typename T>
static tb_status enqueue_batched(tb_ctx* c, int n, int mode, int done_words, int64_t& launches) {
  cudaStream_t s = c->stream;
  const ItemDev<T>* items = reinterpret_cast<const ItemDev<T>*>(c->items.p);
  const Group* groups = reinterpret_cast<const Group*>(c->groups.p);
  float* out_item = reinterpret_cast<float*>(c->out_item.p);
  const float* rv = reinterpret_cast<const float*>(c->rvals.p);
  const int smem = max_stream_smem_bytes();
  CU(cudaMemsetAsync(c->misc.p, 0, 64, s));
  if (mode == TB_MODE_FUSED) {
    const int32_t* order = reinterpret_cast<const int32_t*>(c->small_order_dev.p);
    for (const SmallGroup& g : c->small_groups) {
      CU(launch_small<T>((unsigned)g.count, g.smem, s, items, order + g.first, g.count, out_item, rv));
      launches++;
    }
  } else if (mode == TB_MODE_BATCHED) {
    CU(cudaMemsetAsync(c->done.p, 0, sizeof(int) * done_words, s));
    unsigned long long* ticket = reinterpret_cast<unsigned long long*>(c->misc.p);
    int* err = reinterpret_cast<int*>(reinterpret_cast<char*>(c->misc.p) + 16);
    int64_t timeout_ns = (int64_t)c->opt.timeout_ms * 1000000LL;
    CU(launch_persistent<T>(c->persistent_ctas, smem, s, items, groups,
                                                               reinterpret_cast<const Chunk*>(c->chunks.p),
                                                               c->n_chunks, reinterpret_cast<int*>(c->done.p),
                                                               ticket, err, out_item, rv, timeout_ns));
    CU(cudaGetLastError());
    launches++;
  } else {
    for (auto& lr : c->level_ranges) {
      tb_status st = enqueue_level<T>(c, lr);
      if (st) return st;
      launches++;
    }
  }
  k_reduce_max<<<1, kThreads, 0, s>>>(out_item, n, out_item + n);
  CU(cudaGetLastError());
  launches++;
  return TB_OK;
}

template <typename T>
static tb_status solve_batch_t(tb_ctx* c, int n, tb_plan* const* plans, const int8_t* slice_vals, const float* r,
                               float* out_item, float* out_max, int mode) {
  CU(cudaSetDevice(c->device));
  tb_status st = set_kernel_attrs<T>();
  if (st) return st;
  for (int i = 0; i < n; i++) {
    if (!plans[i]) return fail(TB_ERR_INVALID, "null plan");
    if (plans[i]->ctx != c) return fail(TB_ERR_INVALID, "plan belongs to another context");
    if (!plans[i]->h.has_weights) return fail(TB_ERR_INVALID, "plan has no bound weights (tb_plan_bind_mis)");
    if ((st = upload_plan(plans[i], false))) return st;
  }
  if (mode == TB_MODE_FUSED) {
    // one launch; every block asks for the largest shared-memory need of the
    // batch (the item order is built with the batch upload)
    int smem = 16;
    for (int i = 0; i < n; i++) {
      const PlanHost& h = plans[i]->h;
      if (!h.small_ok) return fail(TB_ERR_UNSUPPORTED, "TB_MODE_FUSED: a plan has no small form");
      smem = std::max(smem, (int)(h.small_words * sizeof(T)));
    }
    c->small_groups.assign(1, SmallGroup{0, n, smem});
  }
  // weights of each distinct plan, staged once per call
  std::vector<int64_t> w_off(n);
  std::vector<char> w_first(n, 0);
  int64_t w_total = 0;
  {
    // first sighting of a plan in this call: its stamp is older than the call
    const uint64_t call = ++c->call_counter;
    for (int i = 0; i < n; i++) {
      tb_plan* p = plans[i];
      if (p->seen_call == call) {
        w_off[i] = p->seen_off;
      } else {
        w_off[i] = w_total;
        w_first[i] = 1;
        p->seen_call = call;
        p->seen_off = w_total;
        w_total += align_up(std::max<int64_t>(p->h.n_labels, 1), 4);
      }
    }
  }
  // slice values (concatenated)
  std::vector<int64_t> sv_off(n);
  size_t sv = 0;
  for (int i = 0; i < n; i++) {
    sv_off[i] = (int64_t)sv;
    sv += plans[i]->h.sliced.size();
  }
  if (sv > 0 && !slice_vals) return fail(TB_ERR_INVALID, "slice_vals required for sliced plans");
  for (size_t k = 0; k < sv; k++)
    if (slice_vals[k] != 0 && slice_vals[k] != 1) return fail(TB_ERR_INVALID, "slice values must be 0 or 1");
  CU(c->slice_vals.ensure(std::max<size_t>(sv, 16)));
  CU(c->out_item.ensure(sizeof(float) * (n + 1)));
  CU(c->h_out.ensure(sizeof(float) * (n + 1) + 64));
  // pinned staging of the per-call inputs: r values, slice values, weights
  const size_t r_bytes = align_up(sizeof(float) * n, 16);
  const size_t sv_bytes = align_up(std::max<size_t>(sv, 16), 16);
  const size_t w_bytes = sizeof(float) * (size_t)std::max<int64_t>(w_total, 4);
  CU(c->h_in.ensure(r_bytes + sv_bytes + w_bytes));
  CU(c->rvals.ensure(r_bytes));
  CU(c->wvals.ensure(w_bytes));
  float* h_r = reinterpret_cast<float*>(c->h_in.p);
  int8_t* h_sv = reinterpret_cast<int8_t*>(c->h_in.p) + r_bytes;
  float* h_w = reinterpret_cast<float*>(reinterpret_cast<char*>(c->h_in.p) + r_bytes + sv_bytes);
  for (int i = 0; i < n; i++) h_r[i] = r ? r[i] : 0.0f;
  if (sv) std::memcpy(h_sv, slice_vals, sv);
  {
    bool same = c->stage_hin_gen == c->h_in.gen && c->stage_wbase == r_bytes + sv_bytes &&
                c->stage_plans.size() == (size_t)n;
    for (int i = 0; same && i < n; i++) same = c->stage_plans[i] == plans[i];
    if (!same) {
      c->stage_plans.assign(plans, plans + n);
      c->stage_wbase = r_bytes + sv_bytes;
      c->stage_hin_gen = c->h_in.gen;
      c->stage_epoch++;
    }
    for (int i = 0; i < n; i++) {
      tb_plan* p = plans[i];
      if (!w_first[i] || (p->staged_epoch == c->stage_epoch && p->staged_wgen == p->wgen)) continue;
      std::memcpy(h_w + w_off[i], p->weights.data(), sizeof(float) * p->h.n_labels);
      p->staged_epoch = c->stage_epoch;
      p->staged_wgen = p->wgen;
    }
  }
  const float* d_w = reinterpret_cast<const float*>(c->wvals.p);
  float* hout = reinterpret_cast<float*>(c->h_out.p);
  int64_t launches = 0;
  CU(cudaEventRecord(c->ev0, c->stream));
  if (mode == TB_MODE_PLAIN) {
    // one item at a time, as the reference loop
    int64_t need = 0;
    for (int i = 0; i < n; i++) need = std::max(need, plans[i]->h.plain_elems);
    size_t bytes = (size_t)need * sizeof(T) + 256;
    if (bytes > c->budget) return fail(TB_ERR_OOM, "plan needs more device memory than the budget");
    CU(c->arena.ensure(bytes));
    if (sv) CU(cudaMemcpyAsync(c->slice_vals.p, h_sv, sv, cudaMemcpyHostToDevice, c->stream));
    CU(cudaMemcpyAsync(c->wvals.p, h_w, w_bytes, cudaMemcpyHostToDevice, c->stream));
    T* arena = reinterpret_cast<T*>(c->arena.p);
    for (int i = 0; i < n; i++) {
      tb_plan* p = plans[i];
      const int8_t* d_sv = reinterpret_cast<const int8_t*>(c->slice_vals.p) + sv_off[i];
      if ((st = plain_item<T>(c, p, arena, d_sv, true, d_w + w_off[i], launches))) return st;
      CU(launch_final<T>(c->stream, p->h.fin, arena, r ? r[i] : 0.0f,
                                                reinterpret_cast<float*>(c->out_item.p) + i));
      CU(cudaGetLastError());
      launches++;
      // synchronous read-back per item (Array(...)[] in solve_slice)
      CU(cudaMemcpyAsync(hout + i, reinterpret_cast<float*>(c->out_item.p) + i, sizeof(float),
                         cudaMemcpyDeviceToHost, c->stream));
      CU(cudaStreamSynchronize(c->stream));
    }
    float m = -INFINITY;
    for (int i = 0; i < n; i++) m = std::max(m, hout[i]);
    hout[n] = m;
    CU(cudaEventRecord(c->ev1, c->stream));
    CU(cudaEventSynchronize(c->ev1));
  } else {
    // arenas of all items side by side; waves when over budget
    std::vector<int64_t> aoff(n, 0);
    int64_t tot = 0;
    if (mode != TB_MODE_FUSED) {  // the fused form keeps every tensor in shared memory
      for (int i = 0; i < n; i++) {
        aoff[i] = tot;
        tot = align_up(tot + plans[i]->h.arena_elems, 64);
      }
    }
    size_t bytes = (size_t)tot * sizeof(T) + 256;
    if (bytes > c->budget) {
      // split into waves that fit
      int i0 = 0;
      std::vector<float> all(n + 1, -INFINITY);
      while (i0 < n) {
        int i1 = i0;
        int64_t t2 = 0;
        while (i1 < n && ((size_t)(t2 + plans[i1]->h.arena_elems) * sizeof(T) + 256 <= c->budget || i1 == i0)) {
          t2 = align_up(t2 + plans[i1]->h.arena_elems, 64);
          i1++;
        }
        if ((size_t)t2 * sizeof(T) + 256 > c->budget) return fail(TB_ERR_OOM, "one item exceeds the device budget");
        std::vector<float> part(i1 - i0);
        float pm;
        st = solve_batch_t<T>(c, i1 - i0, plans + i0, slice_vals ? slice_vals + sv_off[i0] : nullptr,
                              r ? r + i0 : nullptr, part.data(), &pm, mode);
        if (st) return st;
        for (int i = i0; i < i1; i++) all[i] = part[i - i0];
        i0 = i1;
      }
      float m = -INFINITY;
      for (int i = 0; i < n; i++) m = std::max(m, all[i]);
      if (out_item) std::memcpy(out_item, all.data(), sizeof(float) * n);
      if (out_max) *out_max = m;
      return TB_OK;
    }
    CU(c->arena.ensure(bytes));
    GraphKey key;
    key.mode = mode;
    key.sched = ((c->persistent_ctas * 64 + c->chunk_div) * 4 + (c->stream_wide ? 1 : 0) + (c->kpart_atomic ? 2 : 0)) *
                    2 + (c->kpart_merge ? 1 : 0);
    key.plans.reserve(n);
    key.versions.reserve(n);
    for (int i = 0; i < n; i++) {
      key.plans.push_back(plans[i]);
      key.versions.push_back(plans[i]->version);
    }
    bool reuse = c->have_key && c->key == key && c->n_items == n;
    int done_words = 0;
    for (int i = 0; i < n; i++) done_words += (int)plans[i]->h.steps.size();
    if (!reuse) {
      if (c->gexec) {
        cudaGraphExecDestroy(c->gexec);
        c->gexec = nullptr;
      }
      c->have_key = false;
      if ((st = upload_batch<T>(c, n, plans, aoff, sv_off, false, &w_off))) return st;
      if (mode == TB_MODE_FUSED) {
        // items longest first: blocks start roughly in index order, and the
        // longest networks bound the launch
        c->small_order.resize(n);
        for (int i = 0; i < n; i++) c->small_order[i] = i;
        std::stable_sort(c->small_order.begin(), c->small_order.end(),
                         [&](int a, int b) { return plans[a]->h.small_cost > plans[b]->h.small_cost; });
        CU(c->small_order_dev.ensure(sizeof(int32_t) * n));
        CU(cudaMemcpyAsync(c->small_order_dev.p, c->small_order.data(), sizeof(int32_t) * n,
                           cudaMemcpyHostToDevice, c->stream));
      }
      CU(cudaStreamSynchronize(c->stream));
      c->key = key;
      c->have_key = true;
      c->n_items = n;
      c->sv_bytes = sv;
      if (c->opt.use_graphs) {
        cudaGraph_t g;
        CU(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        int64_t l2 = 0;
        cudaError_t e = cudaMemcpyAsync(c->rvals.p, h_r, sizeof(float) * n, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess && sv) e = cudaMemcpyAsync(c->slice_vals.p, h_sv, sv, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(c->wvals.p, h_w, w_bytes, cudaMemcpyHostToDevice, c->stream);
        if (e != cudaSuccess) {
          cudaStreamEndCapture(c->stream, &g);
          return fail(TB_ERR_CUDA, cudaGetErrorString(e));
        }
        st = enqueue_batched<T>(c, n, mode, done_words, l2);
        cudaError_t e1 = cudaMemcpyAsync(hout, c->out_item.p, sizeof(float) * (n + 1), cudaMemcpyDeviceToHost,
                                         c->stream);
        cudaError_t e2 = cudaStreamEndCapture(c->stream, &g);
        if (st) return st;
        if (e1 != cudaSuccess) return fail(TB_ERR_CUDA, cudaGetErrorString(e1));
        if (e2 != cudaSuccess) return fail(TB_ERR_CUDA, cudaGetErrorString(e2));
        cudaError_t e3 = cudaGraphInstantiate(&c->gexec, g, 0);
        cudaGraphDestroy(g);
        if (e3 != cudaSuccess) return fail(TB_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e3));
        c->launches_graph = l2;
      }
    }
    if (c->opt.use_graphs && c->gexec) {
      CU(cudaGraphLaunch(c->gexec, c->stream));
      launches += c->launches_graph;
    } else {
      CU(cudaMemcpyAsync(c->rvals.p, h_r, sizeof(float) * n, cudaMemcpyHostToDevice, c->stream));
      if (sv) CU(cudaMemcpyAsync(c->slice_vals.p, h_sv, sv, cudaMemcpyHostToDevice, c->stream));
      CU(cudaMemcpyAsync(c->wvals.p, h_w, w_bytes, cudaMemcpyHostToDevice, c->stream));
      if ((st = enqueue_batched<T>(c, n, mode, done_words, launches))) return st;
      CU(cudaMemcpyAsync(hout, c->out_item.p, sizeof(float) * (n + 1), cudaMemcpyDeviceToHost, c->stream));
    }
    CU(cudaEventRecord(c->ev1, c->stream));
    CU(cudaEventSynchronize(c->ev1));
    {
      int err = 0;
      CU(cudaMemcpy(&err, reinterpret_cast<char*>(c->misc.p) + 16, sizeof(int), cudaMemcpyDeviceToHost));
      if (err) {
        c->have_key = false;
        return fail(TB_ERR_TIMEOUT, "a bounded device-side wait timed out");
      }
    }
  }
  float ms = 0;
  cudaEventElapsedTime(&ms, c->ev0, c->ev1);
  c->last_ms = ms;
  c->last_launches = launches;
  if (out_item) std::memcpy(out_item, hout, sizeof(float) * n);
  if (out_max) *out_max = hout[n];
  return TB_OK;
}

// ---------------------------------------------------------------------------
// Autotuner: tile shapes, then the executor's schedule, by timing the batch.
// ---------------------------------------------------------------------------
static void retile_all(tb_ctx* c, const std::vector<tb_plan*>& uniq, int bits, std::string& err) {
  for (tb_plan* p : uniq) {
    if (p->h.tile_bits == bits) continue;
    std::string e = retile_plan(p->h, bits);
    if (!e.empty()) {
      err = e;
      return;
    }
    p->structure_uploaded = false;
    p->version = ++c->plan_counter;
  }
}

static tb_status time_batch(tb_ctx* c, int n, tb_plan* const* plans, const int8_t* sv, const float* r, int mode,
                            double& best_ms) {
  tb_status st = TB_OK;
  best_ms = 1e30;
  for (int rep = 0; rep < 3; rep++) {  // first run builds the batch and its graph
    st = c->opt.dtype == TB_DTYPE_F32 ? solve_batch_t<float>(c, n, plans, sv, r, nullptr, nullptr, mode)
                                      : solve_batch_t<int32_t>(c, n, plans, sv, r, nullptr, nullptr, mode);
    if (st) return st;
    if (rep > 0) best_ms = std::min(best_ms, c->last_ms);
  }
  return TB_OK;
}

static tb_status autotune_locked(tb_ctx* c, int n, tb_plan* const* plans, const int8_t* sv, const float* r,
                                 tb_tune_result* out) {
  std::vector<tb_plan*> uniq;
  for (int i = 0; i < n; i++)
    if (std::find(uniq.begin(), uniq.end(), plans[i]) == uniq.end()) uniq.push_back(plans[i]);
  tb_tune_result res{};
  res.n_tried = 0;
  std::string err;
  tb_status st;
  // the defaults first, as the reference point
  const int base_bits = uniq.empty() ? 9 : uniq[0]->h.tile_bits;
  c->chunk_div = 4;
  c->persistent_ctas = c->opt.persistent_ctas > 0 ? c->opt.persistent_ctas : c->ctas_per_sm_max * c->sms;
  double ms;
  if ((st = time_batch(c, n, plans, sv, r, TB_MODE_BATCHED, ms))) return st;
  res.ms_default = ms;
  res.n_tried++;
  // 1. stream tile size under both schedules (per-level launches and the
  // persistent executor prefer different tile sizes)
  // (per-level launches in both register budgets of the stream kernel)
  int best_bits = base_bits, best_mode = TB_MODE_BATCHED, batched_bits = base_bits;
  bool best_wide = false;
  double best = ms, best_batched = ms;
  for (int bits = 8; bits <= 11; bits++) {
    retile_all(c, uniq, bits, err);
    if (!err.empty()) return fail(TB_ERR_INVALID, "autotune: " + err);
    for (int form = 0; form < 3; form++) {
      const int mode = form == 0 ? TB_MODE_BATCHED : TB_MODE_LAYERED;
      if (bits == base_bits && mode == TB_MODE_BATCHED) continue;  // timed above
      c->stream_wide = form == 2;
      if ((st = time_batch(c, n, plans, sv, r, mode, ms))) return st;
      res.n_tried++;
      if (ms < best) {
        best = ms;
        best_bits = bits;
        best_mode = mode;
        best_wide = c->stream_wide;
      }
      if (mode == TB_MODE_BATCHED && ms < best_batched) {
        best_batched = ms;
        batched_bits = bits;
      }
    }
  }
  c->stream_wide = best_wide;
  // 2. the persistent executor with 1..max CTAs per SM and coarser or finer
  // runs of stream tiles, at its own best tile size
  int best_cps = c->ctas_per_sm_max, best_div = 4;
  if (c->opt.persistent_ctas <= 0) {
    retile_all(c, uniq, batched_bits, err);
    if (!err.empty()) return fail(TB_ERR_INVALID, "autotune: " + err);
    for (int cps = 1; cps <= c->ctas_per_sm_max; cps++) {
      for (int div : {1, 4, 16}) {
        if (cps == c->ctas_per_sm_max && div == 4) continue;  // timed above
        c->persistent_ctas = cps * c->sms;
        c->chunk_div = div;
        if ((st = time_batch(c, n, plans, sv, r, TB_MODE_BATCHED, ms))) return st;
        res.n_tried++;
        if (ms < best) {
          best = ms;
          best_mode = TB_MODE_BATCHED;
          best_bits = batched_bits;
          best_cps = cps;
          best_div = div;
        }
      }
    }
  }
  retile_all(c, uniq, best_bits, err);
  if (!err.empty()) return fail(TB_ERR_INVALID, "autotune: " + err);
  c->persistent_ctas = c->opt.persistent_ctas > 0 ? c->opt.persistent_ctas : best_cps * c->sms;
  c->chunk_div = best_div;
  c->tune_fallback = best_mode;
  // 3. split-K GEMM nodes: parts through partials and a max step, or by
  // atomic max into the output (where every value is >= 0 or -inf)
  bool has_split = false;
  for (tb_plan* p : uniq)
    for (const GemmDesc& g : p->h.gemms) has_split = has_split || g.ks_log2 > 0;
  bool best_atomic = c->kpart_atomic;
  if (has_split && best_mode != TB_MODE_FUSED) {
    c->kpart_atomic = !best_atomic;
    if ((st = time_batch(c, n, plans, sv, r, best_mode, ms))) return st;
    res.n_tried++;
    if (ms < best) {
      best = ms;
      best_atomic = c->kpart_atomic;
    }
    c->kpart_atomic = best_atomic;
  }
  // 4. the fused small form, when every plan has one
  bool all_small = true;
  for (tb_plan* p : uniq) all_small = all_small && p->h.small_ok;
  if (all_small) {
    if ((st = time_batch(c, n, plans, sv, r, TB_MODE_FUSED, ms))) return st;
    res.n_tried++;
    if (ms < best) {
      best = ms;
      best_mode = TB_MODE_FUSED;
    }
  }
  res.mode = best_mode;
  res.tile_bits = best_bits;
  res.ctas_per_sm = c->persistent_ctas / std::max(1, c->sms);
  res.chunk_div = best_div;
  res.stream_ctas_per_sm = (c->stream_wide ? c->stream_ctas_wide : c->stream_ctas) / std::max(1, c->sms);
  res.kpart_atomic = c->kpart_atomic ? 1 : 0;
  res.ms = best;
  c->tune = res;
  c->tuned = true;
  if (out) *out = res;
  return TB_OK;
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

tb_status tb_autotune(tb_ctx* c, int32_t n, tb_plan* const* plans, const int8_t* slice_vals, const float* r,
                      tb_tune_result* out) {
  if (!c) return fail(TB_ERR_INVALID, "null context");
  if (n <= 0 || !plans) return fail(TB_ERR_INVALID, "empty batch");
  std::lock_guard<std::mutex> lk(c->mu);
  try {
    return autotune_locked(c, n, plans, slice_vals, r, out);
  } catch (const std::exception& ex) {
    return fail(TB_ERR_INVALID, std::string("internal: ") + ex.what());
  }
}

void tb_options_default(tb_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->dtype = TB_DTYPE_F32;
  o->use_graphs = 1;
  o->max_device_bytes = 0;
  o->timeout_ms = 20000;
  o->autotune = 1;
  o->persistent_ctas = 0;
}

const char* tb_version(void) { return "tb 0.1 sm_103a"; }

const char* tb_last_error(const tb_ctx*) { return g_err.c_str(); }

tb_status tb_ctx_create(int32_t device, const tb_options* opt, tb_ctx** out) {
  if (!out) return fail(TB_ERR_INVALID, "out is null");
  *out = nullptr;
  int ndev = 0;
  CU(cudaGetDeviceCount(&ndev));
  if (device < 0 || device >= ndev) return fail(TB_ERR_INVALID, "no such CUDA device");
  std::unique_ptr<tb_ctx> c(new tb_ctx());
  c->device = device;
  if (opt) c->opt = *opt; else tb_options_default(&c->opt);
  if (c->opt.dtype != TB_DTYPE_F32 && c->opt.dtype != TB_DTYPE_I32) return fail(TB_ERR_INVALID, "unknown dtype");
  if (c->opt.timeout_ms <= 0) c->opt.timeout_ms = 20000;
  CU(cudaSetDevice(device));
  CU(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  CU(cudaEventCreate(&c->ev0));
  CU(cudaEventCreate(&c->ev1));
  CU(cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device));
  size_t fr = 0, tot = 0;
  CU(cudaMemGetInfo(&fr, &tot));
  c->budget = c->opt.max_device_bytes > 0 ? (size_t)c->opt.max_device_bytes : (size_t)(fr * 0.8);
  tb_status st = c->opt.dtype == TB_DTYPE_F32 ? set_kernel_attrs<float>() : set_kernel_attrs<int32_t>();
  if (st) return st;
  int per_sm = 0;
  if (c->opt.dtype == TB_DTYPE_F32)
    CU(occupancy_persistent<float>(&per_sm, max_stream_smem_bytes()));
  else
    CU(occupancy_persistent<int32_t>(&per_sm, max_stream_smem_bytes()));
  per_sm = std::max(1, per_sm);
  c->ctas_per_sm_max = per_sm;
  c->persistent_ctas = c->opt.persistent_ctas > 0 ? c->opt.persistent_ctas : per_sm * c->sms;
  int per_sm_stream = 0;
  if (c->opt.dtype == TB_DTYPE_F32)
    CU((occupancy_level<float, 1>(&per_sm_stream, smem_bytes(1))));
  else
    CU((occupancy_level<int32_t, 1>(&per_sm_stream, smem_bytes(1))));
  c->stream_ctas = std::max(1, per_sm_stream) * c->sms;
  int per_sm_wide = 0;
  if (c->opt.dtype == TB_DTYPE_F32)
    CU((occupancy_level<float, 5>(&per_sm_wide, smem_bytes(1))));
  else
    CU((occupancy_level<int32_t, 5>(&per_sm_wide, smem_bytes(1))));
  c->stream_ctas_wide = std::max(1, per_sm_wide) * c->sms;
  int per_sm_gemm = 0;
  if (c->opt.dtype == TB_DTYPE_F32)
    CU((occupancy_level<float, 2>(&per_sm_gemm, smem_bytes(2))));
  else
    CU((occupancy_level<int32_t, 2>(&per_sm_gemm, smem_bytes(2))));
  c->gemm_ctas = std::max(1, per_sm_gemm) * c->sms;
  *out = c.release();
  return TB_OK;
}

void tb_ctx_destroy(tb_ctx* c) {
  if (!c) return;
  {
    // plans that outlive their context keep only their own buffers
    std::lock_guard<std::mutex> lk(c->plans_mu);
    for (tb_plan* p : c->live_plans) p->ctx = nullptr;
    c->live_plans.clear();
  }
  cudaSetDevice(c->device);
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

tb_status tb_plan_create(tb_ctx* ctx, int32_t n_labels, int32_t n_tensors, const int32_t* ix_off,
                         const int32_t* ix_lab, int32_t n_iy, const int32_t* iy, int32_t n_nodes,
                         const int32_t* children, const int32_t* node_iy_off, const int32_t* node_iy_lab,
                         int32_t n_sliced, const int32_t* sliced, tb_plan** out) {
  if (!ctx || !out) return fail(TB_ERR_INVALID, "null argument");
  *out = nullptr;
  if (n_iy > 0 && !iy) return fail(TB_ERR_INVALID, "iy is null");
  if (n_nodes > 0 && !children) return fail(TB_ERR_INVALID, "children is null");
  if (n_sliced > 0 && !sliced) return fail(TB_ERR_INVALID, "sliced is null");
  if ((node_iy_off == nullptr) != (node_iy_lab == nullptr) && n_nodes > 0)
    return fail(TB_ERR_INVALID, "node_iy_off and node_iy_lab go together");
  PlanInput in;
  in.n_labels = n_labels;
  in.n_tensors = n_tensors;
  in.ix_off = ix_off;
  in.ix_lab = ix_lab;
  in.n_iy = n_iy;
  in.iy = iy;
  in.n_nodes = n_nodes;
  in.children = children;
  in.node_iy_off = node_iy_off;
  in.node_iy_lab = node_iy_lab;
  in.n_sliced = n_sliced;
  in.sliced = sliced;
  std::unique_ptr<tb_plan> p(new tb_plan());
  p->ctx = ctx;
  p->h.gemm_ctas = ctx->gemm_ctas;
  std::string e;
  try {
    e = compile_plan(in, p->h, 4);
  } catch (const std::exception& ex) {
    e = std::string("plan compiler: ") + ex.what();
  }
  if (!e.empty()) return fail(TB_ERR_INVALID, e);
  for (auto& lab : p->h.labels)
    if (lab.size() > 30) return fail(TB_ERR_UNSUPPORTED, "a tensor of rank > 30 (over 4 GiB)");
  p->version = ++ctx->plan_counter;
  {
    std::lock_guard<std::mutex> lk(ctx->plans_mu);
    ctx->live_plans.insert(p.get());
  }
  *out = p.release();
  return TB_OK;
}

void tb_plan_destroy(tb_plan* p) {
  if (!p) return;
  if (p->ctx) {
    {
      std::lock_guard<std::mutex> lk(p->ctx->plans_mu);
      p->ctx->live_plans.erase(p);
    }
    if (p->ctx->have_key) {
      for (auto* q : p->ctx->key.plans)
        if (q == p) {
          p->ctx->have_key = false;
          break;
        }
    }
  }
  delete p;
}

tb_status tb_plan_stats_get(const tb_plan* p, tb_plan_stats* o) {
  if (!p || !o) return fail(TB_ERR_INVALID, "null argument");
  std::memset(o, 0, sizeof(*o));
  o->tc = p->h.tc;
  o->sc = p->h.sc;
  o->rwc = p->h.rwc;
  o->ops = p->h.ops;
  o->bytes = p->h.bytes;
  o->arena_bytes = p->h.arena_elems * 4;
  o->n_steps = (int32_t)p->h.steps.size();
  o->n_tensors = p->h.n_tensors;
  o->n_open = (int32_t)p->h.open.size();
  o->n_sliced = (int32_t)p->h.sliced.size();
  o->n_tiles = (int32_t)std::min<int64_t>(p->h.total_tiles, 0x7fffffff);
  o->small_words = p->h.small_ok ? p->h.small_words : 0;
  return TB_OK;
}

tb_status tb_plan_node_labels(const tb_plan* p, int32_t node, int32_t cap, int32_t* labels_out, int32_t* n_out) {
  if (!p || !n_out) return fail(TB_ERR_INVALID, "null argument");
  if (node < 0 || node >= p->h.n_nodes) return fail(TB_ERR_INVALID, "node out of range");
  const auto& l = p->h.labels[p->h.n_tensors + node];
  *n_out = (int32_t)l.size();
  for (int i = 0; i < (int)l.size() && i < cap; i++) labels_out[i] = l[i];
  return TB_OK;
}

tb_status tb_plan_bind_mis(tb_plan* p, const float* w) {
  if (!p || !w) return fail(TB_ERR_INVALID, "null argument");
  if (!p->ctx) return fail(TB_ERR_INVALID, "the plan's context was destroyed");
  if (!p->mis_checked) {
    for (int i = 0; i < p->h.n_tensors; i++) {
      if (p->h.leaves[i].nraw < 1 || p->h.leaves[i].nraw > 2)
        return fail(TB_ERR_INVALID, "independent-set leaves have one (vertex) or two (edge) labels");
      if (p->h.leaves[i].nraw == 1) p->vertex_leaves.push_back(i);
    }
    // the usual layout: vertex leaf k carries label k
    p->vertex_dense = true;
    for (size_t k = 0; k < p->vertex_leaves.size(); k++)
      p->vertex_dense = p->vertex_dense && p->h.leaves[p->vertex_leaves[k]].label == (int32_t)k;
    p->mis_checked = true;
  }
  // the same weights again: nothing changes (they were checked when bound)
  if (p->h.has_weights && p->weights.size() == (size_t)p->h.n_labels &&
      std::memcmp(p->weights.data(), w, sizeof(float) * p->h.n_labels) == 0)
    return TB_OK;
  const bool is_int = p->ctx->opt.dtype == TB_DTYPE_I32;
  // every finite tensor value is an integer in [0, 8191] when the weights
  // are integers >= 0 summing below 8192: the GEMM tiles may then add and max
  // them as packed int16 exactly.  One pass without branches (contiguous in
  // the usual layout), the errors after it.
  double sum = 0;
  bool finite = true, integral = true, nonneg = true;
  float maxabs = 0.0f;
  auto scan = [&](float x) {
    finite &= std::isfinite(x);
    integral &= x == std::trunc(x);
    nonneg &= x >= 0.0f;
    maxabs = std::max(maxabs, std::fabs(x));
    sum += x;
  };
  if (p->vertex_dense) {
    const int nv = (int)p->vertex_leaves.size();
    for (int k = 0; k < nv; k++) scan(w[k]);
  } else {
    for (int i : p->vertex_leaves) scan(w[p->h.leaves[i].label]);
  }
  if (!finite) return fail(TB_ERR_INVALID, "weights must be finite");
  if (is_int && (!integral || maxabs > 1e8f))
    return fail(TB_ERR_INVALID, "int32 weights must be integers of magnitude below 1e8");
  const bool ok16 = integral && nonneg && sum < 8192;
  // the weights travel with each solve (one staged copy for the whole
  // batch); LeafDesc::w is refreshed only for the paths that read it
  p->weights.assign(w, w + p->h.n_labels);
  p->h.has_weights = true;
  p->leaves_dirty = true;
  p->wgen++;
  if (ok16 != p->i16_ok || nonneg != p->nonneg_ok) {
    p->i16_ok = ok16;
    p->nonneg_ok = nonneg;
    p->version = ++p->ctx->plan_counter;  // captured batches hold the flags
  }
  return TB_OK;
}

tb_status tb_score_trees(tb_ctx* c, int32_t n_labels, int32_t n_tensors, const int32_t* ix_off,
                         const int32_t* ix_lab, int32_t n_iy, const int32_t* iy, int32_t n_trees,
                         const int32_t* children, double* out) {
  if (!c || !ix_off || !out || (n_trees > 0 && n_tensors > 1 && !children)) return fail(TB_ERR_INVALID, "null argument");
  if (n_tensors < 1 || n_trees < 1) return fail(TB_ERR_INVALID, "no tensors or no trees");
  if (n_labels < 1 || n_labels > 4096) return fail(TB_ERR_UNSUPPORTED, "tree scoring takes 1..4096 labels");
  if (n_iy < 0 || (n_iy > 0 && !iy)) return fail(TB_ERR_INVALID, "bad iy");
  const int T = n_tensors, nodes = T - 1, nn = 2 * T - 1, W = (n_labels + 31) / 32;
  std::vector<uint32_t> leaf((size_t)T * W, 0), iyb(W, 0);
  if (ix_off[0] != 0) return fail(TB_ERR_INVALID, "ix_off[0] must be 0");
  for (int i = 0; i < T; i++) {
    if (ix_off[i + 1] < ix_off[i]) return fail(TB_ERR_INVALID, "ix_off not monotone");
    for (int k = ix_off[i]; k < ix_off[i + 1]; k++) {
      const int l = ix_lab[k];
      if (l < 0 || l >= n_labels) return fail(TB_ERR_INVALID, "label out of range");
      leaf[(size_t)i * W + l / 32] |= 1u << (l % 32);
    }
  }
  for (int k = 0; k < n_iy; k++) {
    if (iy[k] < 0 || iy[k] >= n_labels) return fail(TB_ERR_INVALID, "open label out of range");
    iyb[iy[k] / 32] |= 1u << (iy[k] % 32);
  }
  // every tree: post-order pairs over ids < T + j, each id used once
  std::vector<char> used(nn);
  for (int tr = 0; tr < n_trees; tr++) {
    std::fill(used.begin(), used.end(), 0);
    const int32_t* ch = children + (size_t)tr * 2 * nodes;
    for (int j = 0; j < nodes; j++)
      for (int q = 0; q < 2; q++) {
        const int x = ch[2 * j + q];
        if (x < 0 || x >= T + j || used[x]) return fail(TB_ERR_INVALID, "tree " + std::to_string(tr) + " is not a post-order binary tree");
        used[x] = 1;
      }
  }
  std::lock_guard<std::mutex> lk(c->mu);
  CU(cudaSetDevice(c->device));
  int warps = std::min(n_trees, 16 * c->sms);
  const size_t per_warp = (size_t)2 * nn * W + nn;
  while (warps > 8 && (size_t)((warps + 7) / 8 * 8) * per_warp * 4 > ((size_t)1 << 30)) warps /= 2;
  const size_t scratch_words = (size_t)((warps + 7) / 8 * 8) * per_warp;
  DevBuf d_leaf, d_iy, d_ch, d_out, d_scr;
  CU(d_leaf.ensure(leaf.size() * 4));
  CU(d_iy.ensure(iyb.size() * 4 + 4));
  CU(d_ch.ensure(std::max<size_t>((size_t)n_trees * 2 * nodes * 4, 4)));
  CU(d_out.ensure((size_t)n_trees * 4 * sizeof(double)));
  CU(d_scr.ensure(scratch_words * 4));
  CU(cudaMemcpyAsync(d_leaf.p, leaf.data(), leaf.size() * 4, cudaMemcpyHostToDevice, c->stream));
  CU(cudaMemcpyAsync(d_iy.p, iyb.data(), iyb.size() * 4, cudaMemcpyHostToDevice, c->stream));
  if (nodes > 0)
    CU(cudaMemcpyAsync(d_ch.p, children, (size_t)n_trees * 2 * nodes * 4, cudaMemcpyHostToDevice, c->stream));
  CU(launch_score_trees(warps, c->stream, n_trees, T, W, reinterpret_cast<const uint32_t*>(d_leaf.p),
                        reinterpret_cast<const uint32_t*>(d_iy.p), reinterpret_cast<const int32_t*>(d_ch.p),
                        reinterpret_cast<uint32_t*>(d_scr.p), reinterpret_cast<double*>(d_out.p)));
  CU(cudaMemcpyAsync(out, d_out.p, (size_t)n_trees * 4 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CU(cudaStreamSynchronize(c->stream));
  return TB_OK;
}

tb_status tb_plan_bind_mis_batch(int32_t n, tb_plan* const* plans, const float* weights, const int64_t* offsets) {
  if (n < 0 || (n > 0 && (!plans || !weights || !offsets))) return fail(TB_ERR_INVALID, "null argument");
  for (int32_t i = 0; i < n; i++) {
    tb_status st = tb_plan_bind_mis(plans[i], weights + offsets[i]);
    if (st) return st;
  }
  return TB_OK;
}

tb_status tb_solve_batch(tb_ctx* c, int32_t n, tb_plan* const* plans, const int8_t* slice_vals, const float* r,
                         float* out_item, float* out_max, int32_t mode) {
  if (!c) return fail(TB_ERR_INVALID, "null context");
  if (n <= 0 || !plans) return fail(TB_ERR_INVALID, "empty batch");
  if (mode != TB_MODE_PLAIN && mode != TB_MODE_BATCHED && mode != TB_MODE_LAYERED && mode != TB_MODE_AUTO &&
      mode != TB_MODE_FUSED)
    return fail(TB_ERR_INVALID, "unknown mode");
  std::lock_guard<std::mutex> lk(c->mu);
  try {
    if (mode == TB_MODE_AUTO) {
      if (!c->tuned && c->opt.autotune) {
        tb_status st = autotune_locked(c, n, plans, slice_vals, r, nullptr);
        if (st) return st;
      }
      mode = c->tuned ? c->tune.mode : TB_MODE_BATCHED;
      if (mode == TB_MODE_FUSED)
        for (int32_t i = 0; i < n; i++)
          if (plans[i] && !plans[i]->h.small_ok) {
            mode = c->tune_fallback;
            break;
          }
    }
    if (c->opt.dtype == TB_DTYPE_F32) return solve_batch_t<float>(c, n, plans, slice_vals, r, out_item, out_max, mode);
    return solve_batch_t<int32_t>(c, n, plans, slice_vals, r, out_item, out_max, mode);
  } catch (const std::exception& ex) {
    return fail(TB_ERR_INVALID, std::string("internal: ") + ex.what());
  }
}

}  // extern "C"

// leaf data with raw labels -> stored (distinct) labels: diagonal of repeats
static std::vector<float> leaf_stored(const std::vector<int32_t>& raw, const std::vector<int32_t>& stored,
                                      const float* data) {
  std::vector<float> out((size_t)1 << stored.size());
  for (size_t e = 0; e < out.size(); e++) {
    size_t x = 0;
    for (size_t k = 0; k < raw.size(); k++) {
      int b = -1;
      for (size_t q = 0; q < stored.size(); q++)
        if (stored[q] == raw[k]) b = (int)q;
      x |= (size_t)((e >> b) & 1) << k;
    }
    out[e] = data[x];
  }
  return out;
}

template <typename T>
static tb_status run_single(tb_ctx* c, tb_plan* p, const float* const* leaf_data, const int8_t* slice_vals,
                            int mode) {
  CU(cudaSetDevice(c->device));
  tb_status st = set_kernel_attrs<T>();
  if (st) return st;
  if ((st = upload_plan(p, true))) return st;
  const PlanHost& h = p->h;
  int64_t need = mode == TB_MODE_PLAIN ? h.plain_elems : h.arena_elems;
  size_t bytes = (size_t)need * sizeof(T) + 256;
  if (bytes > c->budget) return fail(TB_ERR_OOM, "plan needs more device memory than the budget");
  CU(c->arena.ensure(bytes));
  T* arena = reinterpret_cast<T*>(c->arena.p);
  size_t sv = h.sliced.size();
  CU(c->slice_vals.ensure(std::max<size_t>(sv, 16)));
  if (sv) CU(cudaMemcpy(c->slice_vals.p, slice_vals, sv, cudaMemcpyHostToDevice));
  if (leaf_data) {
    for (int i = 0; i < h.n_tensors; i++) {
      std::vector<float> v = leaf_stored(h.leaf_raw[i], h.labels[i], leaf_data[i]);
      if (std::is_same<T, float>::value) {
        CU(cudaMemcpy(arena + h.off[i], v.data(), v.size() * 4, cudaMemcpyHostToDevice));
      } else {
        std::vector<int32_t> iv(v.size());
        for (size_t k = 0; k < v.size(); k++) iv[k] = std::isinf(v[k]) ? TB_I32_NEG : (int32_t)v[k];
        CU(cudaMemcpy(arena + h.off[i], iv.data(), iv.size() * 4, cudaMemcpyHostToDevice));
      }
    }
  }
  int64_t launches = 0;
  const int8_t* d_sv = reinterpret_cast<const int8_t*>(c->slice_vals.p);
  if (mode == TB_MODE_PLAIN) {
    if ((st = plain_item<T>(c, p, arena, d_sv, leaf_data == nullptr, nullptr, launches))) return st;
  } else {
    // fused tiles, one launch per level for this single item
    std::vector<int64_t> aoff{0}, svo{0};
    tb_plan* pl[1] = {p};
    c->have_key = false;
    if (c->gexec) {
      cudaGraphExecDestroy(c->gexec);
      c->gexec = nullptr;
    }
    if ((st = upload_batch<T>(c, 1, pl, aoff, svo, leaf_data != nullptr, nullptr))) return st;
    CU(c->out_item.ensure(sizeof(float) * 2));
    CU(cudaMemsetAsync(c->misc.p, 0, 64, c->stream));
    const int smem = max_stream_smem_bytes();
    int* err = reinterpret_cast<int*>(reinterpret_cast<char*>(c->misc.p) + 16);
    const ItemDev<T>* items = reinterpret_cast<const ItemDev<T>*>(c->items.p);
    const Group* groups = reinterpret_cast<const Group*>(c->groups.p);
    float* oi = reinterpret_cast<float*>(c->out_item.p);
    for (auto& lr : c->level_ranges) {
      CU(launch_range<T>(c, lr, c->stream, items, groups, oi, nullptr, err));
      CU(cudaGetLastError());
    }
  }
  CU(cudaStreamSynchronize(c->stream));
  if (mode != TB_MODE_PLAIN) {
    int err = 0;
    CU(cudaMemcpy(&err, reinterpret_cast<char*>(c->misc.p) + 16, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) return fail(TB_ERR_TIMEOUT, "a bounded device-side wait timed out");
  }
  return TB_OK;
}

// Device layout (fused form) -> reported layout of tensor id, on the host.
static std::vector<float> to_reported(const PlanHost& h, int id, const std::vector<float>& v) {
  const auto& from = h.flabels[id];
  const auto& to = h.labels[id];
  if (from == to) return v;
  std::vector<int> pos(to.size());
  for (size_t q = 0; q < to.size(); q++)
    for (size_t r = 0; r < from.size(); r++)
      if (from[r] == to[q]) pos[q] = (int)r;
  std::vector<float> out(v.size());
  for (size_t e = 0; e < v.size(); e++) {
    size_t x = 0;
    for (size_t q = 0; q < to.size(); q++) x |= ((e >> q) & 1) << pos[q];
    out[e] = v[x];
  }
  return out;
}

extern "C" {

tb_status tb_contract(tb_ctx* c, tb_plan* p, const float* const* leaf_data, float* out, int32_t mode) {
  if (!c || !p || !leaf_data || !out) return fail(TB_ERR_INVALID, "null argument");
  if (!p->h.sliced.empty()) return fail(TB_ERR_INVALID, "tb_contract does not take sliced plans");
  std::lock_guard<std::mutex> lk(c->mu);
  tb_status st = c->opt.dtype == TB_DTYPE_F32 ? run_single<float>(c, p, leaf_data, nullptr, mode)
                                              : run_single<int32_t>(c, p, leaf_data, nullptr, mode);
  if (st) return st;
  const PlanHost& h = p->h;
  size_t n = (size_t)1 << h.fin.root_log2;
  if (c->opt.dtype == TB_DTYPE_F32) {
    CU(cudaMemcpy(out, reinterpret_cast<float*>(c->arena.p) + h.fin.root_off, n * 4, cudaMemcpyDeviceToHost));
  } else {
    std::vector<int32_t> iv(n);
    CU(cudaMemcpy(iv.data(), reinterpret_cast<int32_t*>(c->arena.p) + h.fin.root_off, n * 4, cudaMemcpyDeviceToHost));
    for (size_t k = 0; k < n; k++) out[k] = iv[k] <= TB_I32_NEG / 2 ? -INFINITY : (float)iv[k];
  }
  return TB_OK;
}

tb_status tb_dump_intermediates(tb_ctx* c, tb_plan* p, const int8_t* slice_vals, float* const* node_out,
                                int32_t mode) {
  if (!c || !p || !node_out) return fail(TB_ERR_INVALID, "null argument");
  if (!p->h.has_weights) return fail(TB_ERR_INVALID, "plan has no bound weights");
  if (!p->h.sliced.empty() && !slice_vals) return fail(TB_ERR_INVALID, "slice_vals required");
  std::lock_guard<std::mutex> lk(c->mu);
  tb_status st = c->opt.dtype == TB_DTYPE_F32 ? run_single<float>(c, p, nullptr, slice_vals, mode)
                                              : run_single<int32_t>(c, p, nullptr, slice_vals, mode);
  if (st) return st;
  const PlanHost& h = p->h;
  for (int j = 0; j < h.n_nodes; j++) {
    if (!node_out[j]) continue;
    int id = h.n_tensors + j;
    size_t n = (size_t)1 << h.labels[id].size();
    std::vector<float> v(n);
    if (c->opt.dtype == TB_DTYPE_F32) {
      CU(cudaMemcpy(v.data(), reinterpret_cast<float*>(c->arena.p) + h.off[id], n * 4, cudaMemcpyDeviceToHost));
    } else {
      std::vector<int32_t> iv(n);
      CU(cudaMemcpy(iv.data(), reinterpret_cast<int32_t*>(c->arena.p) + h.off[id], n * 4, cudaMemcpyDeviceToHost));
      for (size_t k = 0; k < n; k++) v[k] = iv[k] <= TB_I32_NEG / 2 ? -INFINITY : (float)iv[k];
    }
    if (mode != TB_MODE_PLAIN) v = to_reported(h, id, v);
    std::memcpy(node_out[j], v.data(), n * 4);
  }
  return TB_OK;
}

tb_status tb_last_timing(const tb_ctx* c, double* ms, int64_t* launches) {
  if (!c) return fail(TB_ERR_INVALID, "null context");
  if (ms) *ms = c->last_ms;
  if (launches) *launches = c->last_launches;
  return TB_OK;
}

tb_status tb_gemm_device(tb_ctx* c, int64_t M, int64_t N, int64_t K, int64_t batch, const void* A, const void* B,
                         void* C, void* stream) {
  if (!c || !A || !B || !C) return fail(TB_ERR_INVALID, "null argument");
  auto pow2 = [](int64_t x) { return x > 0 && (x & (x - 1)) == 0; };
  if (!pow2(M) || !pow2(N) || !pow2(K) || batch < 1 || M < 16 || N < 16 || K < 16)
    return fail(TB_ERR_UNSUPPORTED, "K1 takes power-of-two M, N, K >= 16");
  if (M > (1 << 30) || N > (1 << 30) || K > (1 << 30)) return fail(TB_ERR_UNSUPPORTED, "dimension too large");
  CU(cudaSetDevice(c->device));
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);  // NULL: the default stream
  if (c->opt.dtype == TB_DTYPE_F32) {
    CU(launch_k1_any<float>((const float*)A, (const float*)B, (float*)C, M, N, K, batch, s));
  } else {
    CU(launch_k1_any<int32_t>((const int32_t*)A, (const int32_t*)B, (int32_t*)C, M, N, K, batch, s));
  }
  return TB_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Internal (not part of include/tb.h): compile a plan on the host only and
// hand back its device program as one blob, so tests can check the kernels'
// index arithmetic on a machine without a GPU.  Layout:
//   int64 header[8] = {n_tensors, n_nodes, n_steps, n_tiles, n_leaves,
//                      arena_elems, plain_elems, n_plain_ops}
//   int64 off[n_tensors + n_nodes]; int32 rank[n_tensors + n_nodes]
//   Step steps[]; TileDesc tiles[]; LeafDesc leaves[]; FinalDesc fin;
//   per plain op: int32 node, int32 kind, TileDesc tile, int64 a,b,c,M,N,K,batch
// ---------------------------------------------------------------------------
extern "C" int32_t tbi_plan_describe(int32_t n_labels, int32_t n_tensors, const int32_t* ix_off,
                                     const int32_t* ix_lab, int32_t n_iy, const int32_t* iy, int32_t n_nodes,
                                     const int32_t* children, const int32_t* node_iy_off,
                                     const int32_t* node_iy_lab, int32_t n_sliced, const int32_t* sliced,
                                     int32_t gemm_min, int32_t tile_bits, void** blob, int64_t* blob_bytes,
                                     char* err, int32_t err_cap) {
  PlanInput in;
  in.n_labels = n_labels; in.n_tensors = n_tensors; in.ix_off = ix_off; in.ix_lab = ix_lab;
  in.n_iy = n_iy; in.iy = iy; in.n_nodes = n_nodes; in.children = children;
  in.node_iy_off = node_iy_off; in.node_iy_lab = node_iy_lab; in.n_sliced = n_sliced; in.sliced = sliced;
  PlanHost h;
  std::string e = compile_plan(in, h, gemm_min);
  if (e.empty() && tile_bits != h.tile_bits) e = retile_plan(h, tile_bits);
  if (!e.empty()) {
    if (err && err_cap > 0) {
      std::strncpy(err, e.c_str(), err_cap - 1);
      err[err_cap - 1] = 0;
    }
    return TB_ERR_INVALID;
  }
  int64_t total = h.n_tensors + h.n_nodes;
  int64_t nplain = 0;
  for (auto& v : h.plain) nplain += (int64_t)v.size();
  int64_t nlab = 0;
  for (int64_t i = 0; i < total; i++) nlab += (int64_t)h.labels[i].size();
  struct PlainRec { int32_t node, kind; TileDesc tile; int64_t a, b, c, M, N, K, batch; };
  size_t bytes = 8 * 9 + total * 8 + total * 4 + nlab * 8 + h.steps.size() * sizeof(Step) +
                 h.tiles.size() * sizeof(TileDesc) + h.leaves.size() * sizeof(LeafDesc) + sizeof(FinalDesc) +
                 h.gemms.size() * sizeof(GemmDesc) + nplain * sizeof(PlainRec) + h.steps.size() * sizeof(Step) +
                 h.gemms.size() * sizeof(GemmDesc);
  char* b = (char*)std::malloc(bytes);
  if (!b) return TB_ERR_OOM;
  char* p = b;
  int64_t hdr[9] = {h.n_tensors, h.n_nodes, (int64_t)h.steps.size(), (int64_t)h.tiles.size(),
                    (int64_t)h.leaves.size(), h.arena_elems, h.plain_elems, nplain, (int64_t)h.gemms.size()};
  std::memcpy(p, hdr, sizeof(hdr)); p += sizeof(hdr);
  std::memcpy(p, h.off.data(), total * 8); p += total * 8;
  for (int64_t i = 0; i < total; i++) { int32_t r = (int32_t)h.labels[i].size(); std::memcpy(p, &r, 4); p += 4; }
  for (int64_t i = 0; i < total; i++) {
    std::memcpy(p, h.labels[i].data(), h.labels[i].size() * 4); p += h.labels[i].size() * 4;
    std::memcpy(p, h.flabels[i].data(), h.flabels[i].size() * 4); p += h.flabels[i].size() * 4;
  }
  std::memcpy(p, h.steps.data(), h.steps.size() * sizeof(Step)); p += h.steps.size() * sizeof(Step);
  if (!h.tiles.empty()) std::memcpy(p, h.tiles.data(), h.tiles.size() * sizeof(TileDesc));
  p += h.tiles.size() * sizeof(TileDesc);
  std::memcpy(p, h.leaves.data(), h.leaves.size() * sizeof(LeafDesc)); p += h.leaves.size() * sizeof(LeafDesc);
  std::memcpy(p, &h.fin, sizeof(FinalDesc)); p += sizeof(FinalDesc);
  if (!h.gemms.empty()) std::memcpy(p, h.gemms.data(), h.gemms.size() * sizeof(GemmDesc));
  p += h.gemms.size() * sizeof(GemmDesc);
  for (int j = 0; j < h.n_nodes; j++)
    for (const PlainOp& op : h.plain[j]) {
      PlainRec rec;
      std::memset(&rec, 0, sizeof(rec));
      rec.node = j; rec.kind = op.kind; rec.tile = op.tile;
      rec.a = op.a_off; rec.b = op.b_off; rec.c = op.c_off; rec.M = op.M; rec.N = op.N; rec.K = op.K; rec.batch = op.batch;
      std::memcpy(p, &rec, sizeof(rec)); p += sizeof(rec);
    }
  // the merged split-K form, same counts as steps and gemms
  std::memcpy(p, h.steps_merged.data(), h.steps.size() * sizeof(Step)); p += h.steps.size() * sizeof(Step);
  if (!h.gemms.empty()) std::memcpy(p, h.gemms_merged.data(), h.gemms.size() * sizeof(GemmDesc));
  p += h.gemms.size() * sizeof(GemmDesc);
  *blob = b;
  *blob_bytes = (int64_t)bytes;
  return TB_OK;
}

// The fused small form of a plan (host only, for the CPU emulator): blob =
//   int32 {small_ok, n_small, n_leaves, words, root_off, root_log2};
//   SmallNode nodes[n_small]; int32 leaf_off[n_leaves]
extern "C" int32_t tbi_plan_small(int32_t n_labels, int32_t n_tensors, const int32_t* ix_off, const int32_t* ix_lab,
                                  int32_t n_iy, const int32_t* iy, int32_t n_nodes, const int32_t* children,
                                  int32_t n_sliced, const int32_t* sliced, void** blob, int64_t* blob_bytes,
                                  char* err, int32_t err_cap) {
  PlanInput in;
  in.n_labels = n_labels; in.n_tensors = n_tensors; in.ix_off = ix_off; in.ix_lab = ix_lab;
  in.n_iy = n_iy; in.iy = iy; in.n_nodes = n_nodes; in.children = children;
  in.n_sliced = n_sliced; in.sliced = sliced;
  PlanHost h;
  std::string e = compile_plan(in, h, 4);
  if (!e.empty()) {
    if (err && err_cap > 0) {
      std::strncpy(err, e.c_str(), err_cap - 1);
      err[err_cap - 1] = 0;
    }
    return TB_ERR_INVALID;
  }
  const size_t bytes = 6 * 4 + h.small.size() * sizeof(SmallNode) + h.small_leaf.size() * 4;
  char* b = (char*)std::malloc(bytes);
  if (!b) return TB_ERR_OOM;
  int32_t hdr[6] = {h.small_ok ? 1 : 0, (int32_t)h.small.size(), (int32_t)h.small_leaf.size(), h.small_words,
                    h.small_root, h.small_root_log2};
  char* q = b;
  std::memcpy(q, hdr, sizeof(hdr)); q += sizeof(hdr);
  if (!h.small.empty()) std::memcpy(q, h.small.data(), h.small.size() * sizeof(SmallNode));
  q += h.small.size() * sizeof(SmallNode);
  if (!h.small_leaf.empty()) std::memcpy(q, h.small_leaf.data(), h.small_leaf.size() * 4);
  *blob = b;
  *blob_bytes = (int64_t)bytes;
  return TB_OK;
}

extern "C" void tbi_free(void* p) { std::free(p); }

extern "C" int32_t tbi_sizes(int32_t* out, int32_t n) {
  int32_t v[6] = {(int32_t)sizeof(TileDesc), (int32_t)sizeof(Step), (int32_t)sizeof(LeafDesc),
                  (int32_t)sizeof(FinalDesc), (int32_t)sizeof(GemmDesc), (int32_t)sizeof(TinyDesc)};
  for (int i = 0; i < n && i < 6; i++) out[i] = v[i];
  return 0;
}

// Internal: the launch span level_span gives a range of `count` tickets
// from `first`, the first `tiny` of them tiny steps and the rest one-tile
// steps, on at most max_ctas CTAs: out7 = {grid, first, mid, last, chunk,
// chunk2, split_cta}.
extern "C" int32_t tbi_level_span(int64_t first, int64_t count, int64_t tiny, int64_t max_ctas, int64_t* out7) {
  if (!out7 || count < 1 || tiny < 0 || tiny > count) return TB_ERR_INVALID;
  tb_ctx::LevelRange lr{first, count, 1, 0, 0, tiny, (double)tiny * tiny_cost_us(0, 0),
                        (double)(count - tiny) * (kGroupCostUs + kTileCostUs)};
  int64_t grid = 0;
  const LevelSpan sp = level_span(lr, max_ctas, grid);
  const int64_t v[7] = {grid, sp.first, sp.mid, sp.last, sp.chunk, sp.chunk2, sp.split_cta};
  for (int i = 0; i < 7; i++) out7[i] = v[i];
  return TB_OK;
}

// Internal: the TinyDesc the engine uploads for a stream-tile descriptor;
// returns 1 when the step runs as a tiny step (tiny_node), else 0.
extern "C" int32_t tbi_tiny_desc(const TileDesc* d, TinyDesc* out) {
  if (!d || !out) return TB_ERR_INVALID;
  *out = make_tiny(*d);
  return tiny_step(*d) ? 1 : 0;
}

// ---------------------------------------------------------------------------
// Internal: measured SIMT max-plus peak (roofline denominator).  Sixteen
// loop-carried chains per thread of one packed add (add.f32x2) and one
// three-input max per two (max,+) pairs -- the inner step of the GEMM tiles
// -- so that no operand is loop-invariant.  Returns tropical ops/s (max and
// add counted as two ops).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_peak_f32(float* out, int iters, float seed) {
  constexpr int NC = 16;
  float f[NC];
  uint64_t x[NC];
#pragma unroll
  for (int j = 0; j < NC; j++) {
    f[j] = seed * (float)(j + threadIdx.x);
    float hi = f[j] + 1.0f;
    x[j] = ((uint64_t)__float_as_uint(hi) << 32) | __float_as_uint(f[j]);
  }
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int j = 0; j < NC; j++) {
      uint64_t s = add2(x[j], x[(j + 5) % NC]);
      f[j] = max3(f[j], lo32(s), hi32(s));
      x[j] = s;
    }
  }
  float s = 0;
#pragma unroll
  for (int j = 0; j < NC; j++) s += f[j] + lo32(x[j]);
  if (s == 1.2345f) out[0] = s;
}

// The same for the packed-int16 form: __viaddmax_s16x2, one instruction per
// two tropical MACs; every chain's operand comes from another chain's
// previous value, so nothing is loop-invariant.
__global__ void __launch_bounds__(256) k_peak_i16(unsigned* out, int iters, unsigned seed) {
  constexpr int NC = 16;
  unsigned x[NC];
#pragma unroll
  for (int j = 0; j < NC; j++) x[j] = (seed * (unsigned)(j + 1 + threadIdx.x)) & 0x0fff0fffu;
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int j = 0; j < NC; j++) x[j] = __viaddmax_s16x2(x[(j + 5) % NC], 0x00010001u, x[j]);
  }
  unsigned s = 0;
#pragma unroll
  for (int j = 0; j < NC; j++) s ^= x[j];
  if (s == 0x12345678u) out[0] = s;
}

// Resident CTAs of the context's kernels (stream tiles, GEMM tiles,
// persistent executor) and its SM count, for reports.
// Per-level stream launches in the 128-register form (1) or the 80-register
// form (0), as the autotuner may choose; for tests that pin one.
extern "C" int32_t tbi_ctx_set_stream_wide(tb_ctx* c, int32_t wide) {
  if (!c) return TB_ERR_INVALID;
  std::lock_guard<std::mutex> lk(c->mu);
  c->stream_wide = wide != 0;
  return TB_OK;
}

// The stream form the per-level launches use now: 1 for the 128-register
// k_level<T, 5>, 0 for the 80-register k_level<T, 1>, negative on error.
extern "C" int32_t tbi_ctx_stream_wide(tb_ctx* c) {
  if (!c) return TB_ERR_INVALID;
  std::lock_guard<std::mutex> lk(c->mu);
  return c->stream_wide ? 1 : 0;
}

// Split-K parts by atomic max into the output where every value is >= 0 or
// -inf (1), or through partials and a max step (0), as the autotuner may
// choose; for tests that pin one.
extern "C" int32_t tbi_ctx_set_kpart_atomic(tb_ctx* c, int32_t atomic) {
  if (!c) return TB_ERR_INVALID;
  std::lock_guard<std::mutex> lk(c->mu);
  c->kpart_atomic = atomic != 0;
  return TB_OK;
}

// Split-K GEMMs of batches whose items fill the GPU run merged (1, the
// default) or always as the plan split them (0); for tests that pin one.
extern "C" int32_t tbi_ctx_set_kpart_merge(tb_ctx* c, int32_t merge) {
  if (!c) return TB_ERR_INVALID;
  std::lock_guard<std::mutex> lk(c->mu);
  c->kpart_merge = merge != 0;
  return TB_OK;
}

extern "C" int32_t tbi_ctx_info(const tb_ctx* c, int32_t* out4) {
  if (!c || !out4) return TB_ERR_INVALID;
  out4[0] = c->stream_ctas;
  out4[1] = c->gemm_ctas;
  out4[2] = c->persistent_ctas;
  out4[3] = c->sms;
  return TB_OK;
}

// Test hook for the bounded waits of the persistent executor: one item whose
// chunk list keeps only the final step, so the wait on the root's done
// counter is never satisfied.  The wait gives up after timeout_ms, the kernel
// sets the error word and returns, and the hook returns TB_ERR_TIMEOUT; the
// context stays usable (the next batch is uploaded afresh).
extern "C" int32_t tbi_timeout_probe(tb_ctx* c, tb_plan* p, int32_t timeout_ms) {
  if (!c || !p || p->ctx != c || timeout_ms <= 0) return fail(TB_ERR_INVALID, "bad probe arguments");
  std::lock_guard<std::mutex> lk(c->mu);
  if (c->opt.dtype != TB_DTYPE_F32) return fail(TB_ERR_UNSUPPORTED, "the probe runs f32 contexts");
  if (!p->h.has_weights) return fail(TB_ERR_INVALID, "plan has no bound weights");
  CU(cudaSetDevice(c->device));
  tb_status st = set_kernel_attrs<float>();
  if (st) return st;
  if ((st = upload_plan(p, true))) return st;
  if (c->gexec) {
    cudaGraphExecDestroy(c->gexec);
    c->gexec = nullptr;
  }
  c->have_key = false;
  std::vector<int64_t> aoff(1, 0), svoff(1, 0);
  CU(c->arena.ensure((size_t)p->h.arena_elems * sizeof(float) + 256));
  CU(c->slice_vals.ensure(16));
  CU(c->out_item.ensure(sizeof(float) * 2));
  CU(c->rvals.ensure(16));
  if ((st = upload_batch<float>(c, 1, &p, aoff, svoff, false, nullptr))) return st;
  Chunk* ch = reinterpret_cast<Chunk*>(c->chunks.p);
  // the final step comes last (highest level): make it the only chunk
  CU(cudaMemcpyAsync(ch, ch + (c->n_chunks - 1), sizeof(Chunk), cudaMemcpyDeviceToDevice, c->stream));
  CU(cudaMemsetAsync(c->misc.p, 0, 64, c->stream));
  CU(cudaMemsetAsync(c->done.p, 0, sizeof(int) * p->h.steps.size(), c->stream));
  CU(cudaMemsetAsync(c->rvals.p, 0, 16, c->stream));
  unsigned long long* ticket = reinterpret_cast<unsigned long long*>(c->misc.p);
  int* err = reinterpret_cast<int*>(reinterpret_cast<char*>(c->misc.p) + 16);
  CU(launch_persistent<float>(c->persistent_ctas, max_stream_smem_bytes(), c->stream, 
      reinterpret_cast<const ItemDev<float>*>(c->items.p), reinterpret_cast<const Group*>(c->groups.p), ch, 1,
      reinterpret_cast<int*>(c->done.p), ticket, err, reinterpret_cast<float*>(c->out_item.p),
      reinterpret_cast<const float*>(c->rvals.p), (int64_t)timeout_ms * 1000000LL));
  CU(cudaGetLastError());
  CU(cudaStreamSynchronize(c->stream));
  int e = 0;
  CU(cudaMemcpy(&e, err, sizeof(int), cudaMemcpyDeviceToHost));
  c->have_key = false;
  if (e == TB_ERR_TIMEOUT) return fail(TB_ERR_TIMEOUT, "a bounded device-side wait timed out");
  return e ? fail(TB_ERR_CUDA, "unexpected device error word") : TB_OK;
}

// Per-launch profile of the per-level schedule (for the benchmark's
// roofline): solves the batch once in TB_MODE_LAYERED, then runs its level
// launches again without a graph, with a CUDA event after each, on the
// context's stream.  Per launch k < *n_out: device milliseconds, kind (1
// stream tiles with leaves / final steps, 2 GEMM tiles) and the algorithmic
// tropical ops (2 2^|L| per node) and bytes (4 (|A|+|B|+|C|) per node) of the
// contraction steps it runs (K-split max steps count none).  The batch must
// fit the context's budget in one wave.
template <typename T>
static tb_status profile_levels_t(tb_ctx* c, int n, tb_plan* const* plans, const int8_t* sv, const float* r,
                                  int cap, double* ms, int32_t* kinds, double* ops, double* bytes, int32_t* n_out) {
  tb_status st = solve_batch_t<T>(c, n, plans, sv, r, nullptr, nullptr, TB_MODE_LAYERED);
  if (st) return st;
  if (!c->have_key || c->n_items != n) return fail(TB_ERR_UNSUPPORTED, "the batch ran in waves");
  const int L = (int)c->level_ranges.size();
  if (L > cap) return fail(TB_ERR_INVALID, "more level launches than cap");
  std::vector<cudaEvent_t> ev(L + 1, nullptr);
  auto destroy = [&]() {
    for (cudaEvent_t e : ev)
      if (e) cudaEventDestroy(e);
  };
  for (auto& e : ev) {
    cudaError_t ce = cudaEventCreate(&e);
    if (ce != cudaSuccess) {
      destroy();
      return fail(TB_ERR_CUDA, cudaGetErrorString(ce));
    }
  }
  cudaError_t ce = cudaMemsetAsync(c->misc.p, 0, 64, c->stream);
  if (ce == cudaSuccess) ce = cudaEventRecord(ev[0], c->stream);
  for (int k = 0; k < L && ce == cudaSuccess && st == TB_OK; k++) {
    st = enqueue_level<T>(c, c->level_ranges[k]);
    if (st == TB_OK) ce = cudaEventRecord(ev[k + 1], c->stream);
  }
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(c->stream);
  if (st || ce != cudaSuccess) {
    destroy();
    return st ? st : fail(TB_ERR_CUDA, cudaGetErrorString(ce));
  }
  const Group* hg = reinterpret_cast<const Group*>(c->h_groups.p);
  int g = 0;
  for (int k = 0; k < L; k++) {
    const auto& lr = c->level_ranges[k];
    float t = 0;
    cudaEventElapsedTime(&t, ev[k], ev[k + 1]);
    ms[k] = t;
    kinds[k] = lr.kinds;
    ops[k] = bytes[k] = 0;
    for (; g < c->n_groups && hg[g].first < lr.first + lr.count; g++) {
      const PlanHost& h = plans[hg[g].item]->h;
      const int sn = h.step_node[hg[g].step];
      if (sn >= 0) {
        ops[k] += h.node_ops[sn];
        bytes[k] += h.node_bytes[sn];
      }
    }
  }
  destroy();
  *n_out = L;
  int err = 0;
  CU(cudaMemcpy(&err, reinterpret_cast<char*>(c->misc.p) + 16, sizeof(int), cudaMemcpyDeviceToHost));
  if (err) return fail(TB_ERR_TIMEOUT, "a bounded device-side wait timed out");
  return TB_OK;
}

extern "C" int32_t tbi_profile_levels(tb_ctx* c, int32_t n, tb_plan* const* plans, const int8_t* sv,
                                      const float* r, int32_t cap, double* ms, int32_t* kinds, double* ops,
                                      double* bytes, int32_t* n_out) {
  if (!c || n <= 0 || !plans || !ms || !kinds || !ops || !bytes || !n_out) return fail(TB_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(c->mu);
  try {
    return c->opt.dtype == TB_DTYPE_F32
               ? profile_levels_t<float>(c, n, plans, sv, r, cap, ms, kinds, ops, bytes, n_out)
               : profile_levels_t<int32_t>(c, n, plans, sv, r, cap, ms, kinds, ops, bytes, n_out);
  } catch (const std::exception& ex) {
    return fail(TB_ERR_INVALID, std::string("internal: ") + ex.what());
  }
}

// Measured packed-int16 max-plus rate (ops/s, a max and an add per MAC).
extern "C" int32_t tbi_measure_maxplus_peak_i16(int32_t device, double* ops_per_s) {
  if (!ops_per_s) return TB_ERR_INVALID;
  CU(cudaSetDevice(device));
  int sms = 0;
  CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  unsigned* out = nullptr;
  CU(cudaMalloc(&out, 64));
  cudaEvent_t e0, e1;
  CU(cudaEventCreate(&e0));
  CU(cudaEventCreate(&e1));
  const int blocks = sms * 8, iters = 4096;
  k_peak_i16<<<blocks, 256>>>(out, iters, 7u);
  float best = 1e30f;
  for (int r = 0; r < 3; r++) {
    cudaEventRecord(e0);
    k_peak_i16<<<blocks, 256>>>(out, iters, 7u);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    best = std::min(best, ms);
  }
  cudaError_t e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess) return fail(TB_ERR_CUDA, cudaGetErrorString(e));
  // 16 chains x 1 instruction (2 MACs, 4 ops) per iteration per thread
  *ops_per_s = (double)blocks * 256 * iters * 16 * 4 / (best * 1e-3);
  return TB_OK;
}

// Re-tile a plan's stream steps (tile size), as the autotuner does; for
// tests that pin one configuration.
extern "C" int32_t tbi_plan_retile(tb_plan* p, int32_t bits) {
  if (!p || !p->ctx) return TB_ERR_INVALID;
  std::lock_guard<std::mutex> lk(p->ctx->mu);
  std::string e = retile_plan(p->h, bits);
  if (!e.empty()) return fail(TB_ERR_INVALID, e);
  p->structure_uploaded = false;
  p->version = ++p->ctx->plan_counter;
  return TB_OK;
}

// Per node of a plan: 2 if the fused form runs it as stream tiles, 3 as
// GEMM tiles (the kind of the step that produces the node's output's parts).
extern "C" int32_t tbi_plan_node_kinds(const tb_plan* p, int32_t* kinds) {
  if (!p || !kinds) return TB_ERR_INVALID;
  const PlanHost& h = p->h;
  for (int j = 0; j < h.n_nodes; j++) kinds[j] = STEP_TILE;
  for (size_t si = 0; si < h.steps.size(); si++) {
    const int sn = h.step_node[si];
    if (sn >= 0 && h.steps[si].kind == STEP_GEMM) kinds[sn] = STEP_GEMM;
  }
  return TB_OK;
}

extern "C" int32_t tbi_measure_maxplus_peak(int32_t device, double* ops_per_s) {
  if (!ops_per_s) return TB_ERR_INVALID;
  CU(cudaSetDevice(device));
  int sms = 0;
  CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  float* out = nullptr;
  CU(cudaMalloc(&out, 64));
  cudaEvent_t e0, e1;
  CU(cudaEventCreate(&e0));
  CU(cudaEventCreate(&e1));
  const int blocks = sms * 8, iters = 4096;
  k_peak_f32<<<blocks, 256>>>(out, iters, 1e-7f);
  float best = 1e30f;
  for (int r = 0; r < 3; r++) {
    cudaEventRecord(e0);
    k_peak_f32<<<blocks, 256>>>(out, iters, 1e-7f);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    best = std::min(best, ms);
  }
  cudaError_t e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess) return fail(TB_ERR_CUDA, cudaGetErrorString(e));
  // 16 chains x 2 MAC per iteration per thread, 2 ops per MAC
  *ops_per_s = (double)blocks * 256 * iters * 16 * 2 * 2 / (best * 1e-3);
  return TB_OK;
}

// ---------------------------------------------------------------------------
// Serving: continuous batching in cohorts over several streams.
//
// A device-owner thread admits queued requests while pool memory, item slots
// and a free stream slot allow; the requests admitted together form a
// cohort, which runs as one batch (its items' level launches, as
// TB_MODE_LAYERED, with the result copy and an event) on the slot's stream,
// without the owner thread waiting for it.  Requests that arrive while
// cohorts run are admitted into the next free slot, so their work overlaps on
// the device with the running cohorts.  The owner thread polls the cohorts'
// events; a finished cohort frees its pool memory and slot at once and
// completes its requests.
// ---------------------------------------------------------------------------
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <thread>

struct tb_request {
  struct Item {
    tb_plan* plan;
    std::vector<int8_t> sv;
    float r;
  };
  std::vector<Item> items;
  int items_left = 0;
  float result = -INFINITY;
  tb_status status = TB_OK;
  std::string err;
  int state = 0;  // 0 queued, 1 running, 2 done
  double t_submit = 0, t_start = 0, t_done = 0;
  std::mutex m;
  std::condition_variable cv;
};

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// first-fit allocator over [0, size) in elements
struct PoolAlloc {
  std::map<int64_t, int64_t> free_;  // offset -> length
  void reset(int64_t size) {
    free_.clear();
    free_[0] = size;
  }
  int64_t alloc(int64_t n) {
    n = (n + 63) / 64 * 64;
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= n) {
        int64_t off = it->first, len = it->second;
        free_.erase(it);
        if (len > n) free_[off + n] = len - n;
        return off;
      }
    }
    return -1;
  }
  void release(int64_t off, int64_t n) {
    n = (n + 63) / 64 * 64;
    auto it = free_.emplace(off, n).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
};

}  // namespace

constexpr int kServeSlots = 4;  // cohorts in flight at once (one stream each)

struct Server {
  struct Active {
    tb_request* req;
    int idx;
    tb_plan* plan;
    int64_t off, elems;
  };
  // one stream and the batch state of the cohort running on it
  struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    DevBuf items, groups, sv, rv, out;
    HostBuf h_items, h_groups, h_sv, h_rv, h_out;
    std::vector<tb_ctx::LevelRange> ranges;
    std::vector<Active> act;
    bool busy = false;
  };
  tb_ctx* ctx = nullptr;
  std::thread th;
  std::atomic<bool> stop{false};
  std::mutex qm;
  std::condition_variable qcv;
  std::deque<tb_request*> pending;
  DevBuf pool;
  PoolAlloc palloc;
  int64_t pool_elems = 0;
  int max_items = 0;
  int n_active = 0;  // items of the cohorts in flight
  Slot slots[kServeSlots];
  std::atomic<int64_t> steps{0}, launches{0}, completed{0}, active_items{0};
};

static void serve_complete(tb_request* q, tb_status st, const std::string& msg) {
  std::lock_guard<std::mutex> lq(q->m);
  if (q->state == 2) return;
  q->status = st;
  q->err = msg;
  q->t_done = now_s();
  q->state = 2;
  q->cv.notify_all();
}

// Upload a cohort's batch state and enqueue its level launches, the result
// copy and the completion event on the slot's stream; returns at once.
template <typename T>
static tb_status serve_launch(Server* S, Server::Slot& sl) {
  tb_ctx* c = S->ctx;
  const int n = (int)sl.act.size();
  cudaStream_t s = sl.stream;
  std::vector<tb_plan*> plans(n);
  size_t svn = 0;
  for (int i = 0; i < n; i++) {
    plans[i] = sl.act[i].plan;
    svn += sl.act[i].req->items[sl.act[i].idx].sv.size();
  }
  const std::vector<char> merged = merge_choice(c, n, plans.data());
  const std::vector<GroupKey> gk = sorted_groups(n, plans.data(), false, merged.data());
  const size_t ng = std::max<size_t>(gk.size(), 1);
  CU(sl.h_items.ensure(sizeof(ItemDev<T>) * n));
  CU(sl.items.ensure(sizeof(ItemDev<T>) * n));
  CU(sl.h_groups.ensure(sizeof(Group) * ng));
  CU(sl.groups.ensure(sizeof(Group) * ng));
  CU(sl.h_sv.ensure(std::max<size_t>(svn, 16)));
  CU(sl.sv.ensure(std::max<size_t>(svn, 16)));
  CU(sl.h_rv.ensure(sizeof(float) * n));
  CU(sl.rv.ensure(sizeof(float) * n));
  CU(sl.h_out.ensure(sizeof(float) * n + 64));
  CU(sl.out.ensure(sizeof(float) * n + 64));
  ItemDev<T>* hi = reinterpret_cast<ItemDev<T>*>(sl.h_items.p);
  int8_t* hsv = reinterpret_cast<int8_t*>(sl.h_sv.p);
  float* hr = reinterpret_cast<float*>(sl.h_rv.p);
  size_t so = 0;
  for (int i = 0; i < n; i++) {
    const auto& a = sl.act[i];
    const auto& qi = a.req->items[a.idx];
    tb_plan* p = a.plan;
    ItemDev<T> it{};
    it.arena = reinterpret_cast<T*>(S->pool.p) + a.off;
    it.steps = reinterpret_cast<const Step*>(merged[i] ? p->d_steps_merged.p : p->d_steps.p);
    it.tiles = reinterpret_cast<const TileDesc*>(p->d_tiles.p);
    it.gemms = reinterpret_cast<const GemmDesc*>(merged[i] ? p->d_gemms_merged.p : p->d_gemms.p);
    it.leaves = reinterpret_cast<const LeafDesc*>(p->d_leaves.p);
    it.slice_vals = reinterpret_cast<const int8_t*>(sl.sv.p) + so;
    it.w = nullptr;  // the leaves take their weights from LeafDesc::w (refreshed at submit)
    it.flags = (c->opt.gemm_i16 && std::is_same<T, float>::value && p->i16_ok) ? 1 : 0;
    if (c->kpart_atomic && (!std::is_same<T, float>::value || p->nonneg_ok)) it.flags |= 2;
    it.r = 0.0f;
    it.n_leaves = p->h.n_tensors;
    it.done_base = 0;
    it.n_steps = (int)p->h.steps.size();
    it.fin = p->h.fin;
    hi[i] = it;
    if (!qi.sv.empty()) std::memcpy(hsv + so, qi.sv.data(), qi.sv.size());
    so += qi.sv.size();
    hr[i] = qi.r;
  }
  Group* hg = reinterpret_cast<Group*>(sl.h_groups.p);
  std::vector<void*> arenas(n);
  for (int i = 0; i < n; i++) arenas[i] = hi[i].arena;
  fill_groups(gk, plans.data(), merged.data(), arenas, hg, sl.ranges);
  CU(cudaMemcpyAsync(sl.items.p, hi, sizeof(ItemDev<T>) * n, cudaMemcpyHostToDevice, s));
  if (svn) CU(cudaMemcpyAsync(sl.sv.p, hsv, svn, cudaMemcpyHostToDevice, s));
  CU(cudaMemcpyAsync(sl.rv.p, hr, sizeof(float) * n, cudaMemcpyHostToDevice, s));
  CU(cudaMemcpyAsync(sl.groups.p, hg, sizeof(Group) * gk.size(), cudaMemcpyHostToDevice, s));
  float* dout = reinterpret_cast<float*>(sl.out.p);
  int* derr = reinterpret_cast<int*>(dout + n);  // error word after the results
  CU(cudaMemsetAsync(derr, 0, sizeof(int), s));
  const ItemDev<T>* di = reinterpret_cast<const ItemDev<T>*>(sl.items.p);
  const Group* dg = reinterpret_cast<const Group*>(sl.groups.p);
  const float* drv = reinterpret_cast<const float*>(sl.rv.p);
  for (const auto& lr : sl.ranges) {
    if (lr.count > 0x7fffffffLL) return fail(TB_ERR_UNSUPPORTED, "level too large for one launch");
    CU(launch_range<T>(c, lr, s, di, dg, dout, drv, derr));
    S->launches++;
  }
  // results and the error word back to the host, then the completion event
  CU(cudaMemcpyAsync(sl.h_out.p, dout, sizeof(float) * n + sizeof(int), cudaMemcpyDeviceToHost, s));
  CU(cudaEventRecord(sl.done, s));
  S->steps++;
  return TB_OK;
}

// A cohort's event has completed (or its launch failed): take its results,
// free its memory and slot, complete requests whose last item it held.
static void serve_finish(Server* S, Server::Slot& sl, tb_status st, const std::string& msg) {
  const int n = (int)sl.act.size();
  const float* ho = reinterpret_cast<const float*>(sl.h_out.p);
  if (st == TB_OK && *reinterpret_cast<const int*>(ho + n) != 0) {
    st = TB_ERR_TIMEOUT;
  }
  for (int i = 0; i < n; i++) {
    Server::Active& a = sl.act[i];
    tb_request* q = a.req;
    S->palloc.release(a.off, a.elems);
    if (st != TB_OK) {
      serve_complete(q, st, st == TB_ERR_TIMEOUT && msg.empty() ? "a bounded device-side wait timed out" : msg);
    } else {
      std::unique_lock<std::mutex> lq(q->m);
      q->result = std::max(q->result, ho[i]);
      const bool last = --q->items_left == 0;
      lq.unlock();
      if (last) {
        serve_complete(q, TB_OK, "");
        S->completed++;
      }
    }
  }
  S->n_active -= n;
  S->active_items = S->n_active;
  sl.act.clear();
  sl.busy = false;
}

// Admit queued requests (whole requests, first come first served) into a
// free slot while pool memory and item slots allow; returns whether a cohort
// was formed.
static bool serve_admit(Server* S, Server::Slot& sl) {
  while (!S->pending.empty()) {
    tb_request* q = S->pending.front();
    if (S->n_active + (int)sl.act.size() + (int)q->items.size() > S->max_items &&
        !(S->n_active == 0 && sl.act.empty()))
      break;
    std::vector<Server::Active> adm;
    bool ok = true;
    for (int k = 0; k < (int)q->items.size(); k++) {
      tb_plan* p = q->items[k].plan;
      const int64_t off = S->palloc.alloc(p->h.arena_elems);
      if (off < 0) {
        ok = false;
        break;
      }
      adm.push_back({q, k, p, off, p->h.arena_elems});
    }
    if (!ok) {
      for (auto& a : adm) S->palloc.release(a.off, a.elems);
      if (S->n_active == 0 && sl.act.empty()) {
        // cannot fit even alone: fail the request
        S->pending.pop_front();
        serve_complete(q, TB_ERR_OOM, "request needs more device memory than the serving pool");
        continue;
      }
      break;
    }
    S->pending.pop_front();
    {
      std::lock_guard<std::mutex> lq(q->m);
      q->state = 1;
      q->t_start = now_s();
    }
    for (auto& a : adm) sl.act.push_back(a);
  }
  return !sl.act.empty();
}

template <typename T>
static void serve_loop(Server* S) {
  cudaSetDevice(S->ctx->device);
  while (true) {
    bool busy = false;
    {
      std::unique_lock<std::mutex> lk(S->qm);
      // completions
      for (auto& sl : S->slots) {
        if (!sl.busy) continue;
        const cudaError_t e = cudaEventQuery(sl.done);
        if (e == cudaErrorNotReady) continue;
        serve_finish(S, sl, e == cudaSuccess ? TB_OK : TB_ERR_CUDA,
                     e == cudaSuccess ? "" : std::string("serving: ") + cudaGetErrorString(e));
      }
      // admissions into free slots
      for (auto& sl : S->slots) {
        if (sl.busy || S->pending.empty()) continue;
        if (!serve_admit(S, sl)) break;
        const int n = (int)sl.act.size();
        S->n_active += n;
        S->active_items = S->n_active;
        sl.busy = true;
        const tb_status st = serve_launch<T>(S, sl);
        if (st != TB_OK) {
          cudaStreamSynchronize(sl.stream);  // nothing of it may still run
          serve_finish(S, sl, st, g_err);
        }
      }
      for (auto& sl : S->slots) busy = busy || sl.busy;
      if (!busy) {
        if (S->stop && S->pending.empty()) break;
        S->qcv.wait_for(lk, std::chrono::milliseconds(2));
        continue;
      }
    }
    // cohorts in flight: poll again shortly (a submission also wakes the loop)
    std::unique_lock<std::mutex> lk(S->qm);
    S->qcv.wait_for(lk, std::chrono::microseconds(50));
  }
}

static std::map<tb_ctx*, Server*> g_servers;
static std::mutex g_servers_mu;

extern "C" {

tb_status tb_serve_start(tb_ctx* c, int64_t pool_bytes, int32_t max_items) {
  if (!c) return fail(TB_ERR_INVALID, "null context");
  std::lock_guard<std::mutex> lk(g_servers_mu);
  if (g_servers.count(c)) return fail(TB_ERR_INVALID, "server already running on this context");
  CU(cudaSetDevice(c->device));
  tb_status st = c->opt.dtype == TB_DTYPE_F32 ? set_kernel_attrs<float>() : set_kernel_attrs<int32_t>();
  if (st) return st;
  std::unique_ptr<Server> S(new Server());
  S->ctx = c;
  if (pool_bytes <= 0) pool_bytes = (int64_t)(c->budget / 2);
  S->pool_elems = pool_bytes / 4;
  S->max_items = max_items > 0 ? max_items : 4096;
  CU(S->pool.ensure((size_t)S->pool_elems * 4));
  S->palloc.reset(S->pool_elems);
  for (auto& sl : S->slots) {
    CU(cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking));
    CU(cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming));
  }
  Server* raw = S.release();
  raw->th = c->opt.dtype == TB_DTYPE_F32 ? std::thread(serve_loop<float>, raw) : std::thread(serve_loop<int32_t>, raw);
  g_servers[c] = raw;
  return TB_OK;
}

tb_status tb_serve_stop(tb_ctx* c) {
  Server* S = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_servers_mu);
    auto it = g_servers.find(c);
    if (it == g_servers.end()) return fail(TB_ERR_INVALID, "no server on this context");
    S = it->second;
    g_servers.erase(it);
  }
  {
    std::lock_guard<std::mutex> lk(S->qm);
    S->stop = true;
  }
  S->qcv.notify_all();
  S->th.join();  // runs every queued and admitted request to completion
  for (tb_request* q : S->pending) serve_complete(q, TB_ERR_INVALID, "server stopped");
  for (auto& sl : S->slots) {
    cudaStreamSynchronize(sl.stream);
    cudaEventDestroy(sl.done);
    cudaStreamDestroy(sl.stream);
  }
  delete S;
  return TB_OK;
}

tb_status tb_submit(tb_ctx* c, int32_t n, tb_plan* const* plans, const int8_t* slice_vals, const float* r,
                    tb_request** out) {
  if (!c || !out || n <= 0 || !plans) return fail(TB_ERR_INVALID, "bad arguments");
  *out = nullptr;
  Server* S = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_servers_mu);
    auto it = g_servers.find(c);
    if (it == g_servers.end()) return fail(TB_ERR_INVALID, "no server on this context (tb_serve_start)");
    S = it->second;
  }
  std::unique_ptr<tb_request> q(new tb_request());
  size_t so = 0;
  for (int i = 0; i < n; i++) {
    tb_plan* p = plans[i];
    if (!p || p->ctx != c) return fail(TB_ERR_INVALID, "plan of another context");
    if (!p->h.has_weights) return fail(TB_ERR_INVALID, "plan has no bound weights");
    tb_request::Item it;
    it.plan = p;
    size_t k = p->h.sliced.size();
    if (k && !slice_vals) return fail(TB_ERR_INVALID, "slice_vals required");
    if (k) it.sv.assign(slice_vals + so, slice_vals + so + k);
    for (int8_t v : it.sv)
      if (v != 0 && v != 1) return fail(TB_ERR_INVALID, "slice values must be 0 or 1");
    so += k;
    it.r = r ? r[i] : 0.0f;
    q->items.push_back(std::move(it));
  }
  {
    std::lock_guard<std::mutex> lk(c->mu);
    tb_status st = TB_OK;
    for (auto& it : q->items)
      if ((st = upload_plan(it.plan, true))) return st;
  }
  q->items_left = n;
  q->t_submit = now_s();
  tb_request* raw = q.release();
  {
    std::lock_guard<std::mutex> lk(S->qm);
    S->pending.push_back(raw);
  }
  S->qcv.notify_all();
  *out = raw;
  return TB_OK;
}

tb_status tb_poll(tb_request* q, int32_t* done) {
  if (!q || !done) return fail(TB_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(q->m);
  *done = q->state == 2;
  return TB_OK;
}

tb_status tb_wait(tb_request* q, int32_t timeout_ms, float* out_max, double* latency_ms) {
  if (!q) return fail(TB_ERR_INVALID, "null request");
  std::unique_lock<std::mutex> lk(q->m);
  if (!q->cv.wait_for(lk, std::chrono::milliseconds(timeout_ms < 0 ? 1 << 30 : timeout_ms),
                      [&] { return q->state == 2; }))
    return fail(TB_ERR_TIMEOUT, "request not finished within the timeout");
  if (q->status != TB_OK) return fail(q->status, q->err);
  if (out_max) *out_max = q->result;
  if (latency_ms) *latency_ms = (q->t_done - q->t_submit) * 1000.0;
  return TB_OK;
}

void tb_request_free(tb_request* q) { delete q; }

tb_status tb_serve_stats(tb_ctx* c, int64_t* steps, int64_t* launches, int64_t* completed, int64_t* active) {
  std::lock_guard<std::mutex> lk(g_servers_mu);
  auto it = g_servers.find(c);
  if (it == g_servers.end()) return fail(TB_ERR_INVALID, "no server on this context");
  Server* S = it->second;
  if (steps) *steps = S->steps;
  if (launches) *launches = S->launches;
  if (completed) *completed = S->completed;
  if (active) *active = S->active_items;
  return TB_OK;
}

}  // extern "C"
