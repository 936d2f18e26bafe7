// Host-side plan compiler: turns a contraction tree over dimension-2 labels
// into device work (leaf builder, fused tile steps, final reduction) and into
// the per-contraction lowering of the plain path.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "tb_internal.h"

namespace tb {

// label ids of the K-part index of a split-K GEMM node's partials (above
// every real label)
constexpr int32_t kSplitLabel = 1 << 28;

enum PlainKind : int32_t { PLAIN_TILE = 1, PLAIN_GEMM = 2 };

// One launch of the plain (OMEinsum-style) lowering.
struct PlainOp {
  int32_t kind;
  TileDesc tile;                 // PLAIN_TILE: permute / reduce / small contraction
  int64_t a_off, b_off, c_off;   // PLAIN_GEMM operands (arena offsets)
  int64_t M, N, K, batch;        // PLAIN_GEMM shape, canonical column-major
};

struct PlanInput {
  int32_t n_labels = 0;
  int32_t n_tensors = 0;
  const int32_t* ix_off = nullptr;
  const int32_t* ix_lab = nullptr;
  int32_t n_iy = 0;
  const int32_t* iy = nullptr;
  int32_t n_nodes = 0;
  const int32_t* children = nullptr;
  const int32_t* node_iy_off = nullptr;
  const int32_t* node_iy_lab = nullptr;
  int32_t n_sliced = 0;
  const int32_t* sliced = nullptr;
};

struct PlanHost {
  int32_t n_labels = 0, n_tensors = 0, n_nodes = 0;
  std::vector<std::vector<int32_t>> leaf_raw;  // raw labels of each leaf
  std::vector<std::vector<int32_t>> labels;    // reported labels of tensor id (leaves, then nodes)
  std::vector<std::vector<int32_t>> flabels;   // device layout of tensor id in the fused form
  std::vector<int64_t> off;                    // arena offset of tensor id
  std::vector<int32_t> children;
  std::vector<int32_t> open;                   // open labels, output order
  std::vector<int32_t> sliced;                 // sliced labels, slice-value order
  std::vector<int32_t> slice_index;            // label -> index in sliced (-1)
  int64_t arena_elems = 0;                     // fused form (leaves + node outputs)
  int64_t plain_elems = 0;                     // plain form (adds lowering scratch)
  int32_t root = 0;                            // tensor id of the root
  bool has_weights = false;

  std::vector<Step> steps;
  std::vector<std::vector<int32_t>> levels;    // step indices of each level
  std::vector<TileDesc> tiles;
  std::vector<GemmDesc> gemms;
  std::vector<LeafDesc> leaves;
  FinalDesc fin{};
  std::vector<std::vector<PlainOp>> plain;     // per node, in post-order

  double tc = 0, sc = 0, rwc = 0, ops = 0, bytes = 0;
  std::vector<double> node_ops, node_bytes;    // algorithmic work of each node: 2 2^|L|, 4 (|A|+|B|+|C|)
  int64_t total_tiles = 0;
  int32_t tile_bits = 9;                       // stream tiles grow to 2^tile_bits outputs
  int32_t gemm_ctas = 304;                     // resident GEMM CTAs the K split balances for
  std::vector<int32_t> step_node;              // node a step contracts (-1: leaves, final); a split-K
                                               // reduce step holds -2 - node
  std::vector<int64_t> split_off;              // per node: arena offset of its K-part partials (-1)
  // The same program with every split-K GEMM merged back into one pass over
  // the whole K (for batches whose items fill the GPU without the split):
  // the GEMM step writes the output directly and waits on the A operand's
  // step, the fill and max-over-parts steps have no tiles, and steps that
  // waited on the max wait on the GEMM.  Same step indices and levels.
  bool has_split = false;
  std::vector<Step> steps_merged;
  std::vector<GemmDesc> gemms_merged;

  // fused small form (compile_small): every tensor in the reported label
  // order, leaves packed first, intermediates placed by first fit, every
  // tensor freed after the node that reads it
  bool small_ok = false;
  std::vector<SmallNode> small;
  std::vector<int32_t> small_leaf;
  int32_t small_words = 0, small_root = 0, small_root_log2 = 0;
  double small_cost = 0;                       // issue-slot estimate of one item (launch order)
};

// Build the fused small form of a compiled plan when it fits the limits of
// tb_internal.h; sets small_ok.
void compile_small(PlanHost& p);

// Compile; returns "" on success or an error message.
std::string compile_plan(const PlanInput& in, PlanHost& out, int gemm_min_log2);

// Re-plan every stream-tile step of the fused form with tiles of up to
// 2^bits outputs (8..11); GEMM steps and the arena layout are unchanged.
std::string retile_plan(PlanHost& p, int bits);
// Fill has_split, steps_merged and gemms_merged from steps and gemms.
void merge_split_k(PlanHost& p);

// Plan one stream tile for C = max_{R} A (+ B).  A, C (and B if non-null)
// are label lists in their memory order.  Returns "" or an error.
std::string plan_tile(const std::vector<int32_t>& A, const std::vector<int32_t>* B,
                      const std::vector<int32_t>& C, int64_t a_off, int64_t b_off, int64_t c_off,
                      TileDesc& d, int out_bits_target = 9);

// GEMM descriptor for node (A, B -> C) whose operands are already in the
// k-pair interleaved layouts; returns false if they are not.
bool plan_gemm(const std::vector<int32_t>& A, const std::vector<int32_t>& B,
               const std::vector<int32_t>& C, int64_t a_off, int64_t b_off, int64_t c_off, GemmDesc& g);

}  // namespace tb
