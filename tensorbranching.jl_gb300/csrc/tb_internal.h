// Internal data structures shared by the plan compiler (host) and the
// kernels (device).  Everything here is POD so it can be copied to the GPU.
#pragma once
#include <cstdint>

namespace tb {

constexpr int kMaxTileBits = 16;  // labels inside one CTA tile (per tensor)
constexpr int kMaxBits = 48;      // labels of one tensor / grid / loop
constexpr int kThreads = 256;     // threads of every tile kernel
constexpr int kMaxOpt = 8;        // outputs per thread in the stream tile
constexpr int kSmemFloats = 8192; // stream tile staging (As + Bs), floats
constexpr int kMaxStages = 8;     // stream tile pipeline depth (short operand tiles)

enum StepKind : int32_t {
  STEP_LEAVES = 1,  // build the item's leaf tensors
  STEP_TILE = 2,    // stream tile contraction (fused permute/reduce/contract)
  STEP_GEMM = 3,    // register-blocked gather GEMM contraction
  STEP_FINAL = 4,   // max over the root tensor + r -> item result
  STEP_FILL = 5,    // a split-K GEMM node's output set to the atomic identity (items
                    // whose K parts combine by atomic max; a no-op for the others)
  STEP_KRED = 6,    // max over a split-K GEMM node's part outputs: a stream tile step
                    // (items whose K parts go through partials; a no-op for the others)
};

// The atomic identity STEP_FILL writes: INT_MIN, below every int32 and, read
// as the bits of a float, below every float >= 0 and -inf.
constexpr int32_t kFillBits = (int32_t)0x80000000u;
constexpr int kFillPerTile = 4096;  // elements one STEP_FILL tile writes

// Stream tile contraction:  C[c] = max over reduced labels of A[.] (+ B[.]).
// The node's labels are split into
//   Tc : output labels staged inside a CTA (tile outputs, in C order)
//   Tr : reduced labels staged inside a CTA
//   G  : output labels enumerated by the CTA grid
//   Rl : reduced labels enumerated by a loop inside the CTA
// A CTA loads the sub-tensors of A and B spanned by Tc u Tr into shared
// memory (indexed in each tensor's own label order), reduces over Tr for its
// 2^|Tc| outputs, repeats for every Rl assignment, and writes its C tile.
struct TileDesc {
  int64_t a_off, b_off, c_off;  // element offsets in the item arena; b_off < 0: unary
  int32_t n_grid, n_loop, n_tc, n_tr;
  int32_t na, nb;               // log2 sizes of the A / B sub-tiles
  int32_t pa, pb, pc;           // leading tile bits that are tensor positions 0..p-1
  int32_t split_log2;           // threads cooperating on one output (reduction split)
  int32_t n_tiles;              // CTAs = 2^n_grid
  int32_t pad_;
  int8_t g_pa[kMaxBits], g_pb[kMaxBits], g_pc[kMaxBits];  // grid bit -> tensor position (-1)
  int8_t l_pa[kMaxBits], l_pb[kMaxBits];                  // loop bit -> tensor position (-1)
  int8_t ta_pos[kMaxTileBits], tb_pos[kMaxTileBits];      // tile bit -> tensor position
  int8_t tc_pos[kMaxTileBits];                            // Tc bit -> C position
  int8_t tc_a[kMaxTileBits], tc_b[kMaxTileBits];          // Tc bit -> A / B tile bit (-1)
  int8_t tr_a[kMaxTileBits], tr_b[kMaxTileBits];          // Tr bit -> A / B tile bit (-1)
};
// a TileDesc copied to the front of a stream tile's shared memory, padded
// so the operand buffers after it start on a 16-byte boundary
constexpr int kDescWords = 108;
static_assert(sizeof(TileDesc) <= kDescWords * 4 && kDescWords % 4 == 0, "descriptor copy");

// Register-blocked GEMM for a contraction node with large M, N and K label
// groups.  The plan compiler lays the operands out "k-pair interleaved":
//   A[(k & 1) + 2 m + 2 M (k >> 1) + M K b]    labels [k0, M..., K1..., batch...]
//   B[(k & 1) + 2 n + 2 N (k >> 1) + N K b]    labels [k0, N..., K1..., batch...]
// so each CTA stage is a set of contiguous rows (bulk async copies) and one
// 64-bit shared load yields (x[k], x[k+1]) for a packed f32x2 add.  The
// output C[m, n, b] is scattered to C's own layout through m_pc / n_pc / b_pc.
struct GemmDesc {
  int64_t a_off, b_off, c_off;
  int64_t c_fin;             // the node's output; with a split K, items whose values are
                             // all >= 0 or -inf (f32) or any int32 max their parts into it
                             // atomically instead of writing partials at c_off
  int32_t m_log2, n_log2, k_log2, bt_log2;
  int32_t bm_log2, bn_log2;  // CTA tile BM x BN
  int32_t n_tiles;           // (M / BM) (N / BN) 2^bt 2^ks work units
  int32_t ks_log2;           // K split: unit part p covers K / 2^ks and writes
                             // its partial C at c_off + p 2^(m+n+bt); a
                             // reduce step takes the max over the parts
  int8_t m_pc[32], n_pc[32], b_pc[32];  // C position of m / n / batch bit i
};

// One leaf tensor of the MIS network (GenericTensorNetworks IndependentSet):
// vertex [0, w], edge [[0,0],[0,-inf]]; a self-loop edge is its diagonal.
struct LeafDesc {
  int64_t off;          // output offset in the arena
  int32_t nraw;         // raw labels: 1 vertex, 2 edge
  int32_t n_out;        // output rank
  int8_t out_bit[2];    // raw position -> output bit (-1: label sliced)
  int8_t slice_idx[2];  // raw position -> index into the item's slice values (-1)
  int32_t label;        // vertex label of a vertex leaf (index into a weight array), else -1
  float w;              // vertex weight (vertex leaves) for paths without a weight array
};

struct Step {
  int32_t kind;        // StepKind
  int32_t desc;        // index into the plan's TileDesc / GemmDesc array
  int32_t dep0, dep1;  // steps this one waits for (-1 none)
  int32_t n_tiles;     // CTAs (work units) of this step
  int32_t level;       // 0 for leaves; 1 + max(level(deps))
};

// Final step: max over the root tensor (2^root_log2 values at root_off).
struct FinalDesc {
  int64_t root_off;
  int32_t root_log2;
  int32_t pad_;
};

// Fused small-network form: one block contracts a whole network in shared
// memory.  Limits: tensors of at most kSmallMaxRank labels, nodes of at most
// kSmallMaxL labels (outputs + reduced), kSmallMaxWords shared words.
constexpr int kSmallMaxRank = 13;
constexpr int kSmallMaxL = 16;
constexpr int kSmallMaxWords = 12288;
constexpr int kSmallThreads = 128;  // threads of one item's block

// One contraction C = max_R A + B of the fused small form.  Bit i of the
// index x = o | k << nc (o: output index, k: reduced index) selects bit
// pos_a(i) of A's index and pos_b(i) of B's, packed 4 bits per position in
// pa / pb (15: the label is not in that operand).  Offsets are shared-memory
// words.
struct SmallNode {
  int32_t a_off, b_off, c_off;
  int32_t nc_nk;  // nc | nk << 8
  uint32_t pa[2], pb[2];
};
static_assert(sizeof(SmallNode) == 32, "SmallNode layout");


// One batch item as the persistent executor sees it.
template <typename T>
struct ItemDev {
  T* arena;
  const Step* steps;
  const TileDesc* tiles;
  const GemmDesc* gemms;
  const LeafDesc* leaves;
  const int8_t* slice_vals;
  const float* w;      // vertex weights by label (per call), or null: LeafDesc::w
  int32_t flags;       // bit 0: GEMM tiles may use exact packed-int16 arithmetic;
                       // bit 1: split-K parts combine by atomic max into the output
  float r;
  int32_t n_leaves;
  int32_t done_base;   // offset of this item's step counters
  int32_t n_steps;
  FinalDesc fin;
  // fused small form (null when the plan has none)
  const SmallNode* small;
  const int32_t* small_leaf;  // shared-memory word offset of each leaf
  int32_t n_small;
  int32_t small_root;         // shared-memory offset of the root tensor
  int32_t small_root_log2;
  int32_t small_words;
};

// A group = all tiles of one (item, step); groups are listed in dependency
// order and tickets index tiles within the concatenation of groups.
// Stream steps one warp runs straight from global memory (tiny_node): one
// tile, no reduction loop, at most 2^kTinyOut outputs and 2^kTinyRed reduced
// terms.
constexpr int kTinyOut = 8;
constexpr int kTinyRed = 5;

// A tiny stream step as tiny_node reads it: the operand and output offsets
// and, per output bit and reduced bit, the tensor position the bit moves in
// A, B and C (-1: not in that tensor).  Built on the host from the step's
// TileDesc, so a lane forms its offsets from one 64-byte load.
struct TinyDesc {
  int64_t a_off, b_off, c_off;  // b_off < 0: unary
  int8_t n_tc, n_tr;
  int8_t oa[kTinyOut], ob[kTinyOut], oc[kTinyOut];
  int8_t ra[kTinyRed], rb[kTinyRed];
  int8_t pad_[4];
};
static_assert(sizeof(TinyDesc) == 64, "one 64-byte load");

struct Group {
  int32_t item, step;
  int64_t first;          // first ticket of this group
  int32_t tiny;           // 1: a one-tile stream step small enough for one warp (tiny_node)
  int32_t run;            // tiny: groups from this one to the end of its level's tiny run
  const TinyDesc* tile;   // its descriptor (device), when tiny
  void* arena;            // the item's arena (device), when tiny
};

// The tickets of one per-level launch (k_level): CTAs b < split_cta take
// runs of `chunk` tickets from `first` up to `mid` (the launch's tiny steps,
// listed first), CTAs b >= split_cta runs of `chunk2` from `mid` up to
// `last`.
struct LevelSpan {
  int64_t first, mid, last, chunk, chunk2;
  int32_t split_cta, pad_;
};

// A unit of work of the persistent executor: tiles [t0, t1) of one group.
// Chunks are listed in dependency order.
struct Chunk {
  int32_t group, pad_;
  int64_t t0, t1;
};

}  // namespace tb
