// Plan compiler.  Semantics follow the reference's plan objects:
//   CompressedEinsum{ixs, iy, ct} and uncompress   src/types.jl:51-79
//   node output labels as parse_eincode derives them: the labels of the two
//   operands still needed outside the subtree or open in iy
//   complexity model (tc, sc, rwc)                 src/types.jl:115-121
// and the lowering OMEinsum applies to each binary node (reduce private
// labels, permute to [M,K,b] / [K,N,b], batched GEMM, permute to iy).
#include "plan.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

namespace tb {
namespace {

int index_of(const std::vector<int32_t>& v, int32_t x) {
  for (size_t i = 0; i < v.size(); i++)
    if (v[i] == x) return (int)i;
  return -1;
}

double log2sumexp2(double a, double b) {
  double m = std::max(a, b);
  if (m == -INFINITY) return m;
  return m + std::log2(std::exp2(a - m) + std::exp2(b - m));
}

int64_t align_up(int64_t x, int64_t a) { return (x + a - 1) / a * a; }

}  // namespace

std::string plan_tile(const std::vector<int32_t>& A, const std::vector<int32_t>* Bp,
                      const std::vector<int32_t>& C, int64_t a_off, int64_t b_off, int64_t c_off,
                      TileDesc& d, int out_bits_target) {
  std::memset(&d, 0xff, sizeof(d));  // int8 tables default to -1
  const std::vector<int32_t> empty;
  const std::vector<int32_t>& B = Bp ? *Bp : empty;
  std::vector<int32_t> L;
  for (int32_t x : A)
    if (index_of(L, x) < 0) L.push_back(x);
  for (int32_t x : B)
    if (index_of(L, x) < 0) L.push_back(x);
  if (L.size() != A.size() + B.size() - [&] {
        int s = 0;
        for (int32_t x : B) s += index_of(A, x) >= 0;
        return s;
      }())
    return "repeated label inside a tensor";
  for (int32_t x : C)
    if (index_of(L, x) < 0) return "output label absent from operands";
  if ((int)A.size() > kMaxBits || (int)B.size() > kMaxBits || (int)C.size() > 31)
    return "tensor rank beyond the engine's limit";
  std::vector<int32_t> R;
  for (int32_t x : L)
    if (index_of(C, x) < 0) R.push_back(x);
  std::vector<int32_t> S;
  auto inS = [&](int32_t x) { return index_of(S, x) >= 0; };
  auto feasible = [&](const std::vector<int32_t>& s) {
    int tc = 0, tr = 0, na = 0, nb = 0, pa = 0, pb = 0, pc = 0;
    for (int32_t x : s) {
      if (index_of(C, x) >= 0) tc++; else tr++;
      if (index_of(A, x) >= 0) na++;
      if (index_of(B, x) >= 0) nb++;
    }
    while (pa < (int)A.size() && index_of(s, A[pa]) >= 0) pa++;
    while (pb < (int)B.size() && index_of(s, B[pb]) >= 0) pb++;
    while (pc < (int)C.size() && index_of(s, C[pc]) >= 0) pc++;
    if (tc > std::max(10, out_bits_target) || tr > 8 || na > 13 || nb > 13) return false;
    if (na - pa > 9 || nb - pb > 9 || tc - pc > 9) return false;
    int64_t sm = (int64_t(1) << na) + (Bp ? (int64_t(1) << nb) : 0);
    return sm <= kSmemFloats;
  };
  auto with = [&](std::vector<int32_t> s, int32_t x) {
    if (index_of(s, x) < 0) s.push_back(x);
    return s;
  };
  // 1. leading labels of every tensor, for coalesced loads and stores
  for (int p = 1; p <= 6; p++) {
    std::vector<int32_t> s2 = S;
    for (const std::vector<int32_t>* X : {&C, &A, &B})
      for (int i = 0; i < p && i < (int)X->size(); i++) s2 = with(s2, (*X)[i]);
    if (!feasible(s2)) break;
    S = s2;
  }
  // 2. reduced labels into the tile (fewer loop trips)
  std::vector<int32_t> Rs = R;
  std::stable_sort(Rs.begin(), Rs.end(), [&](int32_t x, int32_t y) {
    int ax = index_of(A, x), ay = index_of(A, y);
    if (ax < 0) ax = 1000;
    if (ay < 0) ay = 1000;
    return ax < ay;
  });
  for (int32_t x : Rs) {
    if (inS(x)) continue;
    auto s2 = with(S, x);
    if (feasible(s2)) S = s2;
  }
  // 3. more outputs per CTA while the grid stays large
  for (;;) {
    int tc = 0;
    for (int32_t x : S) tc += index_of(C, x) >= 0;
    int grid = (int)C.size() - tc;
    int32_t next = -1;
    for (int32_t x : C)
      if (!inS(x)) { next = x; break; }
    if (next < 0) break;
    if (tc >= out_bits_target && grid <= 12) break;
    if (tc >= std::max(10, out_bits_target)) break;
    auto s2 = with(S, next);
    if (!feasible(s2)) break;
    S = s2;
  }
  // 4. emit
  std::vector<int32_t> Tc, Tr, TA, TB, G, Rl;
  for (int32_t x : C)
    if (inS(x)) Tc.push_back(x); else G.push_back(x);
  for (int32_t x : Rs)
    if (inS(x)) Tr.push_back(x); else Rl.push_back(x);
  for (int32_t x : A)
    if (inS(x)) TA.push_back(x);
  for (int32_t x : B)
    if (inS(x)) TB.push_back(x);
  if ((int)G.size() > 30 || (int)Rl.size() > kMaxBits) return "node too large";
  d.a_off = a_off;
  d.b_off = Bp ? b_off : -1;
  d.c_off = c_off;
  d.n_grid = (int32_t)G.size();
  d.n_loop = (int32_t)Rl.size();
  d.n_tc = (int32_t)Tc.size();
  d.n_tr = (int32_t)Tr.size();
  d.na = (int32_t)TA.size();
  d.nb = (int32_t)TB.size();
  d.pa = 0;
  while (d.pa < d.na && index_of(A, TA[d.pa]) == d.pa) d.pa++;
  d.pb = 0;
  while (d.pb < d.nb && index_of(B, TB[d.pb]) == d.pb) d.pb++;
  d.pc = 0;
  while (d.pc < d.n_tc && index_of(C, Tc[d.pc]) == d.pc) d.pc++;
  int lt = 0;
  while ((1 << lt) < kThreads) lt++;
  d.split_log2 = d.n_tc >= lt ? 0 : std::min(lt - d.n_tc, d.n_tr);
  d.n_tiles = 1 << d.n_grid;
  d.pad_ = 0;
  for (size_t i = 0; i < G.size(); i++) {
    d.g_pa[i] = (int8_t)index_of(A, G[i]);
    d.g_pb[i] = (int8_t)index_of(B, G[i]);
    d.g_pc[i] = (int8_t)index_of(C, G[i]);
  }
  for (size_t i = 0; i < Rl.size(); i++) {
    d.l_pa[i] = (int8_t)index_of(A, Rl[i]);
    d.l_pb[i] = (int8_t)index_of(B, Rl[i]);
  }
  for (size_t i = 0; i < TA.size(); i++) d.ta_pos[i] = (int8_t)index_of(A, TA[i]);
  for (size_t i = 0; i < TB.size(); i++) d.tb_pos[i] = (int8_t)index_of(B, TB[i]);
  for (size_t i = 0; i < Tc.size(); i++) {
    d.tc_pos[i] = (int8_t)index_of(C, Tc[i]);
    d.tc_a[i] = (int8_t)index_of(TA, Tc[i]);
    d.tc_b[i] = (int8_t)index_of(TB, Tc[i]);
  }
  for (size_t i = 0; i < Tr.size(); i++) {
    d.tr_a[i] = (int8_t)index_of(TA, Tr[i]);
    d.tr_b[i] = (int8_t)index_of(TB, Tr[i]);
  }
  return "";
}

bool plan_gemm(const std::vector<int32_t>& A, const std::vector<int32_t>& B,
               const std::vector<int32_t>& C, int64_t a_off, int64_t b_off, int64_t c_off, GemmDesc& g) {
  // A = [k0, M..., K1..., Bt...], B = [k0, N..., K1..., Bt...]
  if (A.empty() || B.empty() || A[0] != B[0] || index_of(C, A[0]) >= 0) return false;
  std::vector<int32_t> M, N, K{A[0]}, Bt;
  size_t i = 1;
  while (i < A.size() && index_of(C, A[i]) >= 0 && index_of(B, A[i]) < 0) M.push_back(A[i++]);
  while (i < A.size() && index_of(C, A[i]) < 0) K.push_back(A[i++]);
  while (i < A.size() && index_of(C, A[i]) >= 0 && index_of(B, A[i]) >= 0) Bt.push_back(A[i++]);
  if (i != A.size()) return false;
  size_t j = 1;
  while (j < B.size() && index_of(C, B[j]) >= 0 && index_of(A, B[j]) < 0) N.push_back(B[j++]);
  for (size_t q = 1; q < K.size(); q++, j++)
    if (j >= B.size() || B[j] != K[q]) return false;
  for (size_t q = 0; q < Bt.size(); q++, j++)
    if (j >= B.size() || B[j] != Bt[q]) return false;
  if (j != B.size()) return false;
  if (C.size() != M.size() + N.size() + Bt.size()) return false;
  if (M.size() < 4 || N.size() < 4 || K.size() < 4) return false;  // K >= 16: one BK = 16 chunk
  if (M.size() > 30 || N.size() > 30 || K.size() > 30 || Bt.size() > 30) return false;
  std::memset(&g, 0xff, sizeof(g));
  g.a_off = a_off; g.b_off = b_off; g.c_off = c_off; g.c_fin = c_off;
  g.m_log2 = (int)M.size(); g.n_log2 = (int)N.size(); g.k_log2 = (int)K.size(); g.bt_log2 = (int)Bt.size();
  // CTA tiles the device dispatches: 128x128, 128x64, 64x128, 64x64, 32x32,
  // 16x16, and 256x16 / 16x256 when one side is 16 or 32 and the other >= 256
  int bm = std::min(g.m_log2, 7), bn = std::min(g.n_log2, 7);
  if (std::min(g.m_log2, g.n_log2) <= 5 && std::max(g.m_log2, g.n_log2) >= 8) {
    bm = g.m_log2 >= 8 ? 8 : 4;
    bn = g.n_log2 >= 8 ? 8 : 4;
  } else if (bm < 6 || bn < 6) {
    bm = bn = std::min(std::min(bm, bn), 5);
  }
  g.bm_log2 = bm;
  g.bn_log2 = bn;
  int64_t nt = (int64_t(1) << (g.m_log2 - g.bm_log2)) * (int64_t(1) << (g.n_log2 - g.bn_log2)) *
               (int64_t(1) << g.bt_log2);
  if (nt > 0x7fffffffLL) return false;
  g.n_tiles = (int32_t)nt;
  g.ks_log2 = 0;
  for (size_t q = 0; q < M.size(); q++) g.m_pc[q] = (int8_t)index_of(C, M[q]);
  for (size_t q = 0; q < N.size(); q++) g.n_pc[q] = (int8_t)index_of(C, N[q]);
  for (size_t q = 0; q < Bt.size(); q++) g.b_pc[q] = (int8_t)index_of(C, Bt[q]);
  return true;
}

namespace {

// OMEinsum-style lowering of one binary node for the plain path.
std::string lower_plain(const std::vector<int32_t>& A, const std::vector<int32_t>& B,
                        const std::vector<int32_t>& C, int64_t a_off, int64_t b_off, int64_t c_off,
                        int64_t scratch_base, int64_t& scratch_need, std::vector<PlainOp>& ops) {
  std::vector<int32_t> M, N, K, Bt;
  for (int32_t x : A) {
    bool inb = index_of(B, x) >= 0, inc = index_of(C, x) >= 0;
    if (inb && inc) Bt.push_back(x);
    else if (inb) K.push_back(x);
    else if (inc) M.push_back(x);
  }
  for (int32_t x : B)
    if (index_of(A, x) < 0 && index_of(C, x) >= 0) N.push_back(x);
  std::vector<int32_t> la, lb, lc;
  la.insert(la.end(), M.begin(), M.end());
  la.insert(la.end(), K.begin(), K.end());
  la.insert(la.end(), Bt.begin(), Bt.end());
  lb.insert(lb.end(), K.begin(), K.end());
  lb.insert(lb.end(), N.begin(), N.end());
  lb.insert(lb.end(), Bt.begin(), Bt.end());
  lc.insert(lc.end(), M.begin(), M.end());
  lc.insert(lc.end(), N.begin(), N.end());
  lc.insert(lc.end(), Bt.begin(), Bt.end());
  int64_t pos = scratch_base;
  auto take = [&](size_t rank) {
    int64_t o = pos;
    pos = align_up(pos + (int64_t(1) << rank), 64);
    return o;
  };
  int64_t ap = a_off, bp = b_off, cp = c_off;
  std::string e;
  if (la != A) {
    ap = take(la.size());
    PlainOp op{};
    op.kind = PLAIN_TILE;
    if (!(e = plan_tile(A, nullptr, la, a_off, -1, ap, op.tile)).empty()) return e;
    ops.push_back(op);
  }
  if (lb != B) {
    bp = take(lb.size());
    PlainOp op{};
    op.kind = PLAIN_TILE;
    if (!(e = plan_tile(B, nullptr, lb, b_off, -1, bp, op.tile)).empty()) return e;
    ops.push_back(op);
  }
  bool permute_c = lc != C;
  if (permute_c) cp = take(lc.size());
  int64_t Ms = int64_t(1) << M.size(), Ns = int64_t(1) << N.size(), Ks = int64_t(1) << K.size();
  if (Ms >= 16 && Ns >= 16 && Ks >= 16) {
    PlainOp op{};
    op.kind = PLAIN_GEMM;
    op.a_off = ap; op.b_off = bp; op.c_off = cp;
    op.M = Ms; op.N = Ns; op.K = Ks; op.batch = int64_t(1) << Bt.size();
    ops.push_back(op);
  } else {
    PlainOp op{};
    op.kind = PLAIN_TILE;
    if (!(e = plan_tile(la, &lb, lc, ap, bp, cp, op.tile)).empty()) return e;
    ops.push_back(op);
  }
  if (permute_c) {
    PlainOp op{};
    op.kind = PLAIN_TILE;
    if (!(e = plan_tile(lc, nullptr, C, cp, -1, c_off, op.tile)).empty()) return e;
    ops.push_back(op);
  }
  scratch_need = std::max(scratch_need, pos - scratch_base);
  return "";
}

}  // namespace

std::string compile_plan(const PlanInput& in, PlanHost& p, int gemm_min_log2) {
  const int L = in.n_labels, T = in.n_tensors;
  if (L < 0 || L > (1 << 24)) return "n_labels out of range";
  if (T < 1) return "a plan needs at least one tensor";
  if (in.n_nodes != T - 1) return "n_nodes must be n_tensors - 1";
  if (!in.ix_off || !in.ix_lab) return "ixs missing";
  if (in.ix_off[0] != 0) return "ix_off[0] must be 0";
  p.n_labels = L; p.n_tensors = T; p.n_nodes = in.n_nodes;
  p.slice_index.assign(L, -1);
  for (int i = 0; i < in.n_sliced; i++) {
    int32_t x = in.sliced[i];
    if (x < 0 || x >= L || p.slice_index[x] >= 0) return "invalid sliced label";
    p.slice_index[x] = i;
    p.sliced.push_back(x);
  }
  std::vector<char> open(L, 0);
  for (int i = 0; i < in.n_iy; i++) {
    int32_t x = in.iy[i];
    if (x < 0 || x >= L || open[x]) return "invalid open label";
    if (p.slice_index[x] >= 0) return "a label cannot be both open and sliced";
    open[x] = 1;
    p.open.push_back(x);
  }
  const int total = T + in.n_nodes;
  p.labels.assign(total, {});
  p.leaf_raw.assign(T, {});
  std::vector<int> count(L, 0);
  for (int i = 0; i < T; i++) {
    if (in.ix_off[i + 1] < in.ix_off[i]) return "ix_off not monotone";
    for (int k = in.ix_off[i]; k < in.ix_off[i + 1]; k++) {
      int32_t x = in.ix_lab[k];
      if (x < 0 || x >= L) return "label out of range";
      p.leaf_raw[i].push_back(x);
      if (p.slice_index[x] < 0 && index_of(p.labels[i], x) < 0) p.labels[i].push_back(x);
    }
    if (p.leaf_raw[i].size() > 30) return "leaf tensor of rank above 30";
    for (int32_t x : p.labels[i]) count[x]++;
  }
  for (int32_t x : p.open)
    if (count[x] == 0) return "open label absent from every tensor";
  // tree structure and node output labels
  p.children.assign(in.children, in.children + 2 * in.n_nodes);
  std::vector<char> used(total, 0);
  std::vector<std::vector<std::pair<int32_t, int32_t>>> cnt(total);  // (label, leaves in subtree)
  for (int i = 0; i < T; i++)
    for (int32_t x : p.labels[i]) cnt[i].push_back({x, 1});
  for (int j = 0; j < in.n_nodes; j++) {
    int me = T + j;
    int a = in.children[2 * j], b = in.children[2 * j + 1];
    if (a < 0 || b < 0 || a >= me || b >= me || a == b) return "children must reference earlier ids";
    if (used[a] || used[b]) return "a tensor is used twice in the tree";
    used[a] = used[b] = 1;
    std::vector<int32_t> uni = p.labels[a];
    for (int32_t x : p.labels[b])
      if (index_of(uni, x) < 0) uni.push_back(x);
    auto c_of = [&](int id, int32_t x) {
      for (auto& pr : cnt[id])
        if (pr.first == x) return pr.second;
      return 0;
    };
    std::vector<int32_t> needed;
    for (int32_t x : uni) {
      int c = c_of(a, x) + c_of(b, x);
      if (count[x] - c > 0 || open[x]) needed.push_back(x);
      cnt[me].push_back({x, c});
    }
    if (in.node_iy_off) {
      std::vector<int32_t> given;
      for (int k = in.node_iy_off[j]; k < in.node_iy_off[j + 1]; k++) {
        int32_t x = in.node_iy_lab[k];
        if (x < 0 || x >= L) return "node label out of range";
        if (p.slice_index[x] >= 0) continue;
        if (index_of(uni, x) < 0) return "node label absent from its operands";
        if (index_of(given, x) >= 0) return "repeated node label";
        given.push_back(x);
      }
      for (int32_t x : needed)
        if (index_of(given, x) < 0) return "node output drops a label needed later";
      p.labels[me] = given;
    } else {
      p.labels[me] = needed;
    }
  }
  for (int i = 0; i < total; i++)
    if (p.labels[i].size() > 30) return "a tensor of rank > 30 (over 4 GiB) in the contraction tree";
  p.root = in.n_nodes ? total - 1 : 0;
  if (in.n_nodes && !in.node_iy_off) {
    // the root keeps exactly the open labels, in iy order
    p.labels[p.root] = p.open;
  }
  // arena: leaves, then node outputs, each 128-byte aligned
  p.off.assign(total, 0);
  int64_t pos = 0;
  for (int i = 0; i < total; i++) {
    p.off[i] = pos;
    pos = align_up(pos + (int64_t(1) << p.labels[i].size()), 32);
  }
  int64_t fused_end = pos;
  // the single-tensor case writes its reduced output after the leaf
  int64_t single_out = -1;
  std::vector<int32_t> single_labels;
  if (in.n_nodes == 0) {
    single_out = pos;
    single_labels = p.open;
    pos = align_up(pos + (int64_t(1) << single_labels.size()), 32);
    fused_end = pos;
  }
  p.arena_elems = fused_end;
  // complexity model
  p.tc = -INFINITY; p.sc = 0; p.rwc = -INFINITY; p.ops = 0; p.bytes = 0;
  p.node_ops.assign(in.n_nodes, 0.0);
  p.node_bytes.assign(in.n_nodes, 0.0);
  for (int i = 0; i < total; i++) p.sc = std::max(p.sc, (double)p.labels[i].size());
  for (int j = 0; j < in.n_nodes; j++) {
    int me = T + j, a = p.children[2 * j], b = p.children[2 * j + 1];
    std::vector<int32_t> uni = p.labels[a];
    for (int32_t x : p.labels[b])
      if (index_of(uni, x) < 0) uni.push_back(x);
    double t = (double)uni.size();
    p.tc = log2sumexp2(p.tc, t);
    double rw = log2sumexp2(log2sumexp2((double)p.labels[a].size(), (double)p.labels[b].size()),
                            (double)p.labels[me].size());
    p.rwc = log2sumexp2(p.rwc, rw);
    p.node_ops[j] = 2.0 * std::exp2(t);
    p.node_bytes[j] = 4.0 * (std::exp2((double)p.labels[a].size()) + std::exp2((double)p.labels[b].size()) +
                             std::exp2((double)p.labels[me].size()));
    p.ops += p.node_ops[j];
    p.bytes += p.node_bytes[j];
  }
  if (in.n_nodes == 0) {
    p.tc = (double)p.labels[0].size();
    p.rwc = p.tc;
    p.ops = std::exp2(p.tc);
    p.bytes = 4.0 * (std::exp2(p.tc) + std::exp2((double)single_labels.size()));
  }
  // leaves
  p.leaves.clear();
  for (int i = 0; i < T; i++) {
    LeafDesc ld;
    std::memset(&ld, 0, sizeof(ld));
    ld.off = p.off[i];
    ld.nraw = (int32_t)p.leaf_raw[i].size();
    ld.n_out = (int32_t)p.labels[i].size();
    for (int k = 0; k < 2; k++) {
      ld.out_bit[k] = -1;
      ld.slice_idx[k] = -1;
    }
    // MIS leaves have one or two labels; others only take explicit data
    for (int k = 0; k < ld.nraw && k < 2; k++) {
      int32_t x = p.leaf_raw[i][k];
      ld.out_bit[k] = (int8_t)index_of(p.labels[i], x);
      ld.slice_idx[k] = (int8_t)p.slice_index[x];
    }
    ld.label = ld.nraw == 1 ? p.leaf_raw[i][0] : -1;
    ld.w = 0.0f;
    p.leaves.push_back(ld);
  }
  // fused-form layouts, parents first: a GEMM-shaped node asks for its
  // operands in the k-pair interleaved layouts; any other node asks for its
  // operands ordered like its own output (shared labels first, in C order).
  p.flabels = p.labels;
  const int gmin = gemm_min_log2;
  std::vector<char> gemm_node(in.n_nodes, 0);
  auto loose = [&](int id) {
    // labels of tensor id that its own node keeps from exactly one operand
    std::vector<int32_t> out;
    if (id < T) return out;
    int jj = id - T, x = p.children[2 * jj], y = p.children[2 * jj + 1];
    for (int32_t l : p.labels[id]) {
      bool inx = index_of(p.labels[x], l) >= 0, iny = index_of(p.labels[y], l) >= 0;
      if (inx != iny) out.push_back(l);
    }
    return out;
  };
  for (int j = in.n_nodes - 1; j >= 0; j--) {
    int me = T + j, a = p.children[2 * j], b = p.children[2 * j + 1];
    const std::vector<int32_t>& C = p.flabels[me];
    const std::vector<int32_t>& SA = p.labels[a];
    const std::vector<int32_t>& SB = p.labels[b];
    std::vector<int32_t> M, N, K, Bt;
    bool priv = false;
    for (int32_t l : SA) {
      bool inb = index_of(SB, l) >= 0, inc = index_of(C, l) >= 0;
      if (inb && inc) Bt.push_back(l);
      else if (inb) K.push_back(l);
      else if (inc) M.push_back(l);
      else priv = true;
    }
    for (int32_t l : SB) {
      bool ina = index_of(SA, l) >= 0, inc = index_of(C, l) >= 0;
      if (!ina && inc) N.push_back(l);
      else if (!ina) priv = true;
    }
    // K = 16 (one BK = 16 chunk a tile) pays only with 64 x 64 tiles or
    // larger, or the 256 x 16 skinny tiles: below that the stream tile is
    // faster
    const int lo = (int)std::min(M.size(), N.size()), hi = (int)std::max(M.size(), N.size());
    const bool mn_ok = (int)K.size() > gmin ? lo >= gmin : (lo >= gmin + 2 || (lo >= gmin && hi >= 8));
    bool gemm = gmin > 0 && !priv && a >= T && b >= T && mn_ok && (int)K.size() >= gmin;
    auto by_c = [&](std::vector<int32_t>& v, const std::vector<int32_t>& pref) {
      std::stable_sort(v.begin(), v.end(), [&](int32_t x, int32_t y) {
        bool px = index_of(pref, x) >= 0, py = index_of(pref, y) >= 0;
        if (px != py) return px;
        int cx = index_of(C, x), cy = index_of(C, y);
        if (cx < 0) cx = 1 << 20;
        if (cy < 0) cy = 1 << 20;
        return cx < cy;
      });
    };
    if (gemm) {
      gemm_node[j] = 1;
      std::vector<int32_t> la = loose(a), lb = loose(b), none;
      // M / N order: the operand's producer prefers the labels it keeps from
      // one side first (they sit in its CTA tile); this node's own stores
      // prefer C's order (its tile then covers C's fastest positions).  The
      // larger of the two tensors decides.
      by_c(M, C.size() >= SA.size() ? none : la);
      by_c(N, C.size() >= SB.size() ? none : lb);
      by_c(Bt, none);
      // k0 sits at position 0 of both operands: prefer a label each operand's
      // own node keeps from one side (it is then inside that node's CTA tile)
      {
        int best = 0, bscore = -1;
        for (size_t q = 0; q < K.size(); q++) {
          int sc = (index_of(la, K[q]) >= 0 ? 2 : 0) + (index_of(lb, K[q]) >= 0 ? 2 : 0);
          if (sc > bscore) { bscore = sc; best = (int)q; }
        }
        std::swap(K[0], K[best]);
      }
      std::vector<int32_t> fa{K[0]}, fb{K[0]};
      fa.insert(fa.end(), M.begin(), M.end());
      fb.insert(fb.end(), N.begin(), N.end());
      fa.insert(fa.end(), K.begin() + 1, K.end());
      fb.insert(fb.end(), K.begin() + 1, K.end());
      fa.insert(fa.end(), Bt.begin(), Bt.end());
      fb.insert(fb.end(), Bt.begin(), Bt.end());
      p.flabels[a] = fa;
      p.flabels[b] = fb;
    } else {
      for (int c : {a, b}) {
        if (c < T) continue;  // leaves keep their natural layout
        std::vector<int32_t> v = p.labels[c], none;
        by_c(v, none);
        p.flabels[c] = v;
      }
    }
  }
  // fused steps: 0 = leaves, then one step per node (two for a GEMM node
  // with a split K: the parts, then their max), last = final
  p.steps.clear();
  p.tiles.clear();
  p.gemms.clear();
  p.step_node.clear();
  p.split_off.assign(in.n_nodes, -1);
  std::vector<int> step_of(total, 0);  // leaves -> step 0
  Step s0{STEP_LEAVES, 0, -1, -1, (T + kThreads - 1) / kThreads, 0};
  p.steps.push_back(s0);
  p.step_node.push_back(-1);
  p.total_tiles = s0.n_tiles;
  std::string e;
  int64_t extra = fused_end;  // K-part partials go after the tensors
  for (int j = 0; j < in.n_nodes; j++) {
    int me = T + j, a = p.children[2 * j], b = p.children[2 * j + 1];
    Step st{};
    GemmDesc g;
    if (gemm_node[j] &&
        plan_gemm(p.flabels[a], p.flabels[b], p.flabels[me], p.off[a], p.off[b], p.off[me], g)) {
      // split K when the output tiles alone leave the last wave of CTAs
      // mostly idle: the fewest parts that keep >= 90% of the CTA slots busy
      // (else the best), each unit keeping >= 2 K chunks of 32, <= 16 parts
      int ks = 0;
      {
        const int64_t ctas = std::max(1, p.gemm_ctas);
        double best_u = 0;
        for (int k2 = 0; k2 <= 4 && g.k_log2 - k2 >= 6 - (k2 == 0); k2++) {
          const int64_t units = (int64_t)g.n_tiles << k2;
          const double util = (double)units / (double)(((units + ctas - 1) / ctas) * ctas);
          if (util > best_u + 1e-9) {
            best_u = util;
            ks = k2;
          }
          if (util >= 0.9) break;
        }
      }
      if (ks > 0 && ((int64_t)g.n_tiles << ks) <= 0x7fffffffLL) {
        const int64_t csize = int64_t(1) << (g.m_log2 + g.n_log2 + g.bt_log2);
        const int64_t part_off = extra;
        extra = align_up(extra + (csize << ks), 32);
        g.c_fin = p.off[me];
        g.c_off = part_off;
        g.ks_log2 = ks;
        g.n_tiles <<= ks;
        // the K parts combine either by atomic max straight into the output,
        // which a fill step first sets to the identity (items whose values are
        // all >= 0 or -inf), or through partials and a max step.  The fill
        // comes after the A operand's step, and the GEMM waits for the fill.
        const int32_t gi = (int32_t)p.gemms.size();
        Step fs{STEP_FILL, gi, step_of[a], -1, (int32_t)((csize + kFillPerTile - 1) / kFillPerTile), 0};
        fs.level = 1 + p.steps[fs.dep0].level;
        p.steps.push_back(fs);
        p.step_node.push_back(-1);
        p.total_tiles += fs.n_tiles;
        Step gs{STEP_GEMM, gi, (int32_t)p.steps.size() - 1, step_of[b], g.n_tiles, 0};
        gs.level = 1 + std::max(p.steps[gs.dep0].level, p.steps[gs.dep1].level);
        p.gemms.push_back(g);
        p.steps.push_back(gs);
        p.step_node.push_back(j);
        p.total_tiles += gs.n_tiles;
        p.split_off[j] = part_off;
        // the max over the parts: a unary stream tile over [C..., part bits]
        std::vector<int32_t> pl = p.flabels[me];
        for (int q = 0; q < ks; q++) pl.push_back(kSplitLabel + q);
        TileDesc d;
        if (!(e = plan_tile(pl, nullptr, p.flabels[me], part_off, -1, p.off[me], d, p.tile_bits)).empty())
          return "node " + std::to_string(j) + " (K parts): " + e;
        st.kind = STEP_KRED;
        st.desc = (int32_t)p.tiles.size();
        st.n_tiles = d.n_tiles;
        p.tiles.push_back(d);
        st.dep0 = (int32_t)p.steps.size() - 1;
        st.dep1 = -1;
        st.level = gs.level + 1;
        step_of[me] = (int)p.steps.size();
        p.steps.push_back(st);
        p.step_node.push_back(-2 - j);
        p.total_tiles += st.n_tiles;
        continue;
      }
      g.c_fin = g.c_off;
      st.kind = STEP_GEMM;
      st.desc = (int32_t)p.gemms.size();
      st.n_tiles = g.n_tiles;
      p.gemms.push_back(g);
    } else {
      TileDesc d;
      if (!(e = plan_tile(p.flabels[a], &p.flabels[b], p.flabels[me], p.off[a], p.off[b], p.off[me], d,
                          p.tile_bits))
               .empty())
        return "node " + std::to_string(j) + ": " + e;
      st.kind = STEP_TILE;
      st.desc = (int32_t)p.tiles.size();
      st.n_tiles = d.n_tiles;
      p.tiles.push_back(d);
    }
    st.dep0 = step_of[a];
    st.dep1 = step_of[b];
    st.level = 1 + std::max(p.steps[st.dep0].level, p.steps[st.dep1].level);
    step_of[me] = (int)p.steps.size();
    p.steps.push_back(st);
    p.step_node.push_back(j);
    p.total_tiles += st.n_tiles;
  }
  int64_t root_off = p.off[p.root];
  int root_rank = (int)p.labels[p.root].size();
  if (in.n_nodes == 0) {
    // one tensor: reduce it to the open labels first
    TileDesc d;
    if (!(e = plan_tile(p.labels[0], nullptr, single_labels, p.off[0], -1, single_out, d)).empty())
      return "single tensor: " + e;
    Step st{STEP_TILE, (int32_t)p.tiles.size(), 0, -1, d.n_tiles, 1};
    p.tiles.push_back(d);
    step_of[0] = (int)p.steps.size();
    p.steps.push_back(st);
    p.step_node.push_back(-1);
    p.total_tiles += st.n_tiles;
    root_off = single_out;
    root_rank = (int)single_labels.size();
  }
  Step fin{STEP_FINAL, 0, (int32_t)p.steps.size() - 1, -1, 1, p.steps.back().level + 1};
  p.steps.push_back(fin);
  p.step_node.push_back(-1);
  p.levels.assign(fin.level + 1, {});
  for (size_t si = 0; si < p.steps.size(); si++) p.levels[p.steps[si].level].push_back((int32_t)si);
  p.total_tiles += 1;
  p.fin.root_off = root_off;
  p.fin.root_log2 = root_rank;
  p.fin.pad_ = 0;
  // plain lowering, scratch after the fused arena
  p.plain.assign(in.n_nodes, {});
  int64_t scratch = 0;
  for (int j = 0; j < in.n_nodes; j++) {
    int me = T + j, a = p.children[2 * j], b = p.children[2 * j + 1];
    if (!(e = lower_plain(p.labels[a], p.labels[b], p.labels[me], p.off[a], p.off[b], p.off[me], fused_end,
                          scratch, p.plain[j]))
             .empty())
      return "plain lowering of node " + std::to_string(j) + ": " + e;
  }
  p.plain_elems = fused_end + scratch;
  p.arena_elems = extra;  // the plain path never touches the K-part partials
  merge_split_k(p);
  compile_small(p);
  return "";
}

void merge_split_k(PlanHost& p) {
  p.steps_merged = p.steps;
  p.gemms_merged = p.gemms;
  p.has_split = false;
  std::vector<int32_t> to(p.steps.size());
  for (size_t si = 0; si < p.steps.size(); si++) to[si] = (int32_t)si;
  for (size_t si = 0; si < p.steps.size(); si++) {
    const Step& st = p.steps[si];
    if (st.kind == STEP_GEMM && p.gemms[st.desc].ks_log2 > 0) {
      GemmDesc& g = p.gemms_merged[st.desc];
      g.n_tiles >>= g.ks_log2;
      g.ks_log2 = 0;
      g.c_off = g.c_fin;
      Step& m = p.steps_merged[si];
      m.n_tiles = g.n_tiles;
      const Step& fill = p.steps[st.dep0];  // the fill waits on the A operand's step
      m.dep0 = fill.dep0;
      p.steps_merged[st.dep0].n_tiles = 0;
      p.has_split = true;
    } else if (st.kind == STEP_KRED) {
      p.steps_merged[si].n_tiles = 0;
      to[si] = st.dep0;  // its GEMM step
    }
  }
  for (Step& m : p.steps_merged) {
    if (m.dep0 >= 0) m.dep0 = to[m.dep0];
    if (m.dep1 >= 0) m.dep1 = to[m.dep1];
  }
}

void compile_small(PlanHost& p) {
  p.small_ok = false;
  p.small.clear();
  p.small_leaf.clear();
  const int T = p.n_tensors;
  const int total = T + p.n_nodes;
  for (int i = 0; i < total; i++)
    if ((int)p.labels[i].size() > kSmallMaxRank) return;
  for (int i = 0; i < T; i++)
    if (p.leaf_raw[i].empty() || p.leaf_raw[i].size() > 2) return;  // vertex and edge tensors only
  std::vector<int32_t> off(total, -1);
  int32_t end = 0;
  // first fit over free blocks (start, size), kept sorted and coalesced
  std::vector<std::pair<int32_t, int32_t>> fl;
  auto alloc = [&](int32_t n) -> int32_t {
    for (size_t k = 0; k < fl.size(); k++) {
      if (fl[k].second < n) continue;
      const int32_t o = fl[k].first;
      fl[k].first += n;
      fl[k].second -= n;
      if (fl[k].second == 0) fl.erase(fl.begin() + (long)k);
      return o;
    }
    if (!fl.empty() && fl.back().first + fl.back().second == end) {
      const int32_t o = fl.back().first;
      fl.pop_back();
      end = o + n;
      return o;
    }
    const int32_t o = end;
    end += n;
    return o;
  };
  auto release = [&](int32_t o, int32_t n) {
    const size_t k = (size_t)(std::lower_bound(fl.begin(), fl.end(), std::make_pair(o, 0)) - fl.begin());
    fl.insert(fl.begin() + (long)k, {o, n});
    if (k + 1 < fl.size() && fl[k].first + fl[k].second == fl[k + 1].first) {
      fl[k].second += fl[k + 1].second;
      fl.erase(fl.begin() + (long)k + 1);
    }
    if (k > 0 && fl[k - 1].first + fl[k - 1].second == fl[k].first) {
      fl[k - 1].second += fl[k].second;
      fl.erase(fl.begin() + (long)k);
    }
  };
  // leaves first (packed from 0); each is freed after the node that reads it
  for (int i = 0; i < T; i++) off[i] = alloc(1 << p.labels[i].size());
  std::vector<SmallNode> nodes;
  for (int j = 0; j < p.n_nodes; j++) {
    const int me = T + j, a = p.children[2 * j], b = p.children[2 * j + 1];
    if (a == b) return;
    const std::vector<int32_t>& A = p.labels[a];
    const std::vector<int32_t>& B = p.labels[b];
    const std::vector<int32_t>& C = p.labels[me];
    std::vector<int32_t> R;
    for (const std::vector<int32_t>* v : {&A, &B})
      for (int32_t x : *v)
        if (index_of(C, x) < 0 && index_of(R, x) < 0) R.push_back(x);
    for (int32_t x : C)
      if (index_of(A, x) < 0 && index_of(B, x) < 0) return;  // an output label no operand holds
    const int nc = (int)C.size(), nk = (int)R.size();
    if (nc + nk > kSmallMaxL) return;
    SmallNode nd;
    std::memset(&nd, 0, sizeof(nd));
    nd.a_off = off[a];
    nd.b_off = off[b];
    nd.c_off = alloc(1 << nc);
    nd.nc_nk = nc | (nk << 8);
    for (int i = 0; i < 16; i++) {
      uint32_t qa = 15, qb = 15;
      if (i < nc + nk) {
        const int32_t x = i < nc ? C[i] : R[i - nc];
        const int ia = index_of(A, x), ib = index_of(B, x);
        if (ia >= 0) qa = (uint32_t)ia;
        if (ib >= 0) qb = (uint32_t)ib;
      }
      nd.pa[i >> 3] |= qa << (4 * (i & 7));
      nd.pb[i >> 3] |= qb << (4 * (i & 7));
    }
    off[me] = nd.c_off;
    nodes.push_back(nd);
    release(off[a], 1 << A.size());
    release(off[b], 1 << B.size());
  }
  if (end > kSmallMaxWords) return;
  p.small = std::move(nodes);
  p.small_leaf.assign(off.begin(), off.begin() + T);
  p.small_words = end;
  p.small_root = off[p.root];
  p.small_root_log2 = (int32_t)p.labels[p.root].size();
  // per node: each thread's outputs times (address bits + reduced terms),
  // plus a fixed cost for the record and the barrier
  p.small_cost = 0;
  for (const SmallNode& nd : p.small) {
    const int nc = nd.nc_nk & 0xff, nk = (nd.nc_nk >> 8) & 0xff;
    p.small_cost += std::max(1.0, std::ldexp(1.0, nc - 7)) * (nc + 4.0 * std::ldexp(1.0, nk)) + 24.0;
  }
  p.small_ok = true;
}

std::string retile_plan(PlanHost& p, int bits) {
  if (bits < 8 || bits > 11) return "tile bits outside 8..11";
  const int T = p.n_tensors;
  if (p.n_nodes == 0) {
    p.tile_bits = bits;
    return "";
  }
  std::vector<TileDesc> tiles = p.tiles;
  std::vector<Step> steps = p.steps;
  int64_t total = 0;
  for (size_t si = 0; si < steps.size(); si++) {
    Step& st = steps[si];
    const int sn = p.step_node[si];
    if ((st.kind == STEP_TILE || st.kind == STEP_KRED) && sn != -1) {
      TileDesc d;
      std::string e;
      if (sn >= 0) {
        const int j = sn, me = T + j, a = p.children[2 * j], b = p.children[2 * j + 1];
        e = plan_tile(p.flabels[a], &p.flabels[b], p.flabels[me], p.off[a], p.off[b], p.off[me], d, bits);
      } else {
        const int j = -2 - sn, me = T + j;
        const GemmDesc& g = p.gemms[steps[st.dep0].desc];
        std::vector<int32_t> pl = p.flabels[me];
        for (int q = 0; q < g.ks_log2; q++) pl.push_back(kSplitLabel + q);
        e = plan_tile(pl, nullptr, p.flabels[me], p.split_off[j], -1, p.off[me], d, bits);
      }
      if (!e.empty()) return "step " + std::to_string(si) + ": " + e;
      tiles[st.desc] = d;
      st.n_tiles = d.n_tiles;
    }
    total += st.n_tiles;
  }
  p.tiles.swap(tiles);
  p.steps.swap(steps);
  p.total_tiles = total;
  p.tile_bits = bits;
  merge_split_k(p);
  return "";
}

}  // namespace tb
