// Host-side contraction-order tools for independent-set tensor networks.
//
// These produce the contraction trees that the GPU engine executes; they are
// not on the device path.  They restate, in our own code:
//   * an elimination order -> contraction tree builder, following the
//     semantics of order2eincode (src/decompose.jl:64-94, use_tree=false
//     branch: every elimination group is one vertex) including the isolated
//     vertex case (src/decompose.jl:71-73) and the final merge of connected
//     components (src/decompose.jl:88);
//   * a min-fill greedy elimination order (a stand-in for the TreeSA initial
//     tree used by initialize_code, src/dynamic_ob.jl:50-54);
//   * a tree simulated-annealing refiner over local rotations, the algorithm
//     that OMEinsumContractionOrders.TreeSA implements and that rethermalize
//     (src/utils.jl:142-144) and refine (src/refine.jl:1-19) call;
//   * the contraction complexity model (tc, sc, rwc) used by complexity()
//     (src/types.jl:115-121) and the peak-memory simulation of
//     contraction_peak_memory (src/utils.jl:197-219);
//   * a greedy index slicer that picks labels to fix until sc <= target.
//
// All tensors have dimension 2 per label, so sizes are powers of two and every
// complexity is the log2 of a sum of powers of two.
//
// Tree format ("post-order pairs"): internal node j (0-based) has children
// children[2j], children[2j+1]; an id < n_tensors is a leaf, an id
// n_tensors + k refers to internal node k < j.  The last internal node is the
// root.  A network of one tensor has no internal node.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <random>
#include <thread>
#include <vector>

namespace {

struct Bits {
  // dynamic bitset with a fixed number of 64-bit words per set
  int w = 0;
  std::vector<uint64_t> data;
  void init(int nsets, int nlabels) {
    w = (nlabels + 63) / 64;
    if (w == 0) w = 1;
    data.assign((size_t)nsets * w, 0);
  }
  uint64_t* at(int i) { return data.data() + (size_t)i * w; }
  const uint64_t* at(int i) const { return data.data() + (size_t)i * w; }
};

inline int popc(const uint64_t* a, int w) {
  int s = 0;
  for (int i = 0; i < w; i++) s += __builtin_popcountll(a[i]);
  return s;
}
inline int popc_or(const uint64_t* a, const uint64_t* b, int w) {
  int s = 0;
  for (int i = 0; i < w; i++) s += __builtin_popcountll(a[i] | b[i]);
  return s;
}
inline void set_bit(uint64_t* a, int i) { a[i >> 6] |= 1ull << (i & 63); }
inline bool get_bit(const uint64_t* a, int i) { return (a[i >> 6] >> (i & 63)) & 1; }

double log2sumexp2(double a, double b) {
  double m = std::max(a, b);
  if (m == -INFINITY) return m;
  return m + std::log2(std::exp2(a - m) + std::exp2(b - m));
}

// A binary contraction tree with per-node label sets.
//   S(leaf)     = the leaf's full label set
//   S(internal) = its output labels iy
struct Tree {
  int T = 0;   // leaves
  int L = 0;   // labels
  std::vector<int> left, right, parent;  // size 2T-1
  int root = -1;
  Bits S;
  Bits final_iy;  // one set

  int nnodes() const { return 2 * T - 1; }
  bool is_leaf(int n) const { return n < T; }
  int tc(int n) const { return popc_or(S.at(left[n]), S.at(right[n]), S.w); }
  int sc(int n) const { return popc(S.at(n), S.w); }
};

// Build label sets for leaves; returns false on invalid input.
bool load_leaves(Tree& t, int n_tensors, const int* ix_off, const int* ix_lab, int n_labels,
                 int n_iy, const int* iy) {
  t.T = n_tensors;
  t.L = n_labels;
  int nn = n_tensors > 0 ? 2 * n_tensors - 1 : 0;
  t.S.init(std::max(nn, 1), n_labels);
  t.final_iy.init(1, n_labels);
  t.left.assign(nn, -1);
  t.right.assign(nn, -1);
  t.parent.assign(nn, -1);
  for (int i = 0; i < n_tensors; i++) {
    for (int k = ix_off[i]; k < ix_off[i + 1]; k++) {
      int l = ix_lab[k];
      if (l < 0 || l >= n_labels) return false;
      set_bit(t.S.at(i), l);
    }
  }
  for (int k = 0; k < n_iy; k++) {
    if (iy[k] < 0 || iy[k] >= n_labels) return false;
    set_bit(t.final_iy.at(0), iy[k]);
  }
  return true;
}

// Recompute all internal output sets top-down from leaf sets:
// iy(n) = labels(subtree n) & (labels(outside n) | final_iy).
void recompute_sets(Tree& t) {
  int w = t.S.w, nn = t.nnodes();
  // bottom-up union of leaf labels (post-order: children ids < parent ids is
  // not guaranteed after rotations, so do an explicit DFS)
  Bits U;
  U.init(nn, t.L);
  std::vector<int> order;
  order.reserve(nn);
  std::vector<int> stack{t.root};
  while (!stack.empty()) {
    int n = stack.back();
    stack.pop_back();
    order.push_back(n);
    if (!t.is_leaf(n)) {
      stack.push_back(t.left[n]);
      stack.push_back(t.right[n]);
    }
  }
  for (int i = (int)order.size() - 1; i >= 0; i--) {
    int n = order[i];
    uint64_t* u = U.at(n);
    if (t.is_leaf(n)) {
      std::memcpy(u, t.S.at(n), sizeof(uint64_t) * w);
    } else {
      const uint64_t* a = U.at(t.left[n]);
      const uint64_t* b = U.at(t.right[n]);
      for (int k = 0; k < w; k++) u[k] = a[k] | b[k];
    }
  }
  // top-down "needed outside" sets: O(n) = outside labels of subtree n
  Bits O;
  O.init(nn, t.L);
  std::memcpy(O.at(t.root), t.final_iy.at(0), sizeof(uint64_t) * w);
  for (int n : order) {
    if (t.is_leaf(n)) continue;
    int a = t.left[n], b = t.right[n];
    for (int k = 0; k < w; k++) {
      O.at(a)[k] = O.at(n)[k] | U.at(b)[k];
      O.at(b)[k] = O.at(n)[k] | U.at(a)[k];
    }
    // iy of internal n
    for (int k = 0; k < w; k++) t.S.at(n)[k] = U.at(n)[k] & O.at(n)[k];
  }
}

struct Cost {
  double tc = -INFINITY, sc = 0, rw = -INFINITY;
};

Cost tree_cost(const Tree& t) {
  Cost c;
  for (int n = 0; n < t.T; n++) {
    c.sc = std::max(c.sc, (double)t.sc(n));
  }
  for (int n = t.T; n < t.nnodes(); n++) {
    int tcn = t.tc(n);
    c.tc = log2sumexp2(c.tc, (double)tcn);
    c.sc = std::max(c.sc, (double)t.sc(n));
    double rw = log2sumexp2(log2sumexp2((double)t.sc(t.left[n]), (double)t.sc(t.right[n])), (double)t.sc(n));
    c.rw = log2sumexp2(c.rw, rw);
  }
  if (t.T == 1) {
    c.tc = (double)t.sc(0);
    c.rw = (double)t.sc(0);
  }
  return c;
}

// Emit post-order pairs.  Internal nodes are renumbered in post-order.
void emit(const Tree& t, int* children) {
  if (t.T <= 1) return;
  std::vector<int> newid(t.nnodes(), -1);
  for (int i = 0; i < t.T; i++) newid[i] = i;
  int next = 0;
  // iterative post-order
  std::vector<std::pair<int, int>> st;
  st.push_back({t.root, 0});
  while (!st.empty()) {
    auto& top = st.back();
    int n = top.first;
    if (t.is_leaf(n)) {
      st.pop_back();
      continue;
    }
    if (top.second == 0) {
      top.second = 1;
      st.push_back({t.left[n], 0});
    } else if (top.second == 1) {
      top.second = 2;
      st.push_back({t.right[n], 0});
    } else {
      children[2 * next] = newid[t.left[n]];
      children[2 * next + 1] = newid[t.right[n]];
      newid[n] = t.T + next;
      next++;
      st.pop_back();
    }
  }
}

bool load_tree(Tree& t, const int* children) {
  int T = t.T;
  for (int j = 0; j < T - 1; j++) {
    int n = T + j;
    int a = children[2 * j], b = children[2 * j + 1];
    if (a < 0 || b < 0 || a >= n || b >= n || a == b) return false;
    if (t.parent[a] != -1 || t.parent[b] != -1) return false;
    t.left[n] = a;
    t.right[n] = b;
    t.parent[a] = n;
    t.parent[b] = n;
  }
  t.root = T == 1 ? 0 : 2 * T - 2;
  return true;
}

// ---------------------------------------------------------------------------
// elimination order -> tree (restates order2eincode with single-vertex groups)
// ---------------------------------------------------------------------------
bool tree_from_order(Tree& t, int n_order, const int* order) {
  int T = t.T, w = t.S.w, L = t.L;
  std::vector<int> cnt(L, 0);
  std::vector<char> alive(2 * T - 1, 0);
  std::vector<int> live;  // current tensor node ids
  for (int i = 0; i < T; i++) {
    alive[i] = 1;
    live.push_back(i);
    for (int l = 0; l < L; l++)
      if (get_bit(t.S.at(i), l)) cnt[l]++;
  }
  const uint64_t* fiy = t.final_iy.at(0);
  int next = T;
  auto merge = [&](int a, int b) {
    int n = next++;
    t.left[n] = a;
    t.right[n] = b;
    t.parent[a] = n;
    t.parent[b] = n;
    uint64_t* s = t.S.at(n);
    const uint64_t* sa = t.S.at(a);
    const uint64_t* sb = t.S.at(b);
    for (int k = 0; k < w; k++) s[k] = sa[k] | sb[k];
    for (int l = 0; l < L; l++) {
      if (!get_bit(s, l)) continue;
      cnt[l] -= (int)get_bit(sa, l) + (int)get_bit(sb, l);
      if (cnt[l] > 0 || get_bit(fiy, l)) {
        cnt[l]++;
      } else {
        s[l >> 6] &= ~(1ull << (l & 63));
      }
    }
    alive[a] = alive[b] = 0;
    alive[n] = 1;
    return n;
  };
  auto by_size = [&](int a, int b) {
    int pa = popc(t.S.at(a), w), pb = popc(t.S.at(b), w);
    return pa != pb ? pa < pb : a < b;
  };
  for (int oi = 0; oi < n_order; oi++) {
    int v = order[oi];
    if (v < 0 || v >= L) return false;
    std::vector<int> group;
    for (int n : live)
      if (alive[n] && get_bit(t.S.at(n), v)) group.push_back(n);
    if (group.size() < 2) continue;
    std::sort(group.begin(), group.end(), by_size);
    int cur = group[0];
    for (size_t g = 1; g < group.size(); g++) cur = merge(cur, group[g]);
    std::vector<int> nl;
    for (int n : live)
      if (alive[n]) nl.push_back(n);
    nl.push_back(cur);
    std::sort(nl.begin(), nl.end());
    nl.erase(std::unique(nl.begin(), nl.end()), nl.end());
    live.swap(nl);
  }
  // merge what remains (one tensor per connected component, plus labels
  // absent from the order), smallest first
  std::vector<int> rest;
  for (int n : live)
    if (alive[n]) rest.push_back(n);
  while (rest.size() > 1) {
    std::sort(rest.begin(), rest.end(), by_size);
    int n = merge(rest[0], rest[1]);
    rest.erase(rest.begin(), rest.begin() + 2);
    rest.push_back(n);
  }
  t.root = rest.empty() ? -1 : rest[0];
  return next == 2 * T - 1;
}

// ---------------------------------------------------------------------------
// min-fill elimination order of the label interaction graph
// ---------------------------------------------------------------------------
void minfill_order(int L, const std::vector<std::vector<char>>& adj0, uint64_t seed, int* out) {
  std::vector<std::vector<char>> adj = adj0;
  std::vector<char> done(L, 0);
  std::mt19937_64 rng(seed);
  for (int step = 0; step < L; step++) {
    int best = -1;
    long bestfill = -1, bestdeg = -1;
    uint64_t bestkey = 0;
    for (int v = 0; v < L; v++) {
      if (done[v]) continue;
      std::vector<int> nb;
      for (int u = 0; u < L; u++)
        if (!done[u] && adj[v][u]) nb.push_back(u);
      long fill = 0;
      for (size_t i = 0; i < nb.size(); i++)
        for (size_t j = i + 1; j < nb.size(); j++)
          if (!adj[nb[i]][nb[j]]) fill++;
      uint64_t key = rng();
      if (best < 0 || fill < bestfill || (fill == bestfill && (long)nb.size() < bestdeg) ||
          (fill == bestfill && (long)nb.size() == bestdeg && key < bestkey)) {
        best = v;
        bestfill = fill;
        bestdeg = (long)nb.size();
        bestkey = key;
      }
    }
    std::vector<int> nb;
    for (int u = 0; u < L; u++)
      if (!done[u] && adj[best][u]) nb.push_back(u);
    for (size_t i = 0; i < nb.size(); i++)
      for (size_t j = 0; j < nb.size(); j++)
        if (i != j) adj[nb[i]][nb[j]] = 1;
    done[best] = 1;
    out[step] = best;
  }
}

// ---------------------------------------------------------------------------
// simulated annealing over local tree rotations
// ---------------------------------------------------------------------------
struct SAParams {
  double sc_target, sc_weight, rw_weight;
  const double* betas;
  int nbetas, niters;
};

// Try one random rotation at internal node X; returns true if applied.
bool try_rotation(Tree& t, int X, double beta, const SAParams& p, std::mt19937_64& rng,
                  std::vector<uint64_t>& tmp) {
  int l = t.left[X], r = t.right[X];
  bool li = !t.is_leaf(l), ri = !t.is_leaf(r);
  if (!li && !ri) return false;
  int nrules = (li ? 2 : 0) + (ri ? 2 : 0);
  int rule = (int)(rng() % (uint64_t)nrules);
  if (!li) rule += 2;
  int w = t.S.w;
  // Generic form: X = (Y, o) with Y = (a, b); new Y = (a, o), X = (Y, b)
  // rules: 0: Y=l, keep a=l.left, swap b=l.right <-> o=r
  //        1: Y=l, keep a=l.right, swap b=l.left <-> o=r
  //        2: Y=r, keep a=r.left,  swap b=r.right <-> o=l
  //        3: Y=r, keep a=r.right, swap b=r.left <-> o=l
  int Y, a, b, o;
  if (rule == 0) { Y = l; a = t.left[l]; b = t.right[l]; o = r; }
  else if (rule == 1) { Y = l; a = t.right[l]; b = t.left[l]; o = r; }
  else if (rule == 2) { Y = r; a = t.left[r]; b = t.right[r]; o = l; }
  else { Y = r; a = t.right[r]; b = t.left[r]; o = l; }
  const uint64_t *Sa = t.S.at(a), *Sb = t.S.at(b), *So = t.S.at(o), *SX = t.S.at(X), *SY = t.S.at(Y);
  tmp.resize(w);
  int tcY_new = 0, scY_new = 0, tcX_new = 0;
  for (int k = 0; k < w; k++) {
    uint64_t un = Sa[k] | So[k];
    uint64_t ny = un & (Sb[k] | SX[k]);
    tmp[k] = ny;
    tcY_new += __builtin_popcountll(un);
    scY_new += __builtin_popcountll(ny);
    tcX_new += __builtin_popcountll(ny | Sb[k]);
  }
  int tcY_old = popc_or(Sa, Sb, w);
  int tcX_old = popc_or(SY, So, w);
  int scY_old = popc(SY, w);
  double dtc = log2sumexp2(tcY_new, tcX_new) - log2sumexp2(tcY_old, tcX_old);
  double pen_new = std::max(0.0, scY_new - p.sc_target);
  double pen_old = std::max(0.0, scY_old - p.sc_target);
  double dE = dtc + p.sc_weight * (pen_new - pen_old);
  if (p.rw_weight > 0) {
    double rw_old = log2sumexp2(log2sumexp2(t.sc(a), t.sc(b)), scY_old);
    double rw_new = log2sumexp2(log2sumexp2(t.sc(a), t.sc(o)), scY_new);
    dE += p.rw_weight * (rw_new - rw_old);
  }
  if (dE > 0) {
    double u = (double)(rng() >> 11) * (1.0 / 9007199254740992.0);
    if (u >= std::exp(-beta * dE)) return false;
  }
  // apply: Y gets children (a, o); X gets children (Y, b) keeping Y's side
  bool Yleft = (t.left[X] == Y);
  t.left[Y] = a;
  t.right[Y] = o;
  t.parent[a] = Y;
  t.parent[o] = Y;
  if (Yleft) { t.right[X] = b; } else { t.left[X] = b; }
  t.parent[b] = X;
  std::memcpy(t.S.at(Y), tmp.data(), sizeof(uint64_t) * w);
  return true;
}

void anneal(Tree& t, const SAParams& p, uint64_t seed) {
  std::mt19937_64 rng(seed);
  std::vector<uint64_t> tmp;
  std::vector<int> internal;
  for (int n = t.T; n < t.nnodes(); n++) internal.push_back(n);
  for (int bi = 0; bi < p.nbetas; bi++) {
    double beta = p.betas[bi];
    for (int it = 0; it < p.niters; it++) {
      std::shuffle(internal.begin(), internal.end(), rng);
      for (int X : internal) try_rotation(t, X, beta, p, rng, tmp);
    }
  }
}

bool better(const Cost& a, const Cost& b, double sc_target) {
  double pa = std::max(0.0, a.sc - sc_target), pb = std::max(0.0, b.sc - sc_target);
  if (pa != pb) return pa < pb;
  if (a.tc != b.tc) return a.tc < b.tc;
  return a.sc < b.sc;
}

std::vector<std::vector<char>> label_graph(const Tree& t) {
  std::vector<std::vector<char>> adj(t.L, std::vector<char>(t.L, 0));
  for (int i = 0; i < t.T; i++) {
    std::vector<int> ls;
    for (int l = 0; l < t.L; l++)
      if (get_bit(t.S.at(i), l)) ls.push_back(l);
    for (int x : ls)
      for (int y : ls)
        if (x != y) adj[x][y] = 1;
  }
  return adj;
}

// ---------------------------------------------------------------------------
// greedy pairwise contraction (the GreedyMethod of OMEinsumContractionOrders):
// repeatedly contract the pair of tensors sharing a label whose result grows
// the least, size(out) - size(a) - size(b), ties broken at random
// ---------------------------------------------------------------------------
bool greedy_tree(Tree& t, uint64_t seed) {
  const int T = t.T, w = t.S.w, L = t.L;
  std::mt19937_64 rng(seed);
  std::vector<int> cnt(L, 0);
  std::vector<char> alive(2 * T - 1, 0);
  for (int i = 0; i < T; i++) {
    alive[i] = 1;
    for (int l = 0; l < L; l++)
      if (get_bit(t.S.at(i), l)) cnt[l]++;
  }
  const uint64_t* fiy = t.final_iy.at(0);
  // label -> live tensors holding it
  std::vector<std::vector<int>> holders(L);
  for (int i = 0; i < T; i++)
    for (int l = 0; l < L; l++)
      if (get_bit(t.S.at(i), l)) holders[l].push_back(i);
  int next = T;
  std::vector<uint64_t> tmp(w);
  auto out_set = [&](int a, int b, uint64_t* o) {
    const uint64_t* sa = t.S.at(a);
    const uint64_t* sb = t.S.at(b);
    int sz = 0;
    for (int k = 0; k < w; k++) {
      uint64_t u = sa[k] | sb[k], keep = 0;
      while (u) {
        int bit = __builtin_ctzll(u);
        u &= u - 1;
        int l = k * 64 + bit;
        int c = cnt[l] - (int)get_bit(sa, l) - (int)get_bit(sb, l);
        if (c > 0 || get_bit(fiy, l)) keep |= 1ull << bit;
      }
      o[k] = keep;
      sz += __builtin_popcountll(keep);
    }
    return sz;
  };
  int live = T;
  while (live > 1) {
    double best = INFINITY;
    int ba = -1, bb = -1;
    uint64_t bkey = 0;
    for (int l = 0; l < L; l++) {
      auto& hs = holders[l];
      for (size_t x = 0; x < hs.size(); x++)
        for (size_t y = x + 1; y < hs.size(); y++) {
          int a = hs[x], b = hs[y];
          int so = out_set(a, b, tmp.data());
          double cost = std::exp2((double)so) - std::exp2((double)t.sc(a)) - std::exp2((double)t.sc(b));
          uint64_t key = rng();
          if (cost < best || (cost == best && key < bkey)) {
            best = cost;
            ba = a;
            bb = b;
            bkey = key;
          }
        }
    }
    if (ba < 0) {
      // no shared label left: merge the two smallest live tensors
      std::vector<int> ls;
      for (int i = 0; i < next; i++)
        if (alive[i]) ls.push_back(i);
      std::sort(ls.begin(), ls.end(), [&](int x, int y) { return t.sc(x) < t.sc(y); });
      ba = ls[0];
      bb = ls[1];
    }
    int n = next++;
    t.left[n] = ba;
    t.right[n] = bb;
    t.parent[ba] = n;
    t.parent[bb] = n;
    out_set(ba, bb, t.S.at(n));
    for (int l = 0; l < L; l++) {
      bool ina = get_bit(t.S.at(ba), l), inb = get_bit(t.S.at(bb), l);
      if (!ina && !inb) continue;
      cnt[l] -= (int)ina + (int)inb;
      auto& hs = holders[l];
      hs.erase(std::remove_if(hs.begin(), hs.end(), [&](int x) { return x == ba || x == bb; }), hs.end());
      if (get_bit(t.S.at(n), l)) {
        cnt[l]++;
        hs.push_back(n);
      }
    }
    alive[ba] = alive[bb] = 0;
    alive[n] = 1;
    live--;
  }
  t.root = next - 1;
  return next == 2 * T - 1;
}

}  // namespace

extern "C" {

// Greedy pairwise contraction tree (size-increase greedy, random ties).
int tbo_greedy_tree(int n_tensors, const int* ix_off, const int* ix_lab, int n_labels, int n_iy, const int* iy,
                    uint64_t seed, int* children) {
  if (n_tensors < 1) return 1;
  Tree t;
  if (!load_leaves(t, n_tensors, ix_off, ix_lab, n_labels, n_iy, iy)) return 1;
  if (n_tensors == 1) return 0;
  if (!greedy_tree(t, seed)) return 1;
  emit(t, children);
  return 0;
}

// Contraction complexity of a tree: tc = log2 sum_n 2^{|labels(n)|},
// sc = max log2 tensor size, rw = log2 of total read+write elements.
// Mirrors contraction_complexity as used by complexity() (src/types.jl:115-121).
int tbo_complexity(int n_tensors, const int* ix_off, const int* ix_lab, int n_labels, int n_iy,
                   const int* iy, const int* children, double* out3) {
  if (n_tensors < 1) return 1;
  Tree t;
  if (!load_leaves(t, n_tensors, ix_off, ix_lab, n_labels, n_iy, iy)) return 1;
  if (!load_tree(t, children)) return 1;
  recompute_sets(t);
  Cost c = tree_cost(t);
  out3[0] = c.tc;
  out3[1] = c.sc;
  out3[2] = c.rw;
  return 0;
}

// Output label sets of every internal node (iy), as a dense 0/1 matrix
// [n_tensors-1][n_labels] in post-order.
int tbo_node_labels(int n_tensors, const int* ix_off, const int* ix_lab, int n_labels, int n_iy,
                    const int* iy, const int* children, unsigned char* out) {
  if (n_tensors < 1) return 1;
  Tree t;
  if (!load_leaves(t, n_tensors, ix_off, ix_lab, n_labels, n_iy, iy)) return 1;
  if (!load_tree(t, children)) return 1;
  recompute_sets(t);
  for (int j = 0; j < n_tensors - 1; j++)
    for (int l = 0; l < n_labels; l++) out[(size_t)j * n_labels + l] = get_bit(t.S.at(n_tensors + j), l);
  return 0;
}

// Peak live elements (log2) of a post-order evaluation, restating
// contraction_peak_memory (src/utils.jl:197-219): all inputs live at start,
// each step allocates its output and frees its operands.
int tbo_peak_memory(int n_tensors, const int* ix_off, const int* ix_lab, int n_labels, int n_iy,
                    const int* iy, const int* children, double* out_log2) {
  if (n_tensors < 1) return 1;
  Tree t;
  if (!load_leaves(t, n_tensors, ix_off, ix_lab, n_labels, n_iy, iy)) return 1;
  if (!load_tree(t, children)) return 1;
  recompute_sets(t);
  double cur = 0;
  for (int i = 0; i < n_tensors; i++) cur += std::exp2((double)t.sc(i));
  double peak = cur;
  for (int j = 0; j < n_tensors - 1; j++) {
    int n = n_tensors + j;
    cur += std::exp2((double)t.sc(n));
    cur -= std::exp2((double)t.sc(t.left[n])) + std::exp2((double)t.sc(t.right[n]));
    peak = std::max(peak, cur);
  }
  *out_log2 = std::log2(peak);
  return 0;
}

// Min-fill greedy elimination order over the label interaction graph.
int tbo_minfill_order(int n_tensors, const int* ix_off, const int* ix_lab, int n_labels,
                      uint64_t seed, int* order_out) {
  Tree t;
  if (!load_leaves(t, n_tensors, ix_off, ix_lab, n_labels, 0, nullptr)) return 1;
  minfill_order(n_labels, label_graph(t), seed, order_out);
  return 0;
}

// Contraction tree from an elimination order (order2eincode semantics).
int tbo_tree_from_order(int n_tensors, const int* ix_off, const int* ix_lab, int n_labels, int n_iy,
                        const int* iy, int n_order, const int* order, int* children) {
  if (n_tensors < 1) return 1;
  Tree t;
  if (!load_leaves(t, n_tensors, ix_off, ix_lab, n_labels, n_iy, iy)) return 1;
  if (n_tensors == 1) return 0;
  if (!tree_from_order(t, n_order, order)) return 1;
  emit(t, children);
  return 0;
}

// Simulated-annealing refinement of a tree (TreeSA-style local rotations).
// `children` is read as the initial tree and overwritten with the best of
// `ntrials` independent annealing runs (run on up to `nthreads` threads).
// out3 receives (tc, sc, rw) of the result.
int tbo_treesa(int n_tensors, const int* ix_off, const int* ix_lab, int n_labels, int n_iy,
               const int* iy, int* children, double sc_target, double sc_weight, double rw_weight,
               const double* betas, int nbetas, int niters, int ntrials, int nthreads, uint64_t seed,
               double* out3) {
  if (n_tensors < 1) return 1;
  Tree base;
  if (!load_leaves(base, n_tensors, ix_off, ix_lab, n_labels, n_iy, iy)) return 1;
  if (!load_tree(base, children)) return 1;
  recompute_sets(base);
  if (n_tensors <= 2) {
    Cost c = tree_cost(base);
    out3[0] = c.tc; out3[1] = c.sc; out3[2] = c.rw;
    return 0;
  }
  SAParams p{sc_target, sc_weight, rw_weight, betas, nbetas, niters};
  std::vector<Tree> trees(std::max(ntrials, 1), base);
  std::vector<Cost> costs(trees.size());
  std::atomic<int> next{0};
  auto work = [&]() {
    for (;;) {
      int i = next.fetch_add(1);
      if (i >= (int)trees.size()) break;
      anneal(trees[i], p, seed * 1000003ull + (uint64_t)i * 7919ull + 17);
      costs[i] = tree_cost(trees[i]);
    }
  };
  int nt = std::max(1, std::min(nthreads, (int)trees.size()));
  std::vector<std::thread> th;
  for (int i = 1; i < nt; i++) th.emplace_back(work);
  work();
  for (auto& x : th) x.join();
  int best = 0;
  for (int i = 1; i < (int)trees.size(); i++)
    if (better(costs[i], costs[best], sc_target)) best = i;
  Cost c0 = tree_cost(base);
  if (better(c0, costs[best], sc_target)) {
    out3[0] = c0.tc; out3[1] = c0.sc; out3[2] = c0.rw;
    return 0;
  }
  emit(trees[best], children);
  out3[0] = costs[best].tc;
  out3[1] = costs[best].sc;
  out3[2] = costs[best].rw;
  return 0;
}

// Greedy index slicer: repeatedly fix the label that occurs in the most
// tensors of maximal size until sc <= sc_target (or max_slices labels are
// fixed).  Sliced labels are removed from every tensor; the tree shape is
// kept.  Returns the number of sliced labels in *n_sliced.
int tbo_greedy_slice(int n_tensors, const int* ix_off, const int* ix_lab, int n_labels, int n_iy,
                     const int* iy, const int* children, double sc_target, int max_slices,
                     int* sliced, int* n_sliced, double* out3) {
  if (n_tensors < 1) return 1;
  std::vector<int> off(ix_off, ix_off + n_tensors + 1);
  std::vector<int> lab(ix_lab, ix_lab + ix_off[n_tensors]);
  std::vector<char> removed(n_labels, 0);
  int ns = 0;
  for (;;) {
    // build label lists without removed labels
    std::vector<int> o2{0}, l2;
    for (int i = 0; i < n_tensors; i++) {
      for (int k = off[i]; k < off[i + 1]; k++)
        if (!removed[lab[k]]) l2.push_back(lab[k]);
      o2.push_back((int)l2.size());
    }
    std::vector<int> iy2;
    for (int k = 0; k < n_iy; k++)
      if (!removed[iy[k]]) iy2.push_back(iy[k]);
    Tree t;
    load_leaves(t, n_tensors, o2.data(), l2.data(), n_labels, (int)iy2.size(), iy2.data());
    load_tree(t, children);
    recompute_sets(t);
    Cost c = tree_cost(t);
    out3[0] = c.tc; out3[1] = c.sc; out3[2] = c.rw;
    if (c.sc <= sc_target || ns >= max_slices) break;
    // score labels by weighted presence in large tensors
    std::vector<double> score(n_labels, 0.0);
    for (int n = t.T; n < t.nnodes(); n++) {
      int s = t.sc(n);
      if (s <= sc_target) continue;
      double wgt = std::exp2((double)(s - sc_target));
      for (int l = 0; l < n_labels; l++)
        if (get_bit(t.S.at(n), l)) score[l] += wgt;
    }
    int best = -1;
    for (int l = 0; l < n_labels; l++)
      if (!removed[l] && (best < 0 || score[l] > score[best])) best = l;
    if (best < 0 || score[best] <= 0) break;
    removed[best] = 1;
    sliced[ns++] = best;
  }
  *n_sliced = ns;
  return 0;
}

}  // extern "C"
