/*
 * ORACLE -- test infrastructure only.  Nothing in the product path links,
 * loads or calls this file; only tests/, __graft_entry__.smoke() and the
 * cpu_baseline leg of bench.py use it, as the checker and as the timed CPU
 * stand-in for the reference's CPU contraction.
 *
 * CPU restatement of the arithmetic on the hot path of dynamic_ob_mis
 * (src/dynamic_ob.jl:30-48): the tropical (max,+) contraction of an
 * independent-set tensor network along a binary contraction tree.
 *
 * The arithmetic itself lives in third-party Julia packages that are not in
 * the reference tree (pins from Project.toml:25-41):
 *   GenericTensorNetworks 4.1  -- IndependentSet tensors: vertex [0, w_v],
 *                                 edge [[0,0],[0,-inf]] in Tropical{T}
 *                                 (called at src/dynamic_ob.jl:31-32, tests
 *                                 test/utils.jl:24, test/decompose.jl:27);
 *   OMEinsum 0.9.1             -- binary einsum lowered to permutedims + a
 *                                 batched GEMM, private labels reduced first
 *                                 (test/utils.jl:34, test/decompose.jl:28);
 *   TropicalNumbers 0.6.3      -- + is max, * is +, zero = -inf, one = 0;
 *   TropicalGEMM (test extra)  -- CPU max-plus GEMM (test/slice.jl:5).
 * Their published algorithms are restated here in our own code.  No golden
 * vectors exist in the reference (every reference test draws its graphs from
 * Julia's RNG); parity of this oracle with the Julia implementation itself is
 * UNPINNED.  It is pinned instead to the relations the reference tests check
 * (contraction MIS == exact MIS, test/utils.jl:34; sliced max + r == full
 * solve, test/slice.jl:32), which tests/ re-check with independent exact
 * solvers.
 *
 * Conventions: every label has dimension 2; tensors are column-major (the
 * first label is the fastest index), as in Julia.
 *
 * The file is compiled twice: once for float (suffix _f32, -inf sentinel) and
 * once with -DOR_I32 for int32 (suffix _i32, sentinel OR_NEG_I32 with every
 * accumulator starting at the sentinel, so sums never overflow).
 */
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef OR_I32
typedef int32_t VT;
#define NEGV ((int32_t)(-536870912)) /* INT32_MIN / 4 */
#define FN(x) x##_i32
#else
typedef float VT;
#define NEGV (-INFINITY)
#define FN(x) x##_f32
#endif

#define OR_MAXL 62

static inline VT vmax(VT a, VT b) { return a > b ? a : b; }

/* distinct labels of (ia, ib) in order of first appearance */
static int distinct(int na, const int* ia, int nb, const int* ib, int* out) {
  int n = 0;
  for (int s = 0; s < 2; s++) {
    int m = s ? nb : na;
    const int* l = s ? ib : ia;
    for (int i = 0; i < m; i++) {
      int seen = 0;
      for (int j = 0; j < n; j++)
        if (out[j] == l[i]) seen = 1;
      if (!seen) {
        if (n >= OR_MAXL) return -1;
        out[n++] = l[i];
      }
    }
  }
  return n;
}

static int index_of(const int* l, int n, int x) {
  for (int i = 0; i < n; i++)
    if (l[i] == x) return i;
  return -1;
}

/*
 * Generic binary tropical einsum, restating the einsum definition that
 * OMEinsum evaluates for Tropical eltypes:
 *   C[iy] = max over assignments of labels(ia) U labels(ib) that agree with iy
 *           of A[ia] + B[ib].
 * Repeated labels inside one operand select its diagonal.  B may be NULL
 * (unary: permute, diagonal and max-reduce).  Returns 0 on success.
 */
int FN(or_einsum_naive)(int na, const int* ia, const VT* A, int nb, const int* ib, const VT* B,
                        int nc, const int* ic, VT* C) {
  int lab[OR_MAXL];
  int nl = distinct(na, ia, B ? nb : 0, ib, lab);
  if (nl < 0 || nl > 40) return 1;
  for (int i = 0; i < nc; i++)
    if (index_of(lab, nl, ic[i]) < 0) return 2;
  int pa[OR_MAXL], pb[OR_MAXL], pc[OR_MAXL];
  for (int i = 0; i < na; i++) pa[i] = index_of(lab, nl, ia[i]);
  for (int i = 0; i < (B ? nb : 0); i++) pb[i] = index_of(lab, nl, ib[i]);
  for (int i = 0; i < nc; i++) pc[i] = index_of(lab, nl, ic[i]);
  uint64_t csize = 1ull << nc;
  for (uint64_t i = 0; i < csize; i++) C[i] = NEGV;
  uint64_t n = 1ull << nl;
  for (uint64_t x = 0; x < n; x++) {
    uint64_t ai = 0, bi = 0, ci = 0;
    for (int i = 0; i < na; i++) ai |= ((x >> pa[i]) & 1ull) << i;
    for (int i = 0; i < (B ? nb : 0); i++) bi |= ((x >> pb[i]) & 1ull) << i;
    for (int i = 0; i < nc; i++) ci |= ((x >> pc[i]) & 1ull) << i;
    VT v = B ? (VT)(A[ai] + B[bi]) : A[ai];
    if (v > C[ci]) C[ci] = v;
  }
  return 0;
}

/*
 * Unary permute / reduce with table-driven gathers (used by the GEMM-style
 * lowering).  X has labels ix (distinct), Y has labels iy, a subset of ix;
 * labels of ix absent from iy are max-reduced.
 */
static int unary_fast(int nx, const int* ix, const VT* X, int ny, const int* iy, VT* Y) {
  int pos[OR_MAXL];
  for (int i = 0; i < ny; i++) {
    pos[i] = index_of(ix, nx, iy[i]);
    if (pos[i] < 0) return 1;
  }
  int rp[OR_MAXL], nr = 0;
  for (int i = 0; i < nx; i++)
    if (index_of(iy, ny, ix[i]) < 0) rp[nr++] = i;
  /* gather tables for the output index, split in two halves */
  int lo = ny / 2, hi = ny - lo;
  uint64_t* tlo = (uint64_t*)malloc(sizeof(uint64_t) << lo);
  uint64_t* thi = (uint64_t*)malloc(sizeof(uint64_t) << hi);
  uint64_t* tr = (uint64_t*)malloc(sizeof(uint64_t) << nr);
  if (!tlo || !thi || !tr) { free(tlo); free(thi); free(tr); return 3; }
  for (uint64_t j = 0; j < (1ull << lo); j++) {
    uint64_t o = 0;
    for (int i = 0; i < lo; i++) o |= ((j >> i) & 1ull) << pos[i];
    tlo[j] = o;
  }
  for (uint64_t j = 0; j < (1ull << hi); j++) {
    uint64_t o = 0;
    for (int i = 0; i < hi; i++) o |= ((j >> i) & 1ull) << pos[lo + i];
    thi[j] = o;
  }
  for (uint64_t j = 0; j < (1ull << nr); j++) {
    uint64_t o = 0;
    for (int i = 0; i < nr; i++) o |= ((j >> i) & 1ull) << rp[i];
    tr[j] = o;
  }
  int64_t ysize = (int64_t)1 << ny;
  uint64_t lomask = (1ull << lo) - 1;
  uint64_t nred = 1ull << nr;
#pragma omp parallel for schedule(static) if (ysize > 65536)
  for (int64_t y = 0; y < ysize; y++) {
    uint64_t base = tlo[(uint64_t)y & lomask] | thi[(uint64_t)y >> lo];
    VT m = NEGV;
    for (uint64_t r = 0; r < nred; r++) m = vmax(m, X[base | tr[r]]);
    Y[y] = m;
  }
  free(tlo); free(thi); free(tr);
  return 0;
}

/* labels of l with repeats removed, and the diagonal of X taken on the fly */
static int dedup_operand(int n, const int* l, const VT* X, int* lout, VT** Xout) {
  int m = 0;
  for (int i = 0; i < n; i++)
    if (index_of(lout, m, l[i]) < 0) lout[m++] = l[i];
  if (m == n) { *Xout = NULL; return m; }
  VT* Y = (VT*)malloc(sizeof(VT) << m);
  if (!Y) return -1;
  if (FN(or_einsum_naive)(n, l, X, 0, NULL, NULL, m, lout, Y)) { free(Y); return -1; }
  *Xout = Y;
  return m;
}

/*
 * Binary tropical einsum through the lowering OMEinsum uses for binary rules:
 * reduce labels private to one operand, permute A to [M, K, batch] and B to
 * [K, N, batch], run a batched max-plus GEMM C'[m,n,b] = max_k A'[m,k,b] +
 * B'[k,n,b], then permute C' to iy.  (OMEinsum's binary rule dispatch;
 * TropicalGEMM supplies the GEMM for Tropical eltypes.)  OpenMP-parallel.
 */
int FN(or_einsum_gemm)(int na0, const int* ia0, const VT* A0, int nb0, const int* ib0, const VT* B0,
                       int nc, const int* ic, VT* C) {
  if (!B0) {
    int l[OR_MAXL]; VT* X = NULL;
    int n = dedup_operand(na0, ia0, A0, l, &X);
    if (n < 0) return 3;
    int rc = unary_fast(n, l, X ? X : A0, nc, ic, C);
    free(X);
    return rc;
  }
  int ia[OR_MAXL], ib[OR_MAXL];
  VT *Ad = NULL, *Bd = NULL;
  int na = dedup_operand(na0, ia0, A0, ia, &Ad);
  int nb = dedup_operand(nb0, ib0, B0, ib, &Bd);
  if (na < 0 || nb < 0) { free(Ad); free(Bd); return 3; }
  const VT* A = Ad ? Ad : A0;
  const VT* B = Bd ? Bd : B0;
  int M[OR_MAXL], N[OR_MAXL], K[OR_MAXL], Bt[OR_MAXL];
  int nm = 0, nn = 0, nk = 0, nbt = 0;
  for (int i = 0; i < na; i++) {
    int inb = index_of(ib, nb, ia[i]) >= 0, inc = index_of(ic, nc, ia[i]) >= 0;
    if (inb && inc) Bt[nbt++] = ia[i];
    else if (inb) K[nk++] = ia[i];
    else if (inc) M[nm++] = ia[i];
  }
  for (int i = 0; i < nb; i++) {
    int ina = index_of(ia, na, ib[i]) >= 0, inc = index_of(ic, nc, ib[i]) >= 0;
    if (!ina && inc) N[nn++] = ib[i];
  }
  for (int i = 0; i < nc; i++)
    if (index_of(ia, na, ic[i]) < 0 && index_of(ib, nb, ic[i]) < 0) { free(Ad); free(Bd); return 2; }
  int la[OR_MAXL], lb[OR_MAXL], lc[OR_MAXL];
  int p = 0;
  for (int i = 0; i < nm; i++) la[p++] = M[i];
  for (int i = 0; i < nk; i++) la[p++] = K[i];
  for (int i = 0; i < nbt; i++) la[p++] = Bt[i];
  int nla = p; p = 0;
  for (int i = 0; i < nk; i++) lb[p++] = K[i];
  for (int i = 0; i < nn; i++) lb[p++] = N[i];
  for (int i = 0; i < nbt; i++) lb[p++] = Bt[i];
  int nlb = p; p = 0;
  for (int i = 0; i < nm; i++) lc[p++] = M[i];
  for (int i = 0; i < nn; i++) lc[p++] = N[i];
  for (int i = 0; i < nbt; i++) lc[p++] = Bt[i];
  int nlc = p;
  VT* Ap = (VT*)malloc(sizeof(VT) << nla);
  VT* Bp = (VT*)malloc(sizeof(VT) << nlb);
  VT* Cp = (VT*)malloc(sizeof(VT) << nlc);
  int rc = 0;
  if (!Ap || !Bp || !Cp) { rc = 3; goto done; }
  if ((rc = unary_fast(na, ia, A, nla, la, Ap))) goto done;
  if ((rc = unary_fast(nb, ib, B, nlb, lb, Bp))) goto done;
  {
    int64_t Ms = (int64_t)1 << nm, Ns = (int64_t)1 << nn, Ks = (int64_t)1 << nk, Bs = (int64_t)1 << nbt;
    int64_t jobs = Bs * Ns;
#pragma omp parallel for schedule(static) if (jobs * Ms * Ks > 65536)
    for (int64_t job = 0; job < jobs; job++) {
      int64_t b = job / Ns, n = job % Ns;
      VT* c = Cp + (b * Ns + n) * Ms;
      const VT* a = Ap + b * Ms * Ks;
      const VT* bb = Bp + b * Ks * Ns + n * Ks;
      for (int64_t m = 0; m < Ms; m++) c[m] = NEGV;
      for (int64_t k = 0; k < Ks; k++) {
        VT bv = bb[k];
        const VT* ak = a + k * Ms;
        for (int64_t m = 0; m < Ms; m++) {
          VT v = (VT)(ak[m] + bv);
          c[m] = v > c[m] ? v : c[m];
        }
      }
    }
  }
  rc = unary_fast(nlc, lc, Cp, nc, ic, C);
done:
  free(Ap); free(Bp); free(Cp); free(Ad); free(Bd);
  return rc;
}

/*
 * Post-order executor of a binary contraction tree over an independent-set
 * network, restating solve_slice (src/dynamic_ob.jl:30-34):
 *   leaves with one label l are vertex tensors [0, w_l];
 *   leaves with two labels are edge tensors [[0,0],[0,-inf]]
 *     (two equal labels give the diagonal [0, -inf]);
 *   leaves may instead carry explicit data (leaf_data[i] != NULL).
 * `sliced` labels (n_fix of them, values fix_val) are fixed: every leaf is
 * restricted to the fixed value and the label is removed from every tensor,
 * the index slicing of a SlicedEinsum.
 * Node output labels are node_iy (explicit, post-order), each a subset of
 * its operands' labels.  Root result -> out (2^|iy_root| values).  A network
 * of one tensor has no node; node_iy entry 0 then holds its output labels.
 * When dump != NULL, dump[j] receives internal node j's tensor (caller
 * allocates 2^|node_iy_j| values).  mode 0: naive einsum, 1: GEMM lowering.
 */
int FN(or_execute)(int n_tensors, const int* ix_off, const int* ix_lab, const VT* const* leaf_data,
                   const VT* weights, int n_fix, const int* fix_lab, const signed char* fix_val,
                   int n_nodes, const int* children, const int* node_iy_off, const int* node_iy_lab,
                   VT* out, VT** dump, int mode) {
  if (n_tensors < 1 || n_nodes != n_tensors - 1) return 1;
  int total = n_tensors + n_nodes;
  VT** buf = (VT**)calloc((size_t)total, sizeof(VT*));
  int** labs = (int**)calloc((size_t)total, sizeof(int*));
  int* nlab = (int*)calloc((size_t)total, sizeof(int));
  int* refs = (int*)calloc((size_t)total, sizeof(int));
  int rc = 0;
  if (!buf || !labs || !nlab || !refs) { rc = 3; goto fail; }
  /* leaves */
  for (int i = 0; i < n_tensors; i++) {
    int n = ix_off[i + 1] - ix_off[i];
    const int* l = ix_lab + ix_off[i];
    if (n > OR_MAXL) { rc = 1; goto fail; }
    VT full[4];
    const VT* src = leaf_data ? leaf_data[i] : NULL;
    VT* tmp = NULL;
    if (!src) {
      if (n == 1) { full[0] = 0; full[1] = weights[l[0]]; }
      else if (n == 2) { full[0] = 0; full[1] = 0; full[2] = 0; full[3] = NEGV; }
      else { rc = 1; goto fail; }
      src = full;
    }
    /* restrict fixed labels: keep labels not fixed */
    int kept[OR_MAXL], nk = 0;
    for (int p = 0; p < n; p++)
      if (index_of(fix_lab, n_fix, l[p]) < 0) kept[nk++] = l[p];
    size_t sz = (size_t)1 << n;
    tmp = (VT*)malloc(sizeof(VT) * sz);
    if (!tmp) { rc = 3; goto fail; }
    for (size_t x = 0; x < sz; x++) {
      int ok = 1;
      for (int p = 0; p < n; p++) {
        int f = index_of(fix_lab, n_fix, l[p]);
        if (f >= 0 && (int)((x >> p) & 1u) != (int)fix_val[f]) ok = 0;
      }
      tmp[x] = ok ? src[x] : NEGV;
    }
    /* distinct kept labels (diagonal for repeats), fixed labels reduced */
    int dl[OR_MAXL], nd = 0;
    for (int p = 0; p < nk; p++)
      if (index_of(dl, nd, kept[p]) < 0) dl[nd++] = kept[p];
    buf[i] = (VT*)malloc(sizeof(VT) << nd);
    labs[i] = (int*)malloc(sizeof(int) * (nd ? nd : 1));
    if (!buf[i] || !labs[i]) { free(tmp); rc = 3; goto fail; }
    if (FN(or_einsum_naive)(n, l, tmp, 0, NULL, NULL, nd, dl, buf[i])) { free(tmp); rc = 1; goto fail; }
    free(tmp);
    memcpy(labs[i], dl, sizeof(int) * nd);
    nlab[i] = nd;
  }
  for (int j = 0; j < n_nodes; j++) {
    int a = children[2 * j], b = children[2 * j + 1];
    int me = n_tensors + j;
    if (a < 0 || b < 0 || a >= me || b >= me || refs[a] || refs[b]) { rc = 1; goto fail; }
    refs[a] = refs[b] = 1;
    int n = node_iy_off[j + 1] - node_iy_off[j];
    const int* l = node_iy_lab + node_iy_off[j];
    int dl[OR_MAXL], nd = 0;
    for (int p = 0; p < n; p++)
      if (index_of(fix_lab, n_fix, l[p]) < 0) dl[nd++] = l[p];
    buf[me] = (VT*)malloc(sizeof(VT) << nd);
    labs[me] = (int*)malloc(sizeof(int) * (nd ? nd : 1));
    if (!buf[me] || !labs[me]) { rc = 3; goto fail; }
    memcpy(labs[me], dl, sizeof(int) * nd);
    nlab[me] = nd;
    rc = mode == 0 ? FN(or_einsum_naive)(nlab[a], labs[a], buf[a], nlab[b], labs[b], buf[b], nd, dl, buf[me])
                   : FN(or_einsum_gemm)(nlab[a], labs[a], buf[a], nlab[b], labs[b], buf[b], nd, dl, buf[me]);
    if (rc) goto fail;
    if (dump && dump[j]) memcpy(dump[j], buf[me], sizeof(VT) << nd);
    free(buf[a]); buf[a] = NULL;
    free(buf[b]); buf[b] = NULL;
  }
  if (n_nodes) {
    memcpy(out, buf[total - 1], sizeof(VT) << nlab[total - 1]);
  } else {
    /* a single tensor: node_iy entry 0 holds the output labels */
    int n = node_iy_off[1] - node_iy_off[0];
    const int* l = node_iy_lab + node_iy_off[0];
    int dl[OR_MAXL], nd = 0;
    for (int p = 0; p < n; p++)
      if (index_of(fix_lab, n_fix, l[p]) < 0) dl[nd++] = l[p];
    rc = FN(or_einsum_naive)(nlab[0], labs[0], buf[0], 0, NULL, NULL, nd, dl, out);
  }
fail:
  if (buf) for (int i = 0; i < total; i++) free(buf[i]);
  if (labs) for (int i = 0; i < total; i++) free(labs[i]);
  free(buf); free(labs); free(nlab); free(refs);
  return rc;
}

#ifndef OR_I32
/* OpenMP threads of every later call (the benchmark's single-thread and
 * all-core CPU baselines); n <= 0 restores every host core. */
void or_set_threads(int n) { omp_set_num_threads(n > 0 ? n : omp_get_num_procs()); }
int or_get_threads(void) { return omp_get_max_threads(); }
#endif
