"""The CPU oracle: its three einsum restatements agree, and its MIS values
match exact solvers that use no tensor network (the relation every reference
test checks: contraction MIS == mis2, test/utils.jl:34)."""
import numpy as np
import pytest

from cases import corner_cases, ksg_case, random_generic_network, random_tensor, rr_case


def test_einsum_restatements_agree(orc):
    rng = np.random.default_rng(0)
    for _ in range(300):
        ra, rb = int(rng.integers(0, 6)), int(rng.integers(0, 6))
        ia = [int(x) for x in rng.choice(9, ra, replace=False)]
        ib = [int(x) for x in rng.choice(9, rb, replace=False)]
        uni = list(dict.fromkeys(ia + ib))
        ic = [x for x in uni if rng.random() < 0.5]
        rng.shuffle(ic)
        A, B = random_tensor(rng, ra), random_tensor(rng, rb)
        c1 = orc.einsum(ia, A, ib, B, ic, "naive")
        c2 = orc.einsum(ia, A, ib, B, ic, "gemm")
        c3 = orc.einsum_numpy(ia, A, ib, B, ic)
        assert np.array_equal(c1, c2) and np.array_equal(c1, c3)


def test_einsum_unary_and_diagonal(orc):
    rng = np.random.default_rng(1)
    for _ in range(100):
        r = int(rng.integers(1, 6))
        ia = [int(x) for x in rng.choice(4, r)]  # repeats allowed: diagonals
        ic = [x for x in dict.fromkeys(ia) if rng.random() < 0.6]
        A = random_tensor(rng, r)
        c1 = orc.einsum(ia, A, None, None, ic, "naive")
        c2 = orc.einsum(ia, A, None, None, ic, "gemm")
        c3 = orc.einsum_numpy(ia, A, None, None, ic)
        assert np.array_equal(c1, c2) and np.array_equal(c1, c3)


def test_int32_matches_f32(orc):
    rng = np.random.default_rng(2)
    for _ in range(100):
        ra, rb = int(rng.integers(1, 5)), int(rng.integers(1, 5))
        ia = [int(x) for x in rng.choice(7, ra, replace=False)]
        ib = [int(x) for x in rng.choice(7, rb, replace=False)]
        ic = [x for x in dict.fromkeys(ia + ib) if rng.random() < 0.5]
        A, B = random_tensor(rng, ra), random_tensor(rng, rb)
        Ai = np.where(np.isinf(A), orc.I32_NEG, A).astype(np.int32)
        Bi = np.where(np.isinf(B), orc.I32_NEG, B).astype(np.int32)
        cf = orc.einsum(ia, A, ib, B, ic, "gemm")
        ci = orc.einsum(ia, Ai, ib, Bi, ic, "gemm", dtype=np.int32)
        ci = np.where(ci <= orc.I32_NEG // 2, -np.inf, ci).astype(np.float32)
        assert np.array_equal(cf, ci)


@pytest.mark.parametrize("seed", range(6))
def test_mis_vs_bruteforce(tb, orc, exact, seed):
    g, w, code = rr_case(tb, 20 + 2 * (seed % 3), seed, weighted=seed % 2 == 0)
    v = orc.solve(code, w)
    assert v == exact.brute_force(g.n, g.edges, w)
    assert v == orc.solve(code, w, mode="naive")


@pytest.mark.parametrize("seed", range(3))
def test_mis_vs_branch_and_bound_and_ip(tb, orc, exact, seed):
    g, w, code = rr_case(tb, 50, seed, weighted=True)
    v = orc.solve(code, w)
    assert v == exact.branch_and_bound(g.n, g.edges, w)
    assert v == exact.ip(g.n, g.edges, w)


def test_ksg_mis(tb, orc, exact):
    for seed in range(3):
        g, w, code = ksg_case(tb, 6, seed)
        assert orc.solve(code, w) == exact.branch_and_bound(g.n, g.edges, w)


def test_corner_cases(tb, orc, exact):
    for name, g, w, code in corner_cases(tb):
        assert orc.solve(code, w) == exact.brute_force(g.n, g.edges, w), name


def test_sliced_max_equals_full(tb, orc):
    """max over 2^k slices + r == full contraction (test/slice.jl:32)."""
    g, w, code = rr_case(tb, 24, 3)
    full = orc.solve(code, w)
    sl = [1, 4, 7]
    vals = []
    for s in range(8):
        sv = [(s >> k) & 1 for k in range(3)]
        vals.append(orc.solve(code, w, sliced=sl, slice_vals=sv))
    assert max(vals) == full


def test_generic_networks_naive_vs_gemm(tb, orc):
    rng = np.random.default_rng(5)
    for _ in range(40):
        ixs, iy, ch = random_generic_network(rng, n_labels=9, n_tensors=6, max_rank=4, n_open=int(rng.integers(0, 3)))
        code = tb.CompressedEinsum(ixs, iy, ch)
        data = [random_tensor(rng, len(ix)) for ix in ixs]
        a = orc.execute(code, None, leaf_data=data, mode="naive")
        b = orc.execute(code, None, leaf_data=data, mode="gemm")
        assert np.array_equal(a, b)
