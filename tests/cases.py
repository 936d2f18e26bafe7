"""Small seeded networks shared by the tests."""
import numpy as np


def rr_case(tb, n, seed, weighted=True, optimizer=None):
    g = tb.random_regular_graph(n, 3, seed)
    w = tb.random_weights(n, seed) if weighted else np.ones(n, np.float32)
    code = tb.initialize_code(g, optimizer or tb.GreedyMethod(seed))
    return g, w, code


def ksg_case(tb, L, seed, filling=0.8, weighted=False):
    g = tb.random_ksg(L, filling, seed)
    w = tb.random_weights(g.n, seed) if weighted else np.ones(g.n, np.float32)
    code = tb.initialize_code(g, tb.GreedyMethod(seed))
    return g, w, code


def corner_cases(tb):
    """Disconnected graphs, isolated vertices, self-loops, one vertex."""
    out = []
    g = tb.Graph(9, [(0, 1), (1, 2), (3, 4), (5, 5), (6, 7)])
    out.append(("disconnected", g, np.arange(1, 10, dtype=np.float32)))
    out.append(("single", tb.Graph(1, []), np.array([3.0], np.float32)))
    out.append(("edge", tb.Graph(2, [(0, 1)]), np.array([2.0, 5.0], np.float32)))
    out.append(("isolated", tb.Graph(4, []), np.array([1.0, 2.0, 0.0, 4.0], np.float32)))
    out.append(("selfloops", tb.Graph(3, [(0, 0), (1, 1), (0, 2)]), np.array([5.0, 4.0, 1.0], np.float32)))
    res = []
    for name, g, w in out:
        res.append((name, g, w, tb.initialize_code(g, tb.GreedyMethod(0))))
    return res


def random_generic_network(rng, n_labels=10, n_tensors=6, max_rank=4, n_open=0):
    """A random tensor network (not an MIS one) with a random binary tree."""
    ixs = []
    for _ in range(n_tensors):
        r = int(rng.integers(1, max_rank + 1))
        ixs.append([int(x) for x in rng.choice(n_labels, r, replace=False)])
    used = sorted(set(x for ix in ixs for x in ix))
    iy = [int(x) for x in rng.choice(used, min(n_open, len(used)), replace=False)]
    live = list(range(n_tensors))
    ch = []
    nxt = n_tensors
    while len(live) > 1:
        i, j = rng.choice(len(live), 2, replace=False)
        a, b = live[i], live[j]
        live = [x for k, x in enumerate(live) if k not in (i, j)]
        ch.append((a, b))
        live.append(nxt)
        nxt += 1
    return ixs, iy, np.array(ch, np.int32).reshape(-1, 2)


def random_tensor(rng, rank, p_neg=0.15):
    t = rng.integers(-6, 7, 1 << rank).astype(np.float32)
    t[rng.random(t.size) < p_neg] = -np.inf
    return t


def _merge_seq(ids, ch, nxt):
    cur = ids[0]
    for x in ids[1:]:
        ch.append((cur, x))
        cur = nxt[0]
        nxt[0] += 1
    return cur


def gemm_case(tb, m=4, n=4, k=4, bt=1, seed=0):
    """An MIS network whose middle node is a GEMM (workloads.gemm_node_network)."""
    from tensorbranching_gb300 import workloads

    return workloads.gemm_node_network(m, n, k, bt, seed)
