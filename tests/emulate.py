"""CPU emulation of the engine's device programs (test infrastructure).

Reads a compiled plan through the library's internal ``tbi_plan_describe``
(host-only, no GPU) and replays the index arithmetic of the kernels in
csrc/kernels.cuh with numpy: the leaf builder, the stream tile (grid bits,
load tables, XOR swizzle, thread-to-output mapping, reduction split, store
tables), the final max and the K1 GEMM of the plain lowering.  Every global
and shared-memory access is checked against the buffer it must stay in and
every output element must be written exactly once, so a descriptor that
would read or write out of bounds fails here, before it reaches a GPU.
"""
from __future__ import annotations

import ctypes
from ctypes import c_int8, c_int32, c_int64, c_void_p, c_float

import numpy as np

KMAXBITS = 48
KMAXTILE = 16
KTHREADS = 256
KMAXOPT = 8
KSMEM = 8192
KDESCWORDS = 108  # descriptor copy in front of the operand buffers


class TileDesc(ctypes.Structure):
    _fields_ = [("a_off", c_int64), ("b_off", c_int64), ("c_off", c_int64),
                ("n_grid", c_int32), ("n_loop", c_int32), ("n_tc", c_int32), ("n_tr", c_int32),
                ("na", c_int32), ("nb", c_int32), ("pa", c_int32), ("pb", c_int32), ("pc", c_int32),
                ("split_log2", c_int32), ("n_tiles", c_int32), ("pad_", c_int32),
                ("g_pa", c_int8 * KMAXBITS), ("g_pb", c_int8 * KMAXBITS), ("g_pc", c_int8 * KMAXBITS),
                ("l_pa", c_int8 * KMAXBITS), ("l_pb", c_int8 * KMAXBITS),
                ("ta_pos", c_int8 * KMAXTILE), ("tb_pos", c_int8 * KMAXTILE), ("tc_pos", c_int8 * KMAXTILE),
                ("tc_a", c_int8 * KMAXTILE), ("tc_b", c_int8 * KMAXTILE),
                ("tr_a", c_int8 * KMAXTILE), ("tr_b", c_int8 * KMAXTILE)]


KTINYOUT, KTINYRED = 8, 5


class TinyDesc(ctypes.Structure):
    _fields_ = [("a_off", c_int64), ("b_off", c_int64), ("c_off", c_int64), ("n_tc", c_int8), ("n_tr", c_int8),
                ("oa", c_int8 * KTINYOUT), ("ob", c_int8 * KTINYOUT), ("oc", c_int8 * KTINYOUT),
                ("ra", c_int8 * KTINYRED), ("rb", c_int8 * KTINYRED), ("pad_", c_int8 * 4)]


class Step(ctypes.Structure):
    _fields_ = [("kind", c_int32), ("desc", c_int32), ("dep0", c_int32), ("dep1", c_int32),
                ("n_tiles", c_int32), ("level", c_int32)]


class LeafDesc(ctypes.Structure):
    _fields_ = [("off", c_int64), ("nraw", c_int32), ("n_out", c_int32), ("out_bit", c_int8 * 2),
                ("slice_idx", c_int8 * 2), ("label", c_int32), ("w", c_float)]


class FinalDesc(ctypes.Structure):
    _fields_ = [("root_off", c_int64), ("root_log2", c_int32), ("pad_", c_int32)]


class GemmDesc(ctypes.Structure):
    _fields_ = [("a_off", c_int64), ("b_off", c_int64), ("c_off", c_int64), ("c_fin", c_int64),
                ("m_log2", c_int32), ("n_log2", c_int32), ("k_log2", c_int32), ("bt_log2", c_int32),
                ("bm_log2", c_int32), ("bn_log2", c_int32), ("n_tiles", c_int32), ("ks_log2", c_int32),
                ("m_pc", c_int8 * 32), ("n_pc", c_int8 * 32), ("b_pc", c_int8 * 32)]


class PlainRec(ctypes.Structure):
    _fields_ = [("node", c_int32), ("kind", c_int32), ("tile", TileDesc), ("a", c_int64), ("b", c_int64),
                ("c", c_int64), ("M", c_int64), ("N", c_int64), ("K", c_int64), ("batch", c_int64)]


STEP_LEAVES, STEP_TILE, STEP_GEMM, STEP_FINAL, STEP_FILL, STEP_KRED = 1, 2, 3, 4, 5, 6
PLAIN_TILE, PLAIN_GEMM = 1, 2


def check_layout(lib):
    out = (c_int32 * 6)()
    lib.tbi_sizes(out, 6)
    want = [ctypes.sizeof(TileDesc), ctypes.sizeof(Step), ctypes.sizeof(LeafDesc), ctypes.sizeof(FinalDesc),
            ctypes.sizeof(GemmDesc), ctypes.sizeof(TinyDesc)]
    assert list(out) == want, (list(out), want)


def describe(lib, code, sliced=(), use_node_iy=False, gemm_min=4, tile_bits=9):
    lib.tbi_plan_describe.restype = c_int32
    lib.tbi_plan_describe.argtypes = [c_int32, c_int32, c_void_p, c_void_p, c_int32, c_void_p, c_int32, c_void_p,
                                      c_void_p, c_void_p, c_int32, c_void_p, c_int32, c_int32, ctypes.POINTER(c_void_p),
                                      ctypes.POINTER(c_int64), ctypes.c_char_p, c_int32]
    lib.tbi_free.argtypes = [c_void_p]
    lib.tbi_sizes.argtypes = [c_void_p, c_int32]
    check_layout(lib)
    off, lab = code.csr()
    iy = np.array(code.iy if code.iy else [0], np.int32)
    ch = code.children if code.n_nodes else np.zeros((1, 2), np.int32)
    noff, nlab = code.node_iy_csr() if use_node_iy else (None, None)
    sl = np.array(list(sliced) if len(sliced) else [0], np.int32)
    blob = c_void_p()
    nbytes = c_int64()
    err = ctypes.create_string_buffer(512)
    rc = lib.tbi_plan_describe(code.n_labels, code.n_tensors, off.ctypes.data, lab.ctypes.data, len(code.iy),
                               iy.ctypes.data, code.n_nodes, ch.ctypes.data,
                               None if noff is None else noff.ctypes.data,
                               None if nlab is None else nlab.ctypes.data, len(sliced), sl.ctypes.data,
                               gemm_min, tile_bits, ctypes.byref(blob), ctypes.byref(nbytes), err, 512)
    if rc:
        raise ValueError(err.value.decode())
    raw = ctypes.string_at(blob, nbytes.value)
    lib.tbi_free(blob)
    p = 0
    hdr = np.frombuffer(raw, np.int64, 9, p); p += 72
    n_tensors, n_nodes, n_steps, n_tiles, n_leaves, arena, plain_elems, nplain, ngemm = [int(x) for x in hdr]
    total = n_tensors + n_nodes
    offs = np.frombuffer(raw, np.int64, total, p).copy(); p += 8 * total
    ranks = np.frombuffer(raw, np.int32, total, p).copy(); p += 4 * total
    labels, flabels = [], []
    for i in range(total):
        r = int(ranks[i])
        labels.append(np.frombuffer(raw, np.int32, r, p).tolist()); p += 4 * r
        flabels.append(np.frombuffer(raw, np.int32, r, p).tolist()); p += 4 * r

    def take(cls, n):
        nonlocal p
        out = []
        for _ in range(n):
            out.append(cls.from_buffer_copy(raw[p:p + ctypes.sizeof(cls)]))
            p += ctypes.sizeof(cls)
        return out

    steps = take(Step, n_steps)
    tiles = take(TileDesc, n_tiles)
    leaves = take(LeafDesc, n_leaves)
    fin = take(FinalDesc, 1)[0]
    gemms = take(GemmDesc, ngemm)
    plain = take(PlainRec, nplain)
    # the merged split-K form (PlanHost::steps_merged, gemms_merged)
    steps_merged = take(Step, n_steps)
    gemms_merged = take(GemmDesc, ngemm)
    assert p == len(raw)
    return dict(n_tensors=n_tensors, n_nodes=n_nodes, steps=steps, tiles=tiles, leaves=leaves, fin=fin,
                plain=plain, off=offs, rank=ranks, arena=arena, plain_elems=plain_elems, gemms=gemms,
                labels=labels, flabels=flabels, steps_merged=steps_merged, gemms_merged=gemms_merged)


def merged(desc):
    """The descriptor with its merged split-K form as the program."""
    d = dict(desc)
    d["steps"], d["gemms"] = desc["steps_merged"], desc["gemms_merged"]
    return d


def dep_order(steps):
    """An order of the steps that follows only their dependencies (not the
    list or level order), taking the latest ready step first, with the
    steps that have no tiles left out.  A step without tiles counts as done
    from the start, as in the persistent executor (its done count 0 meets
    its tile count 0).  A dependency missing from the program shows up as a
    read of an unwritten operand."""
    n = len(steps)
    deps = [[d for d in (s.dep0, s.dep1) if d >= 0] if s.n_tiles > 0 else [] for s in steps]
    users = [[] for _ in range(n)]
    for i, ds in enumerate(deps):
        for d in ds:
            users[d].append(i)
    left = [len(ds) for ds in deps]
    ready = [i for i in range(n) if left[i] == 0]
    out = []
    while ready:
        ready.sort()
        i = ready.pop()
        out.append(i)
        for u in users[i]:
            left[u] -= 1
            if left[u] == 0:
                ready.append(u)
    assert len(out) == n, "dependency cycle"
    return [i for i in out if steps[i].n_tiles > 0]


def swz(j):
    """16-byte-granular XOR swizzle of the stream tile (swz16)."""
    return j ^ ((((j >> 5) ^ (j >> 10)) & 7) << 2)


def a_words(d):
    return ((1 << d.na) + 3) & ~3


def buf_words(d):
    return a_words(d) + ((((1 << d.nb) + 3) & ~3) if d.b_off >= 0 else 0)


def stages(d):
    """Pipeline depth of the stream tile (stream_stages)."""
    return max(2, min(8, (2 * KSMEM) // buf_words(d)))


def smem_words(d):
    hasB = d.b_off >= 0
    w = KDESCWORDS + stages(d) * buf_words(d)
    w += 1 << (d.na - d.pa)
    w += (1 << (d.nb - d.pb)) if hasB else 0
    w += 1 << (d.n_tc - d.pc)
    w += 2 * (1 << d.n_tr)
    w += KTHREADS
    return w


def max_smem_words():
    return KDESCWORDS + 2 * KSMEM + 3 * 512 + 2 * 256 + KTHREADS


def tensor_rank(tile_pos, grid_pos, loop_pos):
    """Positions a tile descriptor uses for one tensor must be 0..r-1, each
    exactly once; returns r."""
    ps = [int(x) for x in tile_pos] + [int(x) for x in grid_pos if x >= 0] + [int(x) for x in loop_pos if x >= 0]
    r = len(ps)
    assert sorted(ps) == list(range(r)), f"tensor positions not a permutation: {sorted(ps)}"
    return r


class Neg:
    f32 = np.float32(-np.inf)


def emu_stream_tile(d, arena, written, expect=None):
    """Run every CTA of one stream-tile descriptor on the arena (in place)."""
    hasB = d.b_off >= 0
    ra = tensor_rank(d.ta_pos[:d.na], d.g_pa[:d.n_grid], d.l_pa[:d.n_loop])
    rb = tensor_rank(d.tb_pos[:d.nb], d.g_pb[:d.n_grid], d.l_pb[:d.n_loop]) if hasB else 0
    rc = tensor_rank(d.tc_pos[:d.n_tc], d.g_pc[:d.n_grid], [])
    if expect is not None:
        assert (ra, rb, rc) == expect, ((ra, rb, rc), expect)
    assert smem_words(d) <= max_smem_words()
    assert d.n_tiles == 1 << d.n_grid
    assert d.a_off % 32 == 0 or d.pa == 0 or True
    a_lo, a_hi = d.a_off, d.a_off + (1 << ra)
    b_lo, b_hi = (d.b_off, d.b_off + (1 << rb)) if hasB else (0, 0)
    c_lo, c_hi = d.c_off, d.c_off + (1 << rc)
    assert 0 <= a_lo and a_hi <= arena.size and c_hi <= arena.size and b_hi <= arena.size
    NA = 1 << d.na
    NB = (1 << d.nb) if hasB else 0
    nAh = 1 << (d.na - d.pa)
    nBh = (1 << (d.nb - d.pb)) if hasB else 0
    nCh = 1 << (d.n_tc - d.pc)
    ntr = 1 << d.n_tr
    ldA = np.array([sum(1 << d.ta_pos[d.pa + b] for b in range(d.na - d.pa) if (j >> b) & 1) for j in range(nAh)],
                   np.int64)
    ldB = np.array([sum(1 << d.tb_pos[d.pb + b] for b in range(d.nb - d.pb) if (j >> b) & 1) for j in range(nBh)],
                   np.int64)
    stC = np.array([sum(1 << d.tc_pos[d.pc + b] for b in range(d.n_tc - d.pc) if (j >> b) & 1) for j in range(nCh)],
                   np.int64)
    IAr = np.zeros(ntr, np.int64)
    IBr = np.zeros(ntr, np.int64)
    for j in range(ntr):
        xa = xb = 0
        for b in range(d.n_tr):
            if (j >> b) & 1:
                if d.tr_a[b] >= 0:
                    xa |= 1 << d.tr_a[b]
                if d.tr_b[b] >= 0:
                    xb |= 1 << d.tr_b[b]
        IAr[j] = swz(xa)
        IBr[j] = swz(xb)
    lo_bits = min(d.n_tc, 8)
    split = d.split_log2
    active = 1 << (lo_bits + split)
    opt = 1 << (d.n_tc - lo_bits)
    assert opt <= KMAXOPT and active <= KTHREADS
    t = np.arange(KTHREADS)
    act = t < active
    cl = t & ((1 << lo_bits) - 1)
    s = t >> lo_bits

    def part(xbits, tab):
        out = np.zeros_like(xbits)
        for b in range(d.n_tc):
            if tab[b] >= 0:
                out |= ((xbits >> b) & 1) << tab[b]
        return out

    iat = swz(part(cl, d.tc_a))
    ibt = swz(part(cl, d.tc_b))
    neg = np.float32(-np.inf)
    for tile in range(d.n_tiles):
        oa, ob, oc = d.a_off, d.b_off, d.c_off
        for i in range(d.n_grid):
            if (tile >> i) & 1:
                if d.g_pa[i] >= 0:
                    oa += 1 << d.g_pa[i]
                if d.g_pb[i] >= 0:
                    ob += 1 << d.g_pb[i]
                oc += 1 << d.g_pc[i]
        acc = np.full((KTHREADS, opt), neg, np.float32)
        for rl in range(1 << d.n_loop):
            la, lb = oa, ob
            for i in range(d.n_loop):
                if (rl >> i) & 1:
                    if d.l_pa[i] >= 0:
                        la += 1 << d.l_pa[i]
                    if d.l_pb[i] >= 0:
                        lb += 1 << d.l_pb[i]

            def load(base, n, p, hi, lo, hi_b, region):
                j = np.arange(1 << n)
                g = base + (j & ((1 << p) - 1)) + hi[j >> p]
                assert g.min() >= lo and g.max() < hi_b, "global load out of bounds"
                # async copies: 16 bytes when p >= 2, 8 when p == 1; both ends aligned
                for b in range(stages(d)):  # every pipeline buffer
                    dst = KDESCWORDS + b * buf_words(d) + region + swz(j)
                    if p >= 2:
                        assert np.all(g[::4] % 4 == 0), "misaligned 16-byte global source"
                        assert np.all(dst[::4] % 4 == 0), "misaligned 16-byte shared destination"
                        assert np.all(np.diff(dst.reshape(-1, 4), axis=1) == 1), "16-byte chunk split by swizzle"
                    elif p == 1:
                        assert np.all(g[::2] % 2 == 0), "misaligned 8-byte global source"
                        assert np.all(dst[::2] % 2 == 0), "misaligned 8-byte shared destination"
                sm = np.empty(1 << n, np.float32)
                ph = swz(j)
                assert sorted(ph.tolist()) == list(range(1 << n))
                sm[ph] = arena[g]
                return sm

            As = load(la, d.na, d.pa, ldA, a_lo, a_hi, 0)
            Bs = load(lb, d.nb, d.pb, ldB, b_lo, b_hi, a_words(d)) if hasB else None
            act_idx = np.nonzero(act)[0]
            step = 1 << split
            nq = ntr // step
            rmat = s[act_idx][:, None] + step * np.arange(nq)[None, :]  # reductions per thread
            for i in range(opt):
                xa = np.zeros(KTHREADS, np.int64)
                xb = np.zeros(KTHREADS, np.int64)
                for b in range(lo_bits, d.n_tc):
                    if ((i << lo_bits) >> b) & 1:
                        if d.tc_a[b] >= 0:
                            xa |= 1 << d.tc_a[b]
                        if d.tc_b[b] >= 0:
                            xb |= 1 << d.tc_b[b]
                ia = (iat ^ swz(xa))[act_idx]
                ib = (ibt ^ swz(xb))[act_idx]
                idxa = ia[:, None] ^ IAr[rmat]
                assert idxa.max() < NA and idxa.min() >= 0
                v = As[idxa]
                if hasB:
                    idxb = ib[:, None] ^ IBr[rmat]
                    assert idxb.max() < NB and idxb.min() >= 0
                    v = v + Bs[idxb]
                acc[act_idx, i] = np.maximum(acc[act_idx, i], v.max(axis=1))
        if split > 0:
            red = acc[:, 0].copy()
            for tt in np.nonzero(act & (s == 0))[0]:
                acc[tt, 0] = max(red[cl[tt] + (s2 << lo_bits)] for s2 in range(1 << split))
        cmask = (1 << d.pc) - 1
        wr = np.nonzero(act & (s == 0))[0]
        for i in range(opt):
            c = cl[wr] + (i << lo_bits)
            g = oc + (c & cmask) + stC[c >> d.pc]
            assert g.min() >= c_lo and g.max() < c_hi, "store out of bounds"
            np.add.at(written, g, 1)
            arena[g] = acc[wr, i]
    return (c_lo, c_hi)


def emu_leaves(leaves, arena, written, slice_vals):
    for ld in leaves:
        for e in range(1 << ld.n_out):
            best = -np.inf
            for raw in range(1 << ld.nraw):
                ok = True
                for k in range(ld.nraw):
                    x = (raw >> k) & 1
                    if ld.slice_idx[k] >= 0:
                        ok &= x == int(slice_vals[ld.slice_idx[k]])
                    else:
                        ok &= ((e >> ld.out_bit[k]) & 1) == x
                if not ok:
                    continue
                v = (ld.w if raw & 1 else 0.0) if ld.nraw == 1 else (-np.inf if raw == 3 else 0.0)
                best = max(best, v)
            assert 0 <= ld.off + e < arena.size
            arena[ld.off + e] = best
            written[ld.off + e] += 1


def emu_gemm(rec, arena):
    M, N, K, B = rec.M, rec.N, rec.K, rec.batch
    assert M % 16 == 0 and N % 16 == 0 and K % 16 == 0
    for x, n in ((rec.a, M * K * B), (rec.b, K * N * B), (rec.c, M * N * B)):
        assert 0 <= x and x + n <= arena.size and x % 4 == 0
    A = arena[rec.a:rec.a + M * K * B].reshape(B, K, M)
    Bm = arena[rec.b:rec.b + K * N * B].reshape(B, N, K)
    C = (A[:, None, :, :] + Bm[:, :, :, None]).max(axis=2)  # (B, N, M)
    arena[rec.c:rec.c + M * N * B] = C.reshape(-1)


GEMM_TILES = {(7, 7), (7, 6), (6, 7), (6, 6), (5, 5), (4, 4), (8, 4), (4, 8)}


def emu_gemm_step(g, arena, written, kpart_atomic=False):
    """Fused GEMM tile: k-pair interleaved operands, scatter store to C (or,
    with a split K, part p of the partials at c_off + p |C|, or every part
    by atomic max of the value bits into the output c_fin)."""
    assert (g.bm_log2, g.bn_log2) in GEMM_TILES
    assert g.m_log2 >= g.bm_log2 and g.n_log2 >= g.bn_log2 and g.k_log2 >= 4  # K = 16: BK = 16 tiles
    ks = g.ks_log2
    assert 0 <= ks <= 4 and (ks == 0 or g.k_log2 - ks >= 6)
    M, N, K, Bt = 1 << g.m_log2, 1 << g.n_log2, 1 << g.k_log2, 1 << g.bt_log2
    assert g.n_tiles == (M >> g.bm_log2) * (N >> g.bn_log2) * Bt << ks
    rc = tensor_rank([g.m_pc[i] for i in range(g.m_log2)] + [g.n_pc[i] for i in range(g.n_log2)] +
                     [g.b_pc[i] for i in range(g.bt_log2)], [], [])
    for x, n in ((g.a_off, M * K * Bt), (g.b_off, N * K * Bt), (g.c_off, (1 << rc) << ks)):
        assert 0 <= x and x + n <= arena.size and x % 32 == 0
    for x, n in ((g.a_off, M * K * Bt), (g.b_off, N * K * Bt)):
        assert np.all(written[x:x + n] == 1), "GEMM operand not written before the GEMM step"
    # bulk copies: rows of 2*BM (2*BN) elements at 2*m0 within a k-pair row
    BM, BN = 1 << g.bm_log2, 1 << g.bn_log2
    assert (2 * BM * 4) % 16 == 0 and (2 * BN * 4) % 16 == 0
    A = arena[g.a_off:g.a_off + M * K * Bt].reshape(Bt, K // 2, M, 2)   # [b][kp][m][k&1]
    B = arena[g.b_off:g.b_off + N * K * Bt].reshape(Bt, K // 2, N, 2)
    A = A.transpose(0, 1, 3, 2).reshape(Bt, 1 << ks, K >> ks, M)
    B = B.transpose(0, 1, 3, 2).reshape(Bt, 1 << ks, K >> ks, N)
    C = (A[:, :, :, None, :] + B[:, :, :, :, None]).max(axis=2)  # (Bt, P, N, M)
    C = C.transpose(1, 0, 2, 3)  # (P, Bt, N, M)
    def scat(nbits, pos):
        idx = np.arange(1 << nbits)
        out = np.zeros(1 << nbits, np.int64)
        for q in range(nbits):
            out |= ((idx >> q) & 1) << pos[q]
        return out
    sm = scat(g.m_log2, g.m_pc)
    sn = scat(g.n_log2, g.n_pc)
    sb = scat(g.bt_log2, g.b_pc)
    if kpart_atomic and ks > 0:
        addr = g.c_fin + sb[None, :, None, None] + sn[None, None, :, None] + sm[None, None, None, :]
        addr = np.broadcast_to(addr, C.shape).ravel()
        vals = np.ascontiguousarray(C, np.float32).ravel()
        assert np.all((vals >= 0) | (vals == -np.inf)), "atomic parts need values >= 0 or -inf"
        assert np.all(written[addr] == 1), "the output was not filled first"
        bits = arena.view(np.int32)
        np.maximum.at(bits, addr, vals.view(np.int32))
        return
    part = (np.arange(1 << ks, dtype=np.int64) << rc)
    addr = g.c_off + part[:, None, None, None] + sb[None, :, None, None] + sn[None, None, :, None] + \
        sm[None, None, None, :]
    arena[addr.ravel()] = C.ravel()
    np.add.at(written, addr.ravel(), 1)


def to_reported(v, flab, lab):
    if flab == lab:
        return v
    pos = [flab.index(x) for x in lab]
    e = np.arange(v.size)
    x = np.zeros(v.size, np.int64)
    for q, pq in enumerate(pos):
        x |= ((e >> q) & 1) << pq
    return v[x]


def tiny_desc(lib, d):
    """(is tiny, TinyDesc) of a stream-tile descriptor, from the engine."""
    lib.tbi_tiny_desc.restype = c_int32
    lib.tbi_tiny_desc.argtypes = [c_void_p, c_void_p]
    t = TinyDesc()
    rc = lib.tbi_tiny_desc(ctypes.byref(d), ctypes.byref(t))
    assert rc in (0, 1)
    return bool(rc), t


def emu_tiny_node(t, arena, written):
    """tiny_node: lane l of a pass takes term l mod 2^n_tr of output
    c0 + (l >> n_tr); offsets are sums of 2^position over the set bits of
    the output and term indices; the terms meet in a max."""
    n_tc, n_tr = t.n_tc, t.n_tr
    assert 0 <= n_tc <= KTINYOUT and 0 <= n_tr <= KTINYRED and n_tc + n_tr <= 10
    hasB = t.b_off >= 0

    def offs(nbits, pos, idx):
        o = np.zeros(idx.shape, np.int64)
        for b in range(nbits):
            if pos[b] >= 0:
                o += ((idx >> b) & 1) << pos[b]
        return o

    c = np.arange(1 << n_tc)[:, None]
    r = np.arange(1 << n_tr)[None, :]
    oa = offs(n_tc, t.oa, c) + offs(n_tr, t.ra, r)
    oc = offs(n_tc, t.oc, c)[:, 0]
    assert len(set(oc.tolist())) == len(oc), "outputs collide"
    va = arena[t.a_off + oa]
    assert np.all(written[t.a_off + oa] == 1)
    if hasB:
        ob = offs(n_tc, t.ob, c) + offs(n_tr, t.rb, r)
        assert np.all(written[t.b_off + ob] == 1)
        va = va + arena[t.b_off + ob]
    arena[t.c_off + oc] = va.max(axis=1)
    written[t.c_off + oc] += 1


def run_fused(desc, weights, slice_vals=(), kpart_atomic=False, by_deps=False, lib=None):
    """Replay the fused program; returns (root tensor, arena, node views).
    kpart_atomic: split-K parts combine by atomic max of the value bits into
    the output after STEP_FILL (the form for values >= 0 or -inf), instead of
    partials and STEP_KRED.  by_deps: run the steps in dep_order.  lib: run
    the steps the per-level launches take as tiny steps through their
    TinyDesc (emu_tiny_node), as those launches do."""
    arena = np.full(desc["arena"], np.nan, np.float32)
    written = np.zeros(desc["arena"], np.int32)
    leaves = desc["leaves"]
    for i, ld in enumerate(leaves):
        if ld.nraw == 1:
            pass
    # weights: the engine binds w into LeafDesc; do the same here
    T = desc["n_tensors"]
    for ld, w in zip(leaves, weights):
        ld.w = float(w)
    emu_leaves(leaves, arena, written, slice_vals)
    off, rank = desc["off"], desc["rank"]
    node_of_step = {}
    j = 0
    order = dep_order(desc["steps"]) if by_deps else range(len(desc["steps"]))
    for si in order:
        st = desc["steps"][si]
        if st.kind == STEP_FILL:
            if kpart_atomic:
                g = desc["gemms"][st.desc]
                size = 1 << (g.m_log2 + g.n_log2 + g.bt_log2)
                assert g.c_fin % 32 == 0 and g.c_fin + size <= arena.size
                assert st.n_tiles == -(-size // 4096)
                arena[g.c_fin:g.c_fin + size].view(np.int32)[:] = np.int32(-2 ** 31)
                written[g.c_fin:g.c_fin + size] += 1
            continue
        if st.kind == STEP_KRED and kpart_atomic:
            continue
        if st.kind in (STEP_TILE, STEP_KRED):
            d = desc["tiles"][st.desc]
            expect = None
            if desc["n_nodes"]:
                # node j's operands are its children; ranks known from the blob
                node_of_step[si] = j
                j += 1
            tiny, t = tiny_desc(lib, d) if lib is not None and st.kind == STEP_TILE else (False, None)
            if tiny:
                emu_tiny_node(t, arena, written)
            else:
                emu_stream_tile(d, arena, written)
        elif st.kind == STEP_GEMM:
            emu_gemm_step(desc["gemms"][st.desc], arena, written, kpart_atomic)
    fin = desc["fin"]
    root = arena[fin.root_off:fin.root_off + (1 << fin.root_log2)].copy()
    assert np.all(written[fin.root_off:fin.root_off + (1 << fin.root_log2)] == 1), "root not written exactly once"
    # every node output written exactly once
    for idx in range(T, T + desc["n_nodes"]):
        seg = written[off[idx]:off[idx] + (1 << rank[idx])]
        assert np.all(seg == 1), f"tensor {idx} elements written {np.unique(seg)} times"
    nodes = [to_reported(arena[off[T + k]:off[T + k] + (1 << rank[T + k])].copy(), desc["flabels"][T + k],
                         desc["labels"][T + k]) for k in range(desc["n_nodes"])]
    return root, nodes


def run_plain(desc, weights, slice_vals=()):
    arena = np.full(desc["plain_elems"], np.nan, np.float32)
    written = np.zeros(desc["plain_elems"], np.int32)
    for ld, w in zip(desc["leaves"], weights):
        ld.w = float(w)
    emu_leaves(desc["leaves"], arena, written, slice_vals)
    for rec in desc["plain"]:
        if rec.kind == PLAIN_TILE:
            emu_stream_tile(rec.tile, arena, written)
        else:
            emu_gemm(rec, arena)
    if desc["n_nodes"] == 0:
        emu_stream_tile(desc["tiles"][0], arena, written)
    fin = desc["fin"]
    T = desc["n_tensors"]
    off, rank = desc["off"], desc["rank"]
    nodes = [arena[off[T + k]:off[T + k] + (1 << rank[T + k])].copy() for k in range(desc["n_nodes"])]
    return arena[fin.root_off:fin.root_off + (1 << fin.root_log2)].copy(), nodes


# ---------------------------------------------------------------------------
# fused small form (k_small): one block, the whole network in shared memory
# ---------------------------------------------------------------------------
class SmallNode(ctypes.Structure):
    _fields_ = [("a_off", c_int32), ("b_off", c_int32), ("c_off", c_int32), ("nc_nk", c_int32),
                ("pa", ctypes.c_uint32 * 2), ("pb", ctypes.c_uint32 * 2)]


def describe_small(lib, code, sliced=()):
    """The plan's small form through ``tbi_plan_small`` (host only)."""
    lib.tbi_plan_small.restype = c_int32
    lib.tbi_plan_small.argtypes = [c_int32, c_int32, c_void_p, c_void_p, c_int32, c_void_p, c_int32, c_void_p,
                                   c_int32, c_void_p, ctypes.POINTER(c_void_p), ctypes.POINTER(c_int64),
                                   ctypes.c_char_p, c_int32]
    lib.tbi_free.argtypes = [c_void_p]
    off, lab = code.csr()
    iy = np.array(code.iy if code.iy else [0], np.int32)
    ch = code.children if code.n_nodes else np.zeros((1, 2), np.int32)
    sl = np.array(list(sliced) if len(sliced) else [0], np.int32)
    blob, nbytes = c_void_p(), c_int64()
    err = ctypes.create_string_buffer(512)
    rc = lib.tbi_plan_small(code.n_labels, code.n_tensors, off.ctypes.data, lab.ctypes.data, len(code.iy),
                            iy.ctypes.data, code.n_nodes, ch.ctypes.data, len(sliced), sl.ctypes.data,
                            ctypes.byref(blob), ctypes.byref(nbytes), err, 512)
    if rc:
        raise ValueError(err.value.decode())
    raw = ctypes.string_at(blob, nbytes.value)
    lib.tbi_free(blob)
    ok, n_small, n_leaves, words, root_off, root_log2 = [int(x) for x in np.frombuffer(raw, np.int32, 6, 0)]
    p = 24
    nodes = []
    for _ in range(n_small):
        nodes.append(SmallNode.from_buffer_copy(raw[p:p + 32]))
        p += 32
    leaf_off = np.frombuffer(raw, np.int32, n_leaves, p).copy()
    p += 4 * n_leaves
    assert p == len(raw)
    return dict(ok=bool(ok), nodes=nodes, leaf_off=leaf_off, words=words, root_off=root_off, root_log2=root_log2)


def _small_stride(pw, i):
    q = (int(pw[i >> 3]) >> (4 * (i & 7))) & 15
    return (1 << q) & 0x7FFF


def run_small(sd, leaves, children, weights, slice_vals=(), r=0.0):
    """Replay k_small for one item: the leaf builder into shared memory, every
    node's thread loops (all outputs o, all reduced k) and the root max.  Every
    shared access must stay inside the item's words, every operand word must
    still hold the tensor the node reads (first-fit reuse never overwrote a
    live tensor), and no node may write over its own operands."""
    words = sd["words"]
    assert 0 < words <= 12288
    sm = np.full(words, np.nan, np.float64)
    owner = np.full(words, -1, np.int64)
    T = len(leaves)
    for i, ld in enumerate(leaves):
        w = float(weights[ld.label]) if ld.label >= 0 else float(ld.w)
        base = int(sd["leaf_off"][i])
        for e in range(1 << ld.n_out):
            best = -np.inf
            for raw in range(1 << ld.nraw):
                ok = True
                for k in range(ld.nraw):
                    x = (raw >> k) & 1
                    if ld.slice_idx[k] >= 0:
                        ok &= x == int(slice_vals[ld.slice_idx[k]])
                    else:
                        ok &= ((e >> ld.out_bit[k]) & 1) == x
                if ok:
                    best = max(best, (w if raw & 1 else 0.0) if ld.nraw == 1 else (-np.inf if raw == 3 else 0.0))
            assert 0 <= base + e < words
            sm[base + e] = best
            owner[base + e] = i
    for j, nd in enumerate(sd["nodes"]):
        a, b = int(children[j][0]), int(children[j][1])
        nc, nk = nd.nc_nk & 0xFF, (nd.nc_nk >> 8) & 0xFF
        assert nc + nk <= 16
        o = np.arange(1 << nc)
        k = np.arange(1 << nk)
        ao = sum(((o >> i) & 1) * _small_stride(nd.pa, i) for i in range(nc)) if nc else np.zeros(1, np.int64)
        bo = sum(((o >> i) & 1) * _small_stride(nd.pb, i) for i in range(nc)) if nc else np.zeros(1, np.int64)
        ak = sum(((k >> i) & 1) * _small_stride(nd.pa, nc + i) for i in range(nk)) if nk else np.zeros(1, np.int64)
        bk = sum(((k >> i) & 1) * _small_stride(nd.pb, nc + i) for i in range(nk)) if nk else np.zeros(1, np.int64)
        ia = nd.a_off + np.asarray(ao)[:, None] + np.asarray(ak)[None, :]
        ib = nd.b_off + np.asarray(bo)[:, None] + np.asarray(bk)[None, :]
        ic = nd.c_off + o
        for idx, want in ((ia, a), (ib, b)):
            assert idx.min() >= 0 and idx.max() < words, "operand read out of the item's shared words"
            assert np.all(owner[idx] == want), f"node {j} reads words not holding tensor {want}"
        assert ic.min() >= 0 and ic.max() < words, "output out of the item's shared words"
        assert not (set(ic.tolist()) & (set(ia.ravel().tolist()) | set(ib.ravel().tolist()))), \
            f"node {j} writes over its operands"
        sm[ic] = np.max(sm[ia] + sm[ib], axis=1)
        owner[ic] = T + j
    root_id = T + len(sd["nodes"]) - 1 if sd["nodes"] else 0
    ir = sd["root_off"] + np.arange(1 << sd["root_log2"])
    assert ir.min() >= 0 and ir.max() < words and np.all(owner[ir] == root_id)
    return float(np.max(sm[ir])) + r
