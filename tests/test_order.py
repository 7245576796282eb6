"""Leaf ordering: Morton keys in the reference's initial-cell numbering, the
stable LSD radix sort, the Karras radix tree and point location.

The reference has no counterpart (its leaves stay in allocation order), so the
keys are pinned through the one numbering it does define: the initial cells of
uniformSamplingKernel (kdgrid.cu:144-164).  The oracle's decoded cell boxes
must equal the initial-sampling boxes of the oracle grid, which the golden
fixtures pin against the reference's own kernels; the oracle's top-down tree
must equal a pure-Python restatement of Karras's per-node construction
(HPG 2012, Fig. 4).  The GPU tests then compare the CUDA path with the oracle
bit for bit, and check that none of these calls changes MDAS results.
"""
import numpy as np
import pytest

import pmdas_gb300 as P
from pmdas_gb300 import _native as N
from oracle import pyoracle as O


# ---------------------------------------------------------------------------------- CPU
def py_key(p, D, bpd, eib, F, sx, sy):
    """Key of one point, restated from the initial-cell bit layout (kdgrid.cu:147-157)."""
    K = bpd + F
    key = 0
    for j in range(D):
        u = np.float32(p[j])
        if j == 0:
            u = np.float32(u / np.float32(sx))
        elif j == 1:
            u = np.float32(u / np.float32(sy))
        B = K + (eib if j < 2 else 0)
        s = np.float32(u * np.float32(2.0 ** B))
        q = 0 if not s > 0 else (2 ** B - 1 if s >= 2 ** B else int(s))
        for k in range(K):
            key |= ((q >> k) & 1) << (D * k + (D - 1 - j))
        if j < 2:
            for k in range(K, K + eib):
                key |= ((q >> k) & 1) << (D * K + 2 * (k - K) + 1 - j)
    return key


def py_karras(keys):
    """Karras (HPG 2012) per internal node i: direction, range end, split."""
    n = len(keys)

    def delta(i, j):
        if j < 0 or j >= n:
            return -1
        a, b = int(keys[i]), int(keys[j])
        if a == b:
            x = i ^ j
            return 64 + (32 - x.bit_length())
        return 64 - (a ^ b).bit_length()

    children = np.zeros((max(n - 1, 0), 2), np.int32)
    for i in range(n - 1):
        d = 1 if delta(i, i + 1) - delta(i, i - 1) >= 0 else -1
        dmin = delta(i, i - d)
        lmax = 2
        while delta(i, i + lmax * d) > dmin:
            lmax *= 2
        l, t = 0, lmax // 2
        while t >= 1:
            if delta(i, i + (l + t) * d) > dmin:
                l += t
            t //= 2
        j = i + l * d
        dnode = delta(i, j)
        s, t = 0, l
        while True:
            t = (t + 1) // 2
            if delta(i, i + (s + t) * d) > dnode:
                s += t
            if t <= 1:
                break
        g = i + s * d + min(d, 0)
        children[i] = (~g if min(i, j) == g else g, ~(g + 1) if max(i, j) == g + 1 else g + 1)
    return children


def tree_checks(children, parents, n):
    """Every node reached once from the root; parents agree with children."""
    if n == 1:
        assert parents[0] == -1
        return
    seen = np.zeros(2 * n - 1, np.int64)
    stack = [0]
    assert parents[0] == -1
    while stack:
        v = stack.pop()
        seen[v] += 1
        for c in children[v]:
            idx = c if c >= 0 else (n - 1) + ~c
            assert parents[idx] == v
            if c >= 0:
                stack.append(c)
            else:
                seen[idx] += 1
    assert (seen == 1).all()


@pytest.mark.parametrize("D,bpd,eib,F", [(3, 1, 4, 6), (4, 1, 3, 5), (5, 0, 6, 4), (6, 1, 2, 7), (4, 1, 8, 11)])
def test_oracle_key_layout_and_roundtrip(D, bpd, eib, F):
    rng = np.random.default_rng(D * 100 + F)
    sx, sy = 96.0, 80.0
    pts = rng.random((500, D), dtype=np.float32)
    pts[:, 0] *= sx
    pts[:, 1] *= sy
    pts[:5] = 0.0
    pts[5:10, 0] = sx  # upper face: clamped into the last cell
    pts[10, :] = -1.0
    keys = O.morton_encode(pts, bpd, eib, F, sx, sy)
    for i in range(0, 500, 7):
        assert int(keys[i]) == py_key(pts[i], D, bpd, eib, F, sx, sy), i
    assert P.morton_key_bits(D, bpd, eib, F) == D * (bpd + F) + 2 * eib
    # every initial cell: the key of its centre, shifted, is the cell
    L = (1 << (bpd * D)) << (2 * eib)
    if L <= 1 << 16:
        cells = np.arange(L, dtype=np.uint64)
        boxes = O.morton_decode(cells, D, bpd, eib, sx, sy)
        cent = (np.float32(0.5) * (boxes[:, :D] + boxes[:, D:])).astype(np.float32)
        k = O.morton_encode(cent, bpd, eib, F, sx, sy)
        assert np.array_equal(k >> np.uint64(D * F), cells)
        # keys of the points lie in the cell whose decoded box holds them (interior points)
        inner = O.morton_decode(keys[20:] >> np.uint64(D * F), D, bpd, eib, sx, sy)
        p = pts[20:]
        assert ((inner[:, :D] <= p) & (p <= inner[:, D:])).all()


@pytest.mark.parametrize("D,bpd,eib", [(3, 1, 4), (4, 1, 3), (5, 1, 2), (4, 0, 6)])
def test_oracle_decode_equals_initial_sampling_boxes(D, bpd, eib):
    """The decoded cells are the reference's initial cells (the oracle grid's
    initial boxes are pinned to the reference's kernel by the golden fixtures)."""
    sx, sy = 120.0, 68.0
    L = (1 << (bpd * D)) << (2 * eib)
    o = O.OracleGrid(D, 4 * L + 64, 4, bpd, eib, 0.25, sx, sy)
    o.initial_sampling()
    st = o.dump_state()
    boxes = O.morton_decode(np.arange(L, dtype=np.uint64), D, bpd, eib, sx, sy)
    assert np.array_equal(boxes.view(np.uint32), st["boxes"].view(np.uint32))


@pytest.mark.parametrize("n", [0, 1, 2, 3, 17, 3071, 3072, 3073, 20000])
def test_oracle_sort_is_stable_numpy_order(n):
    rng = np.random.default_rng(n)
    k = rng.integers(0, 2 ** 63, size=n, dtype=np.uint64) | (rng.integers(0, 2, size=n, dtype=np.uint64) << np.uint64(63))
    if n > 10:
        k[::5] = k[1]
    for b, e in ((0, 64), (0, 20), (8, 40), (60, 64), (5, 5)):
        sk, order = O.sort_pairs(k, b, e)
        field = (k >> np.uint64(b)) & np.uint64((1 << (e - b)) - 1 if e - b < 64 else 2 ** 64 - 1)
        want = np.argsort(field, kind="stable")
        assert np.array_equal(order, want.astype(np.uint32)), (b, e)
        assert np.array_equal(sk, k[want])


@pytest.mark.parametrize("n,dup", [(1, 0), (2, 0), (2, 1), (9, 0), (64, 3), (1000, 0), (1000, 7), (777, 50)])
def test_oracle_tree_equals_karras(n, dup):
    rng = np.random.default_rng(n + dup)
    k = np.sort(rng.integers(0, 2 ** 64 - 1, size=n, dtype=np.uint64))
    if dup:
        k = np.sort(rng.choice(k[: max(1, n // dup)], size=n))  # many equal keys
    children, parents = O.karras(k)
    tree_checks(children, parents, n)
    if n > 1:
        assert np.array_equal(children, py_karras(k))


def test_oracle_refit_and_locate_on_a_grid():
    D, bpd, eib, sx, sy = 4, 1, 3, 64.0, 48.0
    o = O.OracleGrid(D, 40000, 4, bpd, eib, 0.25, sx, sy)
    o.initial_sampling()
    rng = np.random.default_rng(3)
    for _ in range(4):
        o.values[: o.N] = rng.random((o.N, 3), dtype=np.float32)
        o.sampling_pass()
    st = o.dump_state()
    F = 5
    keys = O.leaf_keys(st["boxes"], D, bpd, eib, F, sx, sy)
    sk, order = O.sort_pairs(keys)
    children, parents = O.karras(sk)
    n = sk.size
    tree_checks(children, parents, n)
    ib = O.refit(st["boxes"], order, children)
    assert np.array_equal(ib[0, :D], st["boxes"][:, :D].min(0)) and np.array_equal(ib[0, D:], st["boxes"][:, D:].max(0))
    # each sample lies in the (closed) box of the leaf it is located in
    pts = st["coords"][::3]
    loc = O.locate(st["boxes"], order, pts)
    assert (loc >= 0).all()
    b = st["boxes"][loc]
    assert ((b[:, :D] <= pts) & (pts <= b[:, D:])).all()
    # the leaf of a split child's sample: keys of leaves stay inside their initial cell
    cell = sk >> np.uint64(D * F)
    ini = O.morton_decode(cell, D, bpd, eib, sx, sy)
    lb = st["boxes"][order]
    assert ((ini[:, :D] <= lb[:, :D]) & (lb[:, D:] <= ini[:, D:])).all()


# ---------------------------------------------------------------------------------- GPU
def _grid(cuda, D=4, bpd=1, eib=4, W=96, H=80, passes=5, arith=P.ARITH_IEEE, kind=P.SCENE_DISCS_DOF, seed=5):
    sx, sy = float(W), float(H)
    L = (1 << (bpd * D)) << (2 * eib)
    g = P.KDGrid(D, 64 * L, 4, bpd, eib, 0.25, sx, sy, arith=arith)
    sc = P.Scene(kind if D == 4 else (P.SCENE_DISCS_MB if D == 3 else P.SCENE_DISCS_MBDOF), seed, 64, sx, sy, W, H)
    g.InitialSampling()
    sc.evaluate(g, 0, g.GetNumberOfSamples())
    for _ in range(passes):
        g.SamplingPass()
        n, nn = g.GetNumberOfSamples(), g.GetNewSamples()
        sc.evaluate(g, n - nn, nn)
    return g, sc, dict(D=D, bpd=bpd, eib=eib, sx=sx, sy=sy)


def _u64(t):
    return t.cpu().numpy().view(np.uint64)


def max_fine(D, bpd, eib):
    """fineBits = -1: the most that fit a 64-bit key and a 31-bit cell coordinate."""
    return min((64 - D * bpd - 2 * eib) // D, 31 - bpd - eib)


@pytest.mark.gpu
@pytest.mark.parametrize("D,bpd,eib,F", [(3, 1, 4, 6), (4, 1, 8, 11), (5, 1, 3, 8), (6, 0, 5, 9), (4, 2, 0, 14),
                                         (7, 1, 3, 7), (8, 0, 0, 8)])
def test_morton_encode_decode_match_oracle(cuda, D, bpd, eib, F):
    torch = cuda
    rng = np.random.default_rng(D + F)
    sx, sy = 1920.0, 1080.0
    pts = rng.random((100003, D), dtype=np.float32)
    pts[:, 0] *= sx
    pts[:, 1] *= sy
    pts[:7] = 0.0
    pts[7:13, 0] = sx
    pts[13:19, 1] = np.float32(sy) * np.float32(1.5)
    pts[19:25] = -3.0
    pts[25, 2] = np.nan
    pts[26, 0] = np.float32(1e-40)  # subnormal
    keys = P.morton_encode(torch.from_numpy(pts).cuda(), bpd, eib, F, sx, sy)
    assert np.array_equal(_u64(keys), O.morton_encode(pts, bpd, eib, F, sx, sy))
    cells = (O.morton_encode(pts, bpd, eib, F, sx, sy) >> np.uint64(D * F)).astype(np.uint64)
    boxes = P.morton_decode(torch.from_numpy(cells.view(np.int64)).cuda(), D, bpd, eib, sx, sy)
    assert np.array_equal(boxes.cpu().numpy().view(np.uint32), O.morton_decode(cells, D, bpd, eib, sx, sy).view(np.uint32))
    empty = P.morton_encode(torch.zeros((0, D), device="cuda"), bpd, eib, F, sx, sy)
    assert empty.numel() == 0


@pytest.mark.gpu
def test_morton_decode_equals_ieee_initial_boxes(cuda):
    torch = cuda
    g, _, p = _grid(cuda, D=5, bpd=1, eib=3, passes=0)
    st = g.dump_state()
    L = st["L"]
    boxes = P.morton_decode(torch.arange(L, dtype=torch.int64, device="cuda"), 5, 1, 3, p["sx"], p["sy"])
    assert np.array_equal(boxes.cpu().numpy().view(np.uint32), st["boxes"].view(np.uint32))


@pytest.mark.gpu
@pytest.mark.parametrize("n", [0, 1, 5, 3071, 3072, 3073, 100000, 2000003])
def test_radix_sort_matches_stable_numpy(cuda, n):
    torch = cuda
    rng = np.random.default_rng(n + 11)
    k = rng.integers(0, 2 ** 63, size=n, dtype=np.uint64) | (rng.integers(0, 2, size=n, dtype=np.uint64) << np.uint64(63))
    if n > 100:
        k[rng.integers(0, n, size=n // 3)] = k[0]  # heavy duplicates
        k[: n // 10] &= np.uint64(0xff)            # a block of small keys: skewed digits
    kt = torch.from_numpy(k.view(np.int64)).cuda()
    vals = rng.integers(0, 2 ** 32, size=n, dtype=np.uint64).astype(np.uint32)
    vt = torch.from_numpy(vals.view(np.int32)).cuda()
    for b, e in ((0, 64), (0, 20), (8, 40), (57, 64), (9, 9)):
        field = (k >> np.uint64(b)) & np.uint64(((1 << (e - b)) - 1) if e - b < 64 else 2 ** 64 - 1)
        want = np.argsort(field, kind="stable")
        ko, vo = P.radix_sort_pairs(kt, None, b, e)
        assert np.array_equal(_u64(ko), k[want]), (b, e)
        assert np.array_equal(vo.cpu().numpy().view(np.uint32), want.astype(np.uint32)), (b, e)
        ko, vo = P.radix_sort_pairs(kt, vt, b, e)
        assert np.array_equal(vo.cpu().numpy().view(np.uint32), vals[want]), (b, e)
    assert np.array_equal(_u64(kt), k)  # input untouched


@pytest.mark.gpu
@pytest.mark.parametrize("D,passes", [(3, 4), (4, 6), (5, 3), (6, 2)])
def test_leaf_order_and_hierarchy_match_oracle(cuda, D, passes):
    bpd, eib = 1, (4 if D < 5 else 2)
    g, _, p = _grid(cuda, D=D, bpd=bpd, eib=eib, passes=passes)
    st = g.dump_state()
    for F in (-1, 3):
        fine = F if F >= 0 else max_fine(D, bpd, eib)
        keys, order = g.LeafOrder(F)
        want_keys = O.leaf_keys(st["boxes"], D, bpd, eib, fine, p["sx"], p["sy"])
        sk, so = O.sort_pairs(want_keys)
        assert np.array_equal(_u64(keys), sk)
        assert np.array_equal(order.cpu().numpy().view(np.uint32), so)
    g.BuildHierarchy(-1)
    h = g.Hierarchy()
    fine = max_fine(D, bpd, eib)
    sk, so = O.sort_pairs(O.leaf_keys(st["boxes"], D, bpd, eib, fine, p["sx"], p["sy"]))
    ch, par = O.karras(sk)
    assert np.array_equal(h["keys"], sk) and np.array_equal(h["order"], so)
    assert np.array_equal(h["children"], ch) and np.array_equal(h["parents"], par)
    assert np.array_equal(h["boxes"].view(np.uint32), O.refit(st["boxes"], so, ch).view(np.uint32))
    # none of it changed the grid
    after = g.dump_state()
    for k in ("coords", "values", "nodes", "boxes", "errors", "seeds"):
        assert np.array_equal(after[k].view(np.uint8), st[k].view(np.uint8)), k


@pytest.mark.gpu
@pytest.mark.parametrize("n_random", [20000, 150000])  # the larger takes the queries in coarse key order
def test_locate_matches_oracle(cuda, n_random):
    torch = cuda
    g, _, p = _grid(cuda, D=4, bpd=1, eib=3, passes=6)
    st = g.dump_state()
    g.BuildHierarchy(-1)
    h = g.Hierarchy()
    rng = np.random.default_rng(9)
    D = 4
    pts = rng.random((n_random, D), dtype=np.float32)
    pts[:, 0] *= p["sx"]
    pts[:, 1] *= p["sy"]
    pts = np.concatenate([pts, st["coords"][::2],                         # samples (some on faces)
                          st["boxes"][::3, :D], st["boxes"][::5, D:],     # box corners
                          np.full((3, D), -1.0, np.float32), np.full((2, D), 2e3, np.float32)]).astype(np.float32)
    got = g.Locate(torch.from_numpy(pts).cuda()).cpu().numpy()
    want = O.locate(st["boxes"], h["order"], pts)
    assert np.array_equal(got, want)
    assert (got[:n_random] >= 0).all() and (got[-5:] == -1).all()


@pytest.mark.gpu
def test_hierarchy_is_invalidated_and_mdas_results_unchanged(cuda):
    torch = cuda
    a, sa, _ = _grid(cuda, passes=3, seed=7)
    b, sb, _ = _grid(cuda, passes=3, seed=7)
    a.BuildHierarchy(-1)
    a.Locate(torch.zeros((4, 4), device="cuda"))
    a.LeafOrder(2)
    a.BuildHierarchy(4)
    for g, sc in ((a, sa), (b, sb)):
        g.SamplingPass()
        n, nn = g.GetNumberOfSamples(), g.GetNewSamples()
        sc.evaluate(g, n - nn, nn)
    x, y = a.dump_state(), b.dump_state()
    for k in ("coords", "values", "nodes", "boxes", "errors", "seeds"):
        assert np.array_equal(x[k].view(np.uint8), y[k].view(np.uint8)), k
    with pytest.raises(N.MdasError) as e:
        a.Locate(torch.zeros((4, 4), device="cuda"))
    assert e.value.status == N.MDAS_ERR_STATE
    with pytest.raises(N.MdasError):
        a.Hierarchy()


@pytest.mark.gpu
@pytest.mark.slow
def test_full_size_order_properties(cuda):
    """dof1024-sized leaves (~6 M): sorted, a permutation, inside initial cells, tree valid."""
    torch = cuda
    from pmdas_gb300.workloads import WORKLOADS
    w = WORKLOADS["dof1024"]
    g = P.KDGrid(w.dim, w.maxSamples, w.candidatesNum, w.bitsPerDim, w.extraImgBits, w.alpha, w.scaleX, w.scaleY)
    sc = P.Scene(w.scene_kind, w.scene_seed, w.scene_count, w.scaleX, w.scaleY, w.width, w.height)
    P.render_graph(g, sc, w.budget, torch.zeros(w.height, w.width, 4, device="cuda"), w.width, w.height)
    D, bpd, eib = w.dim, w.bitsPerDim, w.extraImgBits
    fine = max_fine(D, bpd, eib)
    g.BuildHierarchy(-1)
    h = g.Hierarchy()
    L = g.GetNumberOfNodes()
    assert L > 4_000_000
    k = h["keys"]
    assert (k[1:] >= k[:-1]).all()
    assert np.array_equal(np.sort(h["order"]), np.arange(L, dtype=np.uint32))
    tree_checks(h["children"], h["parents"], L)
    boxes = g.dump_state()["boxes"]
    ini = O.morton_decode(k >> np.uint64(D * fine), D, bpd, eib, w.scaleX, w.scaleY)
    lb = boxes[h["order"]]
    assert ((ini[:, :D] <= lb[:, :D]) & (lb[:, D:] <= ini[:, D:])).all()
    assert np.array_equal(h["boxes"][0, :D], boxes[:, :D].min(0)) and np.array_equal(h["boxes"][0, D:], boxes[:, D:].max(0))
