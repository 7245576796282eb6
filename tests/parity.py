"""Shared helpers of the parity tests."""
import numpy as np

STATE_KEYS = ("coords", "values", "nodes", "boxes", "errors", "seeds")


def assert_states_equal(a, b, keys=("coords", "nodes", "boxes", "errors", "seeds"), what=""):
    assert (a["N"], a["L"]) == (b["N"], b["L"]), (what, a["N"], a["L"], b["N"], b["L"])
    for k in keys:
        x, y = a[k], b[k]
        if not np.array_equal(x.view(np.uint32) if x.dtype == np.float32 else x,
                              y.view(np.uint32) if y.dtype == np.float32 else y):
            bad = np.argwhere((x != y).reshape(len(x), -1).any(axis=1)).ravel()
            raise AssertionError(f"{what}: {k} differs at {len(bad)} rows, first {bad[:5]}: {x[bad[:3]]} vs {y[bad[:3]]}")


def _canonical_nodes(st, N0, D):
    """Sample indices < N0 kept; new sample indices replaced by the rank of their
    coordinates among the new samples (lexicographic), so that the order in which
    slots were handed out does not matter."""
    n = st["N"]
    newc = st["coords"][N0:n]
    order = np.lexsort(newc.T[::-1]) if len(newc) else np.zeros(0, np.int64)
    rank = np.empty(len(newc), np.int64)
    rank[order] = np.arange(len(newc))
    nodes = st["nodes"].astype(np.int64)
    out = nodes.copy()
    is_new = nodes >= N0
    out[is_new] = N0 + rank[nodes[is_new] - N0]
    out[nodes < 0] = -1 - D
    return out, newc[order]


def assert_pass_equivalent(s0, a, b, D, what=""):
    """One adaptive pass from the same state `s0` gave the same result in `a` and
    `b`, up to the order in which new sample and leaf slots were handed out."""
    assert (a["N"], a["L"]) == (b["N"], b["L"]), (what, a["N"], a["L"], b["N"], b["L"])
    N0, L0 = s0["N"], s0["L"]
    for k in ("seeds", "errors", "boxes"):
        assert np.array_equal(a[k][:L0], b[k][:L0]), (what, k)
    na, ca = _canonical_nodes(a, N0, D)
    nb, cb = _canonical_nodes(b, N0, D)
    assert np.array_equal(ca.view(np.uint32), cb.view(np.uint32)), (what, "new sample coordinates")
    assert np.array_equal(na[:L0], nb[:L0]), (what, "nodes of existing slots")

    def right(st, nodes):
        boxes = st["boxes"][L0:]
        order = np.lexsort(boxes.T[::-1]) if len(boxes) else np.zeros(0, np.int64)
        return boxes[order], nodes[L0:][order], st["errors"][L0:][order], st["seeds"][L0:][order]

    ra, rb = right(a, na), right(b, nb)
    for x, y, k in zip(ra, rb, ("boxes", "nodes", "errors", "seeds")):
        assert np.array_equal(x, y), (what, "right children", k)
    assert np.all(a["errors"][L0:] == -1) and np.all(a["seeds"][L0:] == 0)


def rel_close(img, ref, rtol=1e-5, atol=1e-6):
    """max |img - ref| <= rtol * |ref| + atol, elementwise."""
    err = np.abs(img.astype(np.float64) - ref.astype(np.float64))
    lim = rtol * np.abs(ref.astype(np.float64)) + atol
    return bool(np.all(err <= lim)), float(np.max(err / (np.abs(ref) + atol)))


def rel_mse(img, ref):
    """relMSE of SDK/data/Scripts/parse_logs.py:48-50: mean((ref-img)^2 / (ref^2 + 1e-2)), NaN -> 0."""
    img = img.astype(np.float64)
    ref = ref.astype(np.float64)
    v = (ref - img) ** 2 / (ref ** 2 + 1e-2)
    v[np.isnan(v)] = 0.0
    return float(v.mean())
