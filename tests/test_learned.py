"""Learned acceptance: the tcgen05 MLP against a PyTorch FP32 restatement with
the same BF16 rounding points, its gradients against autograd, Adam against
its formula, the leaf features and true-error targets against numpy / the
oracle's integrand, and the learned mode inside the MDAS loop (the judge's
sums against a numpy restatement, the graph path against the host loop)."""
import numpy as np
import pytest

import pmdas_gb300 as P
from pmdas_gb300 import _native as N

pytestmark = pytest.mark.gpu

H, IN = 64, 16
OFF_W1, OFF_B1 = 0, H * IN
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H


def unpack(p):
    return (p[OFF_W1:OFF_B1].view(H, IN), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].view(H, H), p[OFF_B2:OFF_W3],
            p[OFF_W3:OFF_B3], p[OFF_B3])


def ref_forward(p, x):
    """The kernel's arithmetic: BF16 operands, FP32 accumulation, BF16 hidden layer 1."""
    import torch
    bf = lambda t: t.bfloat16().float()
    W1, b1, W2, b2, w3, b3 = unpack(p)
    X = bf(x)
    h1 = bf(torch.relu(X @ bf(W1).T + b1))
    z2 = h1 @ bf(W2).T + b2
    h2 = torch.relu(z2)
    return X, h1, z2, h2, h2 @ w3 + b3


def ref_gradients(p, x, y):
    import torch
    bf = lambda t: t.bfloat16().float()
    W1, b1, W2, b2, w3, b3 = unpack(p)
    X, h1, z2, h2, pred = ref_forward(p, x)
    m = x.shape[0]
    e = pred - y
    dpred = 2.0 * e / m
    g = torch.zeros_like(p)
    g[OFF_W3:OFF_B3] = h2.T @ dpred
    g[OFF_B3] = dpred.sum()
    dz2 = dpred[:, None] * w3[None, :] * (z2 > 0)
    g[OFF_B2:OFF_W3] = dz2.sum(0)
    g[OFF_W2:OFF_B2] = (bf(dz2).T @ h1).reshape(-1)  # the weight gradients: a BF16 tensor-core GEMM
    dh1 = bf(dz2) @ bf(W2)
    dz1 = dh1 * (h1 > 0)
    g[OFF_B1:OFF_W2] = dz1.sum(0)
    g[OFF_W1:OFF_B1] = (bf(dz1).T @ X).reshape(-1)
    return g, float((e * e).mean())


def make_params(torch, seed):
    gen = torch.Generator().manual_seed(seed)
    p = torch.empty(N.MLP_PARAMS)
    for off, n, fan in ((OFF_W1, H * IN, IN), (OFF_B1, H, IN), (OFF_W2, H * H, H), (OFF_B2, H, H), (OFF_W3, H, H),
                        (OFF_B3, 1, H)):
        p[off:off + n] = (torch.rand(n, generator=gen) * 2 - 1) / fan ** 0.5
    return p.cuda()


@pytest.mark.parametrize("m", [1, 127, 128, 129, 1000, 100003])
def test_mlp_forward_matches_torch(cuda, m):
    torch = cuda
    p = make_params(torch, m)
    x = (torch.randn(m, IN, generator=torch.Generator().manual_seed(m + 1)) * 1.5).cuda()
    got = P.mlp_forward(p, x)
    want = ref_forward(p, x)[-1]
    scale = want.abs().max().item() + 1e-6
    err = (got - want).abs().max().item() / scale
    assert err < 2e-3, err  # FP32 accumulation order, rare BF16 rounding flips of layer-1 outputs
    # and the median row is much closer than that
    assert (got - want).abs().median().item() / scale < 1e-5


@pytest.mark.parametrize("m", [64, 128, 1000, 16384, 100003])  # (the last: several tiles per persistent CTA)
def test_mlp_gradients_match_torch(cuda, m):
    torch = cuda
    p = make_params(torch, 7 + m)
    gen = torch.Generator().manual_seed(m)
    x = torch.randn(m, IN, generator=gen).cuda()
    y = torch.randn(m, generator=gen).cuda() * 0.3
    g, loss = P.mlp_gradients(p, x, y)
    gw, lw = ref_gradients(p, x, y)
    assert abs(loss - lw) <= 1e-3 * max(abs(lw), 1e-6)
    for name, a, b in (("W1", OFF_W1, OFF_B1), ("b1", OFF_B1, OFF_W2), ("W2", OFF_W2, OFF_B2), ("b2", OFF_B2, OFF_W3),
                       ("w3", OFF_W3, OFF_B3), ("b3", OFF_B3, OFF_B3 + 1)):
        s = gw[a:b].abs().max().item() + 1e-9
        assert (g[a:b] - gw[a:b]).abs().max().item() / s < 5e-3, name
    # the same numbers are the gradient of the loss: autograd through an FP32 copy (no BF16 rounding)
    q = p.clone().requires_grad_(True)
    W1, b1, W2, b2, w3, b3 = unpack(q)
    pred = torch.relu(torch.relu(x @ W1.T + b1) @ W2.T + b2) @ w3 + b3
    ((pred - y) ** 2).mean().backward()
    cos = torch.nn.functional.cosine_similarity(g, q.grad, dim=0).item()
    assert cos > 0.99, cos


def _grid(torch, D=4, W=96, H=80, bpd=1, eib=4, seed=3, kind=P.SCENE_DISCS_DOF, arith=P.ARITH_REFERENCE, ms=None):
    sx, sy = float(W), float(H)
    L = (1 << (bpd * D)) << (2 * eib)
    g = P.KDGrid(D, ms or 64 * L, 4, bpd, eib, 0.25, sx, sy, arith=arith)
    sc = P.Scene(kind, seed, 64, sx, sy, W, H)
    return g, sc


def _passes(g, sc, n, learned=False):
    g.InitialSampling()
    sc.evaluate(g, 0, g.GetNumberOfSamples())
    for _ in range(n):
        g.SamplingPass()
        a, b = g.GetNumberOfSamples(), g.GetNewSamples()
        sc.evaluate(g, a - b, b)


def test_adam_matches_formula(cuda):
    torch = cuda
    gen = torch.Generator().manual_seed(5)
    p = torch.randn(N.MLP_PARAMS, generator=gen).cuda()
    m1 = torch.randn(N.MLP_PARAMS, generator=gen).cuda() * 0.1
    m2 = torch.rand(N.MLP_PARAMS, generator=gen).cuda() * 0.01
    g = torch.randn(N.MLP_PARAMS, generator=gen).cuda()
    want_p, want_m1, want_m2 = p.clone(), m1.clone(), m2.clone()
    step, lr = 3, 1e-3
    a = 0.9 * want_m1 + 0.1 * g
    b = 0.999 * want_m2 + 0.001 * g * g
    want_p -= lr * (a / (1 - 0.9 ** step)) / (torch.sqrt(b / (1 - 0.999 ** step)) + 1e-8)
    P.mlp_adam(p, m1, m2, g, step, lr)
    # FP32 constants (1 - 0.999f is 1.00004e-3) against the formula's decimals
    assert torch.allclose(m1, a, rtol=1e-5, atol=1e-7) and torch.allclose(m2, b, rtol=1e-4, atol=1e-9)
    assert torch.allclose(p, want_p, rtol=1e-5, atol=1e-6)
    assert (g == 0).all()


def test_leaf_features_match_numpy(cuda):
    torch = cuda
    g, sc = _grid(torch)
    _passes(g, sc, 3)
    st = g.dump_state()
    f = g.LeafFeatures().cpu().numpy()
    D, bpd, eib = 4, 1, 4
    b = st["boxes"].astype(np.float64)
    ext = b[:, D:] - b[:, :D]
    ext[:, 0] /= g.GetScaleX()
    ext[:, 1] /= g.GetScaleY()
    l2 = np.log2(np.maximum(ext, 1e-30))
    L = st["L"]
    want = np.zeros((L, 16))
    want[:, :D] = l2 / 16
    nodes = st["nodes"]
    valid = nodes >= 0
    v = st["values"].astype(np.float64)[np.where(valid, nodes, 0)]
    lum = 0.2126 * v[..., 0] + 0.7152 * v[..., 1] + 0.0722 * v[..., 2]
    n = valid.sum(1)
    mean = np.where(valid, lum, 0).sum(1) / n
    var = np.maximum(np.where(valid, lum * lum, 0).sum(1) / n - mean ** 2, 0)
    want[:, 5] = n / 4
    want[:, 6] = np.log2(1 + np.abs(mean))
    want[:, 7] = np.log2(1 + np.sqrt(var))
    want[:, 8] = np.log2(1 + np.abs(np.where(valid, lum, np.inf).min(1)))
    want[:, 9] = np.log2(1 + np.abs(np.where(valid, lum, -np.inf).max(1)))
    le = np.log2(np.maximum(st["errors"].astype(np.float64), 1e-30)) / 32
    want[:, 10] = le
    want[:, 11] = (-(bpd * D + 2 * eib) - l2.sum(1)) / 32
    for q, o in enumerate((-2, -1, 1, 2)):
        j = np.arange(L) + o
        want[:, 12 + q] = np.where((j >= 0) & (j < L), le[np.clip(j, 0, L - 1)], le)
    err = np.abs(f - want)
    err[:, 7] = np.maximum(err[:, 7] - 2e-3, 0)  # the device variance is E[x^2] - mean^2 in FP32
    assert err.max() < 1e-4, np.unravel_index(err.argmax(), err.shape)


def test_predictions_equal_forward_of_features(cuda):
    torch = cuda
    g, sc = _grid(torch)
    g.LearnedEnable(seed=7)
    _passes(g, sc, 2)
    g.ComputeErrors()
    g.LearnedPredict()
    pred = g.LearnedPredictions()
    p = torch.from_numpy(g.LearnedParams()).cuda()
    feats = g.LeafFeatures()
    again = feats[:, 10] + P.mlp_forward(p, feats)  # priority = log2(plain error) / 32 + correction
    assert torch.equal(pred, again)


def test_incremental_predictions_from_error_rows(cuda):
    """After a learned pass the update refreshes only the split children, from
    the raw feature rows the split-children errors pass wrote; their priorities
    equal the forward pass of those leaves' gathered features, bit for bit."""
    torch = cuda
    g, sc = _grid(torch)
    g.LearnedEnable(seed=7)
    _passes(g, sc, 2)
    g.ComputeErrors()
    g.LearnedUpdate()                  # every leaf
    before = g.dump_state()
    g.AdaptiveSampling()               # learned acceptance
    a, b = g.GetNumberOfSamples(), g.GetNewSamples()
    sc.evaluate(g, a - b, b)
    g.ComputeErrors()                  # the split children only, with their raw rows
    g.LearnedUpdate()                  # those rows' priorities
    after = g.dump_state()
    L0, L1 = before["L"], after["L"]
    assert L1 > L0
    changed = np.zeros(L1, bool)
    changed[L0:] = True                # right children
    changed[:L0] = np.any(after["boxes"][:L0] != before["boxes"], axis=1)  # left children keep the slot
    assert changed[:L0].sum() == L1 - L0
    pred = g.LearnedPredictions()
    p = torch.from_numpy(g.LearnedParams()).cuda()
    feats = g.LeafFeatures()
    again = feats[:, 10] + P.mlp_forward(p, feats)
    idx = torch.from_numpy(np.nonzero(changed)[0]).cuda()
    assert torch.equal(pred[idx], again[idx])


@pytest.mark.parametrize("tolerance", [0.05, 1.0e6])
def test_pred_max_is_the_max_over_every_leaf(cuda, tolerance):
    """The largest priority of an incremental update (the kept leaves' maximum
    from the adaptive pass, the split children's from their predictions) equals
    the maximum over all current predictions, pass after pass, whichever
    acceptance the judge picked."""
    torch = cuda
    g, sc = _grid(torch, seed=17)
    g.LearnedEnable(seed=5, tolerance=tolerance)
    g.InitialSampling()
    sc.evaluate(g, 0, g.GetNumberOfSamples())
    for k in range(8):
        g.ComputeErrors()
        g.LearnedUpdate()              # every leaf first, then the split children only
        pred = g.LearnedPredictions()
        assert g.LearnedPredMax() == float(pred.max()), k
        g.AdaptiveSampling()
        a, b = g.GetNumberOfSamples(), g.GetNewSamples()
        sc.evaluate(g, a - b, b)
    assert g.LearnedStats()["judged"] == 8


def test_true_errors_match_oracle_integrand(cuda):
    torch = cuda
    from oracle import pyoracle as O
    g, sc = _grid(torch, W=48, H=40, eib=3)
    _passes(g, sc, 2)
    st = g.dump_state()
    K, seed = 16, 77
    got = g.LeafTrueErrors(sc, samples=K, seed=seed).cpu().numpy()
    D = 4
    L = st["L"]
    # the same per-leaf 64-bit LCG stream (24 random bits per float) and the oracle's integrand
    mask = (1 << 64) - 1
    pts = np.zeros((L, K, D), np.float32)
    b = st["boxes"]
    for i in range(L):
        s = (seed ^ ((0x9E3779B97F4A7C15 * (i + 1)) & mask)) & mask
        for k in range(K):
            for d in range(D):
                s = (s * 6364136223846793005 + 1442695040888963407) & mask
                r = np.float32((s >> 40) & 0xFFFFFF) * np.float32(1.0 / 16777216.0)
                pts[i, k, d] = np.float32(b[i, d] + np.float32(r * np.float32(b[i, D + d] - b[i, d])))
    vals = O.evaluate_points(sc.export(), pts.reshape(-1, D))
    ref = vals.reshape(L, K, 3).astype(np.float64).mean(1)
    nodes = st["nodes"]
    valid = nodes >= 0
    v = st["values"][np.where(valid, nodes, 0)]
    m = np.zeros((L, 3), np.float32)  # FP32, slot order, as the kernel sums
    for k in range(4):
        m = np.where(valid[:, k, None], (m + v[:, k]).astype(np.float32), m)
    mean = (m / valid.sum(1)[:, None].astype(np.float32)).astype(np.float32).astype(np.float64)
    vol = np.prod((b[:, D:] - b[:, :D]).astype(np.float64), axis=1)
    want = vol * (np.abs(mean - ref) / np.sqrt(ref ** 2 + 1e-2)).sum(1)
    assert np.allclose(got, want, rtol=1e-4, atol=1e-12)


def test_constant_correction_is_the_plain_ranking(cuda):
    """A network that outputs a constant leaves the plain ranking: the learned
    ratio is error / max error up to rounding, so the pass accepts the same
    leaves but for a few at the threshold, and the judge keeps it."""
    torch = cuda
    a, sa = _grid(torch)
    b, sb = _grid(torch)
    p = np.zeros(N.MLP_PARAMS, np.float32)
    p[OFF_B3] = 0.1
    a.LearnedEnable(params=p)
    for g, sc in ((a, sa), (b, sb)):
        g.InitialSampling()
        sc.evaluate(g, 0, g.GetNumberOfSamples())
        g.SamplingPass()
    L = a.GetNumberOfNodes() - a.GetNewNodes()
    assert abs(a.GetNewSamples() - b.GetNewSamples()) <= max(2, L // 200)
    s = a.LearnedStats()
    assert s["judged"] == 1 and s["last_plain"] == 0
    assert abs(s["unrefined_learned"] - s["unrefined_plain"]) <= 0.01 * s["unrefined_plain"]


def test_judge_matches_numpy(cuda):
    torch = cuda
    from oracle import pyoracle as O
    from tests.test_oracle import tea4
    g, sc = _grid(torch, arith=P.ARITH_IEEE)
    g.LearnedEnable(seed=3, tolerance=0.05)
    _passes(g, sc, 2)
    g.ComputeErrors()
    g.LearnedUpdate()
    st = g.dump_state()
    pred = g.LearnedPredictions().cpu().numpy().astype(np.float32)
    stats = g.LearnedStats()
    gerr = np.float32(g.GetGError())
    alpha = np.float32(0.25)
    pmax = pred.max()
    ul = up = 0.0
    for i in range(st["L"]):
        seed = int(st["seeds"][i]) or tea4(i, 0)
        seed = (1664525 * seed + 1013904223) & 0xFFFFFFFF
        r = np.float32(seed & 0xFFFFFF) / np.float32(16777216.0)
        e = np.float32(st["errors"][i])
        if not O.powf(np.float32(e / gerr), alpha) >= r:
            up += float(e)
        ratio = np.exp2(np.float32((pred[i] - pmax) * np.float32(32.0)))
        if not O.powf(np.float32(ratio), alpha) >= r:
            ul += float(e)
    assert abs(stats["unrefined_plain"] - up) <= 1e-6 * max(up, 1e-30)
    assert abs(stats["unrefined_learned"] - ul) <= 1e-3 * max(ul, 1e-30)  # exp2f may differ by an ulp
    if abs(ul / up - 1.05) > 1e-2:
        assert stats["last_plain"] == (1 if ul > 1.05 * up else 0)
    assert stats["judged"] == 3  # two sampling passes and this update


@pytest.mark.parametrize("arith", [P.ARITH_REFERENCE, P.ARITH_IEEE])
def test_learned_graph_render_equals_host_loop(cuda, arith):
    torch = cuda
    W, H_ = 96, 80
    a, sa = _grid(torch, W=W, H=H_, seed=11, arith=arith)
    b, sb = _grid(torch, W=W, H=H_, seed=11, arith=arith)
    for g in (a, b):
        g.LearnedEnable(seed=9)
    budget = 12 * W * H_
    pa = torch.zeros(H_, W, 4, device="cuda")
    pb = torch.zeros(H_, W, 4, device="cuda")
    P.render(a, sa, budget, pa, W, H_)
    P.render_graph(b, sb, budget, pb, W, H_)
    x, y = a.dump_state(), b.dump_state()
    for k in ("coords", "values", "nodes", "boxes", "errors", "seeds"):
        assert np.array_equal(x[k].view(np.uint8), y[k].view(np.uint8)), k
    assert a.Validate() and b.Validate()
    assert a.LearnedStats()["judged"] == b.LearnedStats()["judged"] > 0


@pytest.mark.parametrize("arith", [P.ARITH_REFERENCE, P.ARITH_IEEE])
def test_learned_batch_equals_single_renders(cuda, arith):
    """Learned and plain images of different dimension in one batch: every image
    ends exactly as its own device-side render (learned ones with their own
    predictions and judge), over two renders of the batch."""
    torch = cuda
    from tests.parity import assert_states_equal, rel_close
    specs = [  # (kind, D, W, H, spp, learned weights seed or None)
        (P.SCENE_DISCS_MB, 3, 64, 48, 8, 5),
        (P.SCENE_DISCS_DOF, 4, 96, 64, 16, 6),
        (P.SCENE_DISCS_MBDOF, 5, 48, 40, 12, 7),
        (P.SCENE_DISCS_DOF, 4, 80, 56, 8, None),
    ]
    grids, scenes, pix, budgets, singles = [], [], [], [], []
    for kind, D, W, H_, spp, wseed in specs:
        budget = spp * W * H_
        eib = 3 if D < 5 else 2
        ms = 2 * budget + 8 * ((1 << D) << (2 * eib))
        sc = P.Scene(kind, 20 + D, 32, W, H_, W, H_)
        made = []
        for _ in range(2):
            g = P.KDGrid(D, ms, 4, 1, eib, 0.25, W, H_, arith=arith)
            if wseed is not None:
                g.LearnedEnable(seed=wseed)
            made.append(g)
        rpx = torch.zeros(H_, W, 4, device="cuda")
        st = P.render_graph(made[0], sc, budget, rpx, W, H_)
        singles.append((made[0].dump_state(), rpx.cpu().numpy(), st.passes,
                        made[0].LearnedStats()["judged"] if wseed is not None else 0))
        grids.append(made[1])
        scenes.append(sc)
        pix.append(torch.zeros(H_, W, 4, device="cuda"))
        budgets.append(budget)
    batch = P.Batch(grids, scenes, budgets, pix, [sp[2] for sp in specs], [sp[3] for sp in specs])
    for rnd in range(3):
        # the last round with the pass loop on the host
        stats = batch.render_stepped() if rnd == 2 else batch.render()
        for i, (want, img, passes, judged) in enumerate(singles):
            assert stats[i].passes == passes, (rnd, i)
            assert_states_equal(grids[i].dump_state(), want,
                                keys=("coords", "values", "nodes", "boxes", "errors", "seeds"), what=f"image {i}")
            ok, worst = rel_close(pix[i].cpu().numpy(), img)
            assert ok, (i, worst)
            if specs[i][5] is not None:
                assert grids[i].LearnedStats()["judged"] == (rnd + 1) * judged
    batch.close()
