"""Learned acceptance: the tcgen05 MLP against a PyTorch FP32 restatement with
the same BF16 rounding points, its gradients against autograd, the leaf
features against a numpy restatement, and the learned mode inside the MDAS
loop (fallback 1.0 must reproduce the plain sampler bit for bit)."""
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
    g[OFF_W2:OFF_B2] = (dz2.T @ h1).reshape(-1)
    dh1 = bf(dz2) @ bf(W2)
    dz1 = dh1 * (h1 > 0)
    g[OFF_B1:OFF_W2] = dz1.sum(0)
    g[OFF_W1:OFF_B1] = (dz1.T @ X).reshape(-1)
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


@pytest.mark.parametrize("m", [64, 128, 1000, 16384])
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


def _grid(torch, D=4, W=96, H=80, bpd=1, eib=4, seed=3, kind=P.SCENE_DISCS_DOF, arith=P.ARITH_REFERENCE):
    sx, sy = float(W), float(H)
    L = (1 << (bpd * D)) << (2 * eib)
    g = P.KDGrid(D, 64 * L, 4, bpd, eib, 0.25, sx, sy, arith=arith)
    sc = P.Scene(kind, seed, 64, sx, sy, W, H)
    return g, sc


def test_leaf_features_match_numpy(cuda):
    torch = cuda
    g, sc = _grid(torch)
    g.InitialSampling()
    sc.evaluate(g, 0, g.GetNumberOfSamples())
    for _ in range(3):
        g.SamplingPass()
        n, nn = g.GetNumberOfSamples(), g.GetNewSamples()
        sc.evaluate(g, n - nn, nn)
    st = g.dump_state()
    f = g.LeafFeatures().cpu().numpy()
    D = 4
    b = st["boxes"].astype(np.float64)
    ext = b[:, D:] - b[:, :D]
    ext[:, 0] /= g.GetScaleX()
    ext[:, 1] /= g.GetScaleY()
    l2 = np.log2(np.maximum(ext, 1e-30))
    want = np.zeros((st["L"], 16))
    want[:, :D] = l2 / 16
    want[:, 6] = l2.sum(1) / (16 * D)
    nodes = st["nodes"]
    valid = nodes >= 0
    v = st["values"].astype(np.float64)[np.where(valid, nodes, 0)] * valid[..., None]
    n = valid.sum(1)
    mean = v.sum(1) / n[:, None]
    dev = (np.abs(v - mean[:, None, :]) * valid[..., None]).sum(1) / n[:, None]
    want[:, 7] = n / 4
    want[:, 8:11] = np.log2(1 + np.abs(mean))
    want[:, 11:14] = np.log2(1 + dev)
    assert np.abs(f - want).max() < 1e-4


def test_predictions_equal_forward_of_features(cuda):
    torch = cuda
    g, sc = _grid(torch)
    g.LearnedEnable(trainSteps=2, batch=4096)
    g.InitialSampling()
    sc.evaluate(g, 0, g.GetNumberOfSamples())
    g.ComputeErrors()
    loss = g.LearnedUpdate()
    assert np.isfinite(loss) and loss > 0
    pred = g.LearnedPredictions()
    p = torch.from_numpy(g.LearnedParams()).cuda()
    again = P.mlp_forward(p, g.LeafFeatures())
    assert torch.equal(pred, again)


def test_learned_mode_trains_and_renders(cuda):
    torch = cuda
    W, H_ = 128, 96
    g, sc = _grid(torch, W=W, H=H_, seed=11)
    g.LearnedEnable(trainSteps=8, batch=8192, learningRate=3e-3)
    g.InitialSampling()
    sc.evaluate(g, 0, g.GetNumberOfSamples())
    losses = []
    budget = 12 * W * H_
    while g.GetNumberOfSamples() < budget:
        g.ComputeErrors()
        losses.append(g.LearnedUpdate())
        g.AdaptiveSampling()
        n, nn = g.GetNumberOfSamples(), g.GetNewSamples()
        sc.evaluate(g, n - nn, nn)
    assert len(losses) >= 4
    assert min(losses[-3:]) < losses[0]  # the model learns the error
    assert g.Validate()
    px = torch.zeros(H_, W, 4, device="cuda")
    g.Integrate(px, W, H_)
    ref = sc.reference_image(W, H_, spp=1024)
    img = px[..., :3].double()
    rel = float(torch.nan_to_num((ref - img) ** 2 / (ref ** 2 + 1e-2)).mean())
    assert rel < 0.05, rel
    with pytest.raises(N.MdasError) as e:
        P.render_graph(g, sc, budget, px, W, H_)
    assert e.value.status == N.MDAS_ERR_STATE


@pytest.mark.parametrize("arith", [P.ARITH_REFERENCE, P.ARITH_IEEE])
def test_full_fallback_is_the_plain_sampler(cuda, arith):
    torch = cuda
    a, sa = _grid(torch, seed=5, arith=arith)
    b, sb = _grid(torch, seed=5, arith=arith)
    a.LearnedEnable(trainSteps=1, batch=2048, fallback=1.0)
    for g, sc in ((a, sa), (b, sb)):
        g.InitialSampling()
        sc.evaluate(g, 0, g.GetNumberOfSamples())
        for _ in range(4):
            g.SamplingPass()
            n, nn = g.GetNumberOfSamples(), g.GetNewSamples()
            sc.evaluate(g, n - nn, nn)
    x, y = a.dump_state(), b.dump_state()
    for k in ("coords", "values", "nodes", "boxes", "errors", "seeds"):
        assert np.array_equal(x[k].view(np.uint8), y[k].view(np.uint8)), k
    a.LearnedEnable(False)
