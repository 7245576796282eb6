"""The integrand kernel (disc scenes: tile-culled candidate lists) against the
oracle's full scans over every primitive, bit for bit, through the C ABI."""
import numpy as np
import pytest

import pmdas_gb300 as P
from pmdas_gb300.kdgrid import SceneDesc
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

CULL_TILES = 64  # tiles per image axis of the disc culling

# (scene kind, dim, primitives)
KINDS = [(P.SCENE_DISCS_MB, 3, 64), (P.SCENE_DISCS_DOF, 4, 256), (P.SCENE_DISCS_MBDOF, 5, 256),
         (P.SCENE_DISCS_MBDOF, 6, 1024), (P.SCENE_DIRECT_LIGHT, 4, 4)]


def points(D, n, sx, sy, seed):
    """Uniform samples, plus image points on the culling tiles' edges and at the
    domain's ends, and time / lens coordinates at 0, 1/2 and just below 1."""
    rng = np.random.default_rng(seed)
    top = np.nextafter(np.float32(1), np.float32(0))
    pts = rng.random((n, D), dtype=np.float32)
    k = n // 4
    edges = np.minimum((np.arange(CULL_TILES + 1) / CULL_TILES).astype(np.float32), top)
    pts[:k, 0] = rng.choice(edges, k)
    pts[:k, 1] = rng.choice(edges, k)
    pts[k:2 * k, 2:] = rng.choice(np.float32([0.0, 0.5, top]), (k, D - 2))
    pts = np.minimum(pts, top)
    pts[:, 0] *= np.float32(sx)
    pts[:, 1] *= np.float32(sy)
    return pts


def gpu_evaluate(sc, pts):
    import torch
    c = torch.from_numpy(np.ascontiguousarray(pts)).cuda()
    v = torch.empty(len(pts), 3, dtype=torch.float32, device="cuda")
    sc.evaluate_buffers(c.data_ptr(), v.data_ptr(), pts.shape[1], 0, len(pts))
    torch.cuda.synchronize()
    return v.cpu().numpy()


@pytest.mark.parametrize("kind,D,count", KINDS)
def test_integrand_matches_full_scan(cuda, kind, D, count):
    W, H = 320, 200
    sx, sy = 0.5 * W, 0.5 * H
    sc = P.Scene(kind, 7, count, sx, sy, W, H)
    pts = points(D, 1 << 20, sx, sy, 1)
    got = gpu_evaluate(sc, pts)
    want = O.evaluate_points(sc.export(), pts)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    # the points hit many primitives, not only the background
    if kind != P.SCENE_DIRECT_LIGHT:
        assert len(np.unique(want, axis=0)) > min(count, 64) // 2
        assert np.all(want == np.float32(0.1), axis=1).mean() < 0.9


def test_culling_follows_new_host_primitives(cuda):
    """mdas_render_host with new primitives rebuilds the tile masks: the scene's
    integrand then matches the oracle on the new primitives."""
    kind, D, W, H = P.SCENE_DISCS_DOF, 4, 64, 64
    sc = P.Scene(kind, 3, 64, W, H, W, H)
    d = sc.export()
    prims = d.prims.copy()
    prims[:, 0] = -prims[:, 0]          # mirrored
    prims[:, 3] *= np.float32(1.5)      # larger discs
    prims[:, 7] = prims[:, 3] * prims[:, 3]
    bpd, eib = 1, 3
    n0 = 4 * ((1 << (bpd * D)) << (2 * eib))
    budget = 8 * W * H
    g = P.KDGrid(D, 2 * budget + n0, 4, bpd, eib, 0.25, W, H)
    pixels = np.zeros(W * H * 4, np.float32)
    P.render_host(g, sc, budget, pixels, W, H, host_prims=prims)
    pts = points(D, 1 << 18, W, H, 2)
    got = gpu_evaluate(sc, pts)
    want = O.evaluate_points(SceneDesc(d.kind, d.dim, d.count, d.desc_bytes, prims), pts)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    old = O.evaluate_points(d, pts)
    assert not np.array_equal(old, want)  # the new primitives change the integrand
    g.close()
    sc.close()
