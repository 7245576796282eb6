"""CPU checks of the C ABI (no GPU needed): the library loads, exports every
function include/mdas.h declares, validates arguments before touching CUDA,
and generates scenes deterministically on the host."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import pmdas_gb300 as P
from pmdas_gb300 import _native as N

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"^[A-Za-z_][\w \*]*?\b(mdas_\w+)\s*\(", text, flags=re.M))
    return sorted(names)


def test_exports_every_declared_symbol():
    lib = C.CDLL(N.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 30
    for name in names:
        assert hasattr(lib, name), name
    # and the Python binding covers all of them
    assert set(names) <= set(N.SIGNATURES)


def test_invalid_arguments_rejected_before_cuda():
    lib = N.load()
    h = C.c_void_p()
    bad = [
        (2, 1000, 4, 1, 2, 0.25, 1.0, 1.0),   # dim < 3
        (7, 1000, 4, 1, 2, 0.25, 1.0, 1.0),   # dim > 6
        (3, 0, 4, 1, 2, 0.25, 1.0, 1.0),      # maxSamples
        (3, 1 << 30, 4, 1, 2, 0.25, 1.0, 1.0),
        (3, 1000, 0, 1, 2, 0.25, 1.0, 1.0),   # candidatesNum
        (4, 1000, 4, 3, 9, 0.25, 1.0, 1.0),   # bitsPerDim*D + 2*extraImgBits > 28
        (3, 1000, 4, 1, 2, 0.25, 0.0, 1.0),   # scale
        (3, 1000, 4, -1, 2, 0.25, 1.0, 1.0),
    ]
    for a in bad:
        assert lib.mdas_create_ex(C.byref(h), *a, None, 0, None) == N.MDAS_ERR_INVALID, a
    assert lib.mdas_create_ex(C.byref(h), 3, 1000, 4, 1, 2, 0.25, 1.0, 1.0, None, 7, None) == N.MDAS_ERR_INVALID
    assert lib.mdas_destroy(None) == N.MDAS_ERR_INVALID
    assert lib.mdas_initial_sampling(None) == N.MDAS_ERR_INVALID
    assert lib.mdas_status_string(N.MDAS_ERR_CAPACITY) == b"sample or leaf capacity exceeded"


def test_create_without_gpu_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(N.MdasError) as e:
        P.KDGrid(3, 1000, 4, 1, 2, 0.25, 16, 16)
    assert e.value.status in (N.MDAS_ERR_CUDA, N.MDAS_ERR_ALLOC)


@pytest.mark.parametrize("kind,dim", [(P.SCENE_DISCS_MB, 3), (P.SCENE_DISCS_DOF, 4), (P.SCENE_DISCS_MBDOF, 5),
                                      (P.SCENE_DIRECT_LIGHT, 4)])
def test_scene_generation_is_seeded(kind, dim):
    a = P.Scene(kind, 5, 32, 64.0, 48.0, 64, 48).export()
    b = P.Scene(kind, 5, 32, 64.0, 48.0, 64, 48).export()
    c = P.Scene(kind, 6, 32, 64.0, 48.0, 64, 48).export()
    assert a.dim == dim and a.count == 32 and a.prims.shape == (32, N.PRIM_STRIDE)
    assert a.desc_bytes == b.desc_bytes and np.array_equal(a.prims, b.prims)
    assert not np.array_equal(a.prims, c.prims)
    if kind in (P.SCENE_DISCS_MB,):
        assert np.all((a.prims[:, 0] >= 0) & (a.prims[:, 0] < 1)) and np.all(a.prims[:, 3] >= 0.02)
        assert np.all(np.abs(a.prims[:, 4:6]) <= 0.1)
    if kind in (P.SCENE_DISCS_DOF, P.SCENE_DISCS_MBDOF):
        assert np.all((a.prims[:, 2] >= 1) & (a.prims[:, 2] < 10))
        assert np.all((a.prims[:, 3] >= 0.05) & (a.prims[:, 3] < 0.3))
    if kind == P.SCENE_DISCS_MBDOF:
        dof = P.Scene(P.SCENE_DISCS_DOF, 5, 32, 64.0, 48.0, 64, 48).export()
        # the 5-D scene is the 4-D scene with velocities added
        np.testing.assert_array_equal(a.prims[:, [0, 1, 2, 3, 6, 7, 8, 9, 10]],
                                      dof.prims[:, [0, 1, 2, 3, 6, 7, 8, 9, 10]])


def test_scene_rejects_bad_arguments():
    with pytest.raises(N.MdasError):
        P.Scene(9, 0, 4, 1.0, 1.0, 4, 4)
    with pytest.raises(N.MdasError):
        P.Scene(P.SCENE_DISCS_MB, 0, 2000, 1.0, 1.0, 4, 4)


def test_scene_values_match_float64_model():
    """The float32 integrand against an independent float64 evaluation (colours only differ
    where a sample sits within float32 rounding of a disc edge)."""
    from oracle import pyoracle as O
    W = H = 64
    sc = P.Scene(P.SCENE_DISCS_MB, 11, 64, W, H, W, H).export()
    g = O.OracleGrid(3, 8192, 4, 1, 3, 0.25, W, H)
    g.initial_sampling()
    g.evaluate(sc, 0, g.N)
    c = g.coords[:g.N].astype(np.float64)
    px, py, t = c[:, 0] / W, c[:, 1] / H, c[:, 2]
    want = np.full((g.N, 3), 0.1)
    for p in sc.prims.astype(np.float64):
        hit = (px - (p[0] + p[4] * t)) ** 2 + (py - (p[1] + p[5] * t)) ** 2 <= p[3] ** 2
        want[hit] = p[8:11]
    agree = np.all(np.abs(g.values[:g.N] - want) < 1e-6, axis=1)
    assert agree.mean() > 0.999
