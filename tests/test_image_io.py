"""Headless image files (mdas_save_image), standing in for the sample apps'
sutil::saveImage calls (optixMotionBlur.cpp:795-840): float4 film and
sampling-density images as PFM in place of OpenEXR, the 8-bit image as PPM."""
import numpy as np
import pytest

import pmdas_gb300 as P
from pmdas_gb300 import _native as N


def test_float_image_roundtrip_bit_exact(tmp_path):
    rng = np.random.default_rng(5)
    img = rng.standard_normal((7, 13, 4)).astype(np.float32)
    img[0, 0, :3] = [0.0, -0.0, np.float32(1e-40)]  # zeros and a subnormal survive
    p = str(tmp_path / "film.pfm")
    P.save_image(p, img)
    with open(p, "rb") as f:
        assert f.read(len(b"PF\n13 7\n-1.0\n")) == b"PF\n13 7\n-1.0\n"  # little-endian PFM header
    back = P.read_image(p)
    assert back.shape == (7, 13, 3)
    assert np.array_equal(back.view(np.uint32), img[..., :3].view(np.uint32))


def test_byte_image_roundtrip(tmp_path):
    rng = np.random.default_rng(6)
    img = rng.integers(0, 256, size=(5, 9, 4), dtype=np.uint8)
    p = str(tmp_path / "film.ppm")
    P.save_image(p, img)
    with open(p, "rb") as f:
        assert f.read(len(b"P6\n9 5\n255\n")) == b"P6\n9 5\n255\n"
    assert np.array_equal(P.read_image(p), img[..., :3])


def test_save_image_errors(tmp_path):
    lib = N.load()
    px = np.zeros((2, 2, 4), np.float32)
    assert lib.mdas_save_image(str(tmp_path / "x.pfm").encode(), px.ctypes.data, 2, 2, 7) == N.MDAS_ERR_INVALID
    assert lib.mdas_save_image(str(tmp_path / "x.pfm").encode(), px.ctypes.data, 0, 2, 0) == N.MDAS_ERR_INVALID
    assert lib.mdas_save_image(str(tmp_path / "no" / "dir.pfm").encode(), px.ctypes.data, 2, 2, 0) == N.MDAS_ERR_INVALID
    with pytest.raises(ValueError):
        P.save_image(str(tmp_path / "x.pfm"), np.zeros((2, 2, 3), np.float32))


@pytest.mark.gpu
def test_render_outputs_to_files(cuda, tmp_path):
    """The apps' outputs of one render: the film, its 8-bit conversion and the
    sampling density, each written and read back unchanged."""
    import torch
    W, H = 96, 64
    g = P.KDGrid(4, 200000, 4, 1, 4, 0.25, W, H)
    sc = P.Scene(P.SCENE_DISCS_DOF, 2, 64, W, H, W, H)
    film = torch.zeros(H, W, 4, device="cuda")
    P.render(g, sc, 6 * W * H, film, W, H)
    byt = torch.zeros(H, W, 4, dtype=torch.uint8, device="cuda")
    g.ConvertToBytes(film, byt, W, H)
    dens = torch.zeros(H, W, 4, device="cuda")
    N.check(N.load().mdas_sampling_density_device(g.handle, dens.data_ptr(), W, H), "density")
    torch.cuda.synchronize()
    for name, img in (("film.pfm", film), ("film.ppm", byt), ("film-density.pfm", dens)):
        p = str(tmp_path / name)
        P.save_image(p, img)
        back = P.read_image(p)
        ref = img.cpu().numpy()[..., :3]
        if ref.dtype == np.float32:
            assert np.array_equal(back.view(np.uint32), ref.view(np.uint32)), name
        else:
            assert np.array_equal(back, ref), name
    assert float(dens[..., 0].sum()) > 0.0
