"""Named MDAS workloads: the benchmark configurations of the build, as
synthetic scenes with the shapes, sizes and parameter values they state.

Every workload runs the reference's budget loop
(SDK/optixMotionBlur/optixMotionBlur.cpp:768-793): initial sampling, then
sampling passes while ``N < spp * width * height``, then integrate.

``maxSamples`` is the apps' hard-coded cap of 30,000,000 samples
(optixMotionBlur.cpp:81), raised to 1.5x the budget where that is larger, so
that the last pass (which can add up to one sample per leaf) still fits.
"""
from __future__ import annotations

from dataclasses import dataclass, replace

from . import _native as N

APP_MAX_SAMPLES = 30_000_000


@dataclass(frozen=True)
class Workload:
    name: str
    dim: int
    width: int
    height: int
    spp: float
    scene_kind: int
    scene_seed: int
    scene_count: int
    scaleFactor: float = 1.0
    alpha: float = 0.25
    bitsPerDim: int = 1
    extraImgBits: int = 8
    candidatesNum: int = 4
    capacity: int = 0  # sample capacity; 0 = the apps' cap, raised to 1.5x the budget where larger

    @property
    def scaleX(self) -> float:
        return self.scaleFactor * self.width

    @property
    def scaleY(self) -> float:
        return self.scaleFactor * self.height

    @property
    def budget(self) -> int:
        return int(self.spp * self.width * self.height)

    @property
    def initial_leaves(self) -> int:
        return (1 << (self.bitsPerDim * self.dim)) << (2 * self.extraImgBits)

    @property
    def maxSamples(self) -> int:
        # the last pass can add one sample per leaf (<= N/2), so 1.5x the budget always fits
        if self.capacity:
            return self.capacity
        need = max(self.budget, 4 * self.initial_leaves)
        return min(max(APP_MAX_SAMPLES, (need * 3 + 1) // 2), (1 << 30) - 1)

    def scaled(self, width: int, height: int, **kw) -> "Workload":
        return replace(self, width=width, height=height, **kw)


WORKLOADS = {
    # 3-D motion blur (x, y, t), 64 moving discs, 256x256 at 8 spp
    "mb256": Workload("mb256", 3, 256, 256, 8, N.SCENE_DISCS_MB, 0, 64),
    # the same with extraImgBits 6, so that the initial grid (2 spp) leaves room for passes
    "mb256_eib6": Workload("mb256_eib6", 3, 256, 256, 8, N.SCENE_DISCS_MB, 0, 64, extraImgBits=6),
    # 4-D depth of field (x, y, u, v), 256 discs, thin lens f=4, aperture 0.1, 1024x1024 at 16 spp
    "dof1024": Workload("dof1024", 4, 1024, 1024, 16, N.SCENE_DISCS_DOF, 1, 256),
    # 5-D motion blur + depth of field (x, y, t, u, v), 1920x1080 at 32 spp; scene seed 100 is the
    # held-out evaluation scene of the learned priority (trained on seeds 1-32)
    "mbdof1080": Workload("mbdof1080", 5, 1920, 1080, 32, N.SCENE_DISCS_MBDOF, 100, 256),
    # 4-D direct lighting (x, y, light u, v), 3840x2160 at 64 spp; scene seed 100 as above
    "dl4k": Workload("dl4k", 4, 3840, 2160, 64, N.SCENE_DIRECT_LIGHT, 100, 4),
}


# ---- the batched workload: 64 images of uneven resolution, budget and dimension
BATCH_RESOLUTIONS = ((256, 256), (512, 512), (1280, 720), (1920, 1080))
BATCH_SPP = (4, 8, 16, 32)
BATCH_KINDS = ((3, N.SCENE_DISCS_MB, 64), (4, N.SCENE_DISCS_DOF, 256))  # (dim, scene, primitives)


def batch_image(seed: int) -> Workload:
    """Image `seed` of the batch: resolution, spp and dimension drawn from the
    seed (numpy PCG64 stream, in that order); extraImgBits chosen so that the
    initial grid holds at most 1 sample per pixel, so every image takes passes."""
    import math
    import numpy as np
    rng = np.random.default_rng(seed)
    W, H = BATCH_RESOLUTIONS[int(rng.integers(4))]
    spp = BATCH_SPP[int(rng.integers(4))]
    dim, kind, count = BATCH_KINDS[int(rng.integers(2))]
    eib = max(0, int(math.floor(math.log(W * H / (4 * 2 ** dim), 4))))
    budget = spp * W * H
    # every image of the batch holds its own state: size it to its budget (1.5x, see maxSamples)
    return Workload(f"batch-{seed}", dim, W, H, spp, kind, seed, count, extraImgBits=eib,
                    capacity=(max(budget, 4 * ((1 << dim) << (2 * eib))) * 3 + 1) // 2)


def batch_workloads(first_seed: int = 200, n: int = 64) -> list:
    return [batch_image(first_seed + k) for k in range(n)]
