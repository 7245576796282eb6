"""Named MDAS workloads: the benchmark configurations of the build, as
synthetic scenes with the shapes, sizes and parameter values they state.

Every workload runs the reference's budget loop
(SDK/optixMotionBlur/optixMotionBlur.cpp:768-793): initial sampling, then
sampling passes while ``N < spp * width * height``, then integrate.

``maxSamples`` is the apps' hard-coded cap of 30,000,000 samples
(optixMotionBlur.cpp:81) where the budget fits under it; above it, the cap is
raised to 1.5x the budget so that the last pass (which can add up to one
sample per leaf) still fits.
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
        need = max(self.budget, 4 * self.initial_leaves)
        if need <= APP_MAX_SAMPLES:
            return APP_MAX_SAMPLES
        return min((need * 3 + 1) // 2, (1 << 30) - 1)

    def scaled(self, width: int, height: int, **kw) -> "Workload":
        return replace(self, width=width, height=height, **kw)


WORKLOADS = {
    # 3-D motion blur (x, y, t), 64 moving discs, 256x256 at 8 spp
    "mb256": Workload("mb256", 3, 256, 256, 8, N.SCENE_DISCS_MB, 0, 64),
    # the same with extraImgBits 6, so that the initial grid (2 spp) leaves room for passes
    "mb256_eib6": Workload("mb256_eib6", 3, 256, 256, 8, N.SCENE_DISCS_MB, 0, 64, extraImgBits=6),
    # 4-D depth of field (x, y, u, v), 256 discs, thin lens f=4, aperture 0.1, 1024x1024 at 16 spp
    "dof1024": Workload("dof1024", 4, 1024, 1024, 16, N.SCENE_DISCS_DOF, 1, 256),
    # 5-D motion blur + depth of field (x, y, t, u, v), 1920x1080 at 32 spp
    "mbdof1080": Workload("mbdof1080", 5, 1920, 1080, 32, N.SCENE_DISCS_MBDOF, 100, 256),
    # 4-D direct lighting (x, y, light u, v), 3840x2160 at 64 spp
    "dl4k": Workload("dl4k", 4, 3840, 2160, 64, N.SCENE_DIRECT_LIGHT, 7, 4),
}
