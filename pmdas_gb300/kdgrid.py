"""Python mirror of the reference's sampler class ``mdas::KDGrid<Point>``
(SDK/lib/mdas/kdgrid.h:10-107) over the C ABI of libpmdas_gb300.

Method names, argument meaning and call order follow the reference:
``InitialSampling()``, ``SamplingPass()`` (= ``ComputeErrors()`` +
``AdaptiveSampling()``), ``Integrate(pixels, w, h)``, ``ConvertToBytes(...)``,
``SamplingDensity(...)``, ``Validate()`` and the ``Get*`` getters.  Device
buffers are exchanged as torch CUDA tensors (torch is only the allocator and
stream plumbing here; all work runs in the library's own kernels).

Differences from the reference, all on error paths: failures raise
:class:`MdasError` instead of printing and continuing, and a pass that would
write past the buffers raises MDAS_ERR_CAPACITY instead of overrunning them.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _native as N


class _DeviceArray:
    """Minimal __cuda_array_interface__ view of a library-owned device buffer."""

    def __init__(self, ptr: int, shape, typestr: str = "<f4"):
        self.__cuda_array_interface__ = {"data": (int(ptr), False), "shape": tuple(shape), "typestr": typestr,
                                         "version": 3, "strides": None}


def _ptr(t) -> int:
    if t is None:
        return 0
    if hasattr(t, "data_ptr"):
        return t.data_ptr()
    if isinstance(t, np.ndarray):
        return t.ctypes.data
    return int(t)


class KDGrid:
    """``mdas::KDGrid<PointN<dim>>`` with ``dim`` in 3..6."""

    def __init__(self, dim: int, maxSamples: int, candidatesNum: int, bitsPerDim: int, extraImgBits: int,
                 alpha: float, scaleX: float, scaleY: float, log: str | None = None,
                 arith: int = N.ARITH_REFERENCE, stream: int | None = None):
        lib = N.load()
        h = C.c_void_p()
        N.check(lib.mdas_create_ex(C.byref(h), dim, maxSamples, candidatesNum, bitsPerDim, extraImgBits,
                                   float(alpha), float(scaleX), float(scaleY),
                                   log.encode() if log else None, arith, stream or 0), "mdas_create")
        self._lib = lib
        self._h = h
        self.dim = dim

    # ---- lifetime
    def close(self):
        if getattr(self, "_h", None):
            self._lib.mdas_destroy(self._h)
            self._h = None

    def __del__(self):  # pragma: no cover - best effort
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream: int | None):
        N.check(self._lib.mdas_set_stream(self._h, stream or 0), "mdas_set_stream")

    # ---- the reference's methods
    def InitialSampling(self):
        N.check(self._lib.mdas_initial_sampling(self._h), "InitialSampling")

    def ComputeErrors(self):
        N.check(self._lib.mdas_compute_errors(self._h), "ComputeErrors")

    def AdaptiveSampling(self):
        N.check(self._lib.mdas_adaptive_sampling(self._h), "AdaptiveSampling")

    def SamplingPass(self):
        N.check(self._lib.mdas_sampling_pass(self._h), "SamplingPass")

    def Integrate(self, pixels, width: int, height: int):
        """``pixels``: CUDA float32 tensor with width*height*4 elements (float4 per pixel)."""
        N.check(self._lib.mdas_integrate(self._h, _ptr(pixels), width, height), "Integrate")

    def ConvertToBytes(self, pixels, pixelsBytes, width: int, height: int):
        N.check(self._lib.mdas_convert_to_bytes(self._h, _ptr(pixels), _ptr(pixelsBytes), width, height),
                "ConvertToBytes")

    def SamplingDensity(self, pixels: np.ndarray, width: int, height: int):
        """``pixels``: HOST float32 array with width*height*4 elements, as in the reference."""
        assert pixels.dtype == np.float32 and pixels.flags.c_contiguous and pixels.size >= width * height * 4
        N.check(self._lib.mdas_sampling_density(self._h, _ptr(pixels), width, height), "SamplingDensity")

    def Validate(self) -> bool:
        v = C.c_int()
        N.check(self._lib.mdas_validate(self._h, C.byref(v)), "Validate")
        return bool(v.value)

    # ---- getters (kdgrid.h:65-77)
    def _counts(self):
        a, b, c, d = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        N.check(self._lib.mdas_get_counts(self._h, C.byref(a), C.byref(b), C.byref(c), C.byref(d)), "counts")
        return a.value, b.value, c.value, d.value

    def _info(self):
        d, m, c, n, a = C.c_int(), C.c_int(), C.c_int(), C.c_int(), C.c_int()
        sx, sy = C.c_float(), C.c_float()
        N.check(self._lib.mdas_get_info(self._h, C.byref(d), C.byref(m), C.byref(c), C.byref(n), C.byref(sx),
                                        C.byref(sy), C.byref(a)), "info")
        return dict(dim=d.value, maxSamples=m.value, candidatesNum=c.value, maxNodeSize=n.value, scaleX=sx.value,
                    scaleY=sy.value, arith=a.value)

    def GetNumberOfSamples(self) -> int:
        return self._counts()[0]

    def GetNewSamples(self) -> int:
        return self._counts()[1]

    def GetNumberOfNodes(self) -> int:
        return self._counts()[2]

    def GetNewNodes(self) -> int:
        return self._counts()[3]

    def GetMaxSamples(self) -> int:
        return self._info()["maxSamples"]

    def GetCandidatesNum(self) -> int:
        return self._info()["candidatesNum"]

    def GetMaxNodeSize(self) -> int:
        return self._info()["maxNodeSize"]

    def GetScaleX(self) -> float:
        return self._info()["scaleX"]

    def GetScaleY(self) -> float:
        return self._info()["scaleY"]

    def GetGError(self) -> float:
        f = C.c_float()
        N.check(self._lib.mdas_get_gerror(self._h, C.byref(f)), "g_error")
        return f.value

    def GetSampleCoordinatesPtr(self) -> int:
        return self._lib.mdas_sample_coordinates(self._h)

    def GetSampleValuesPtr(self) -> int:
        return self._lib.mdas_sample_values(self._h)

    def GetSampleCoordinates(self, count: int | None = None):
        """Device view (torch CUDA tensor [count, dim]) of the coordinate buffer."""
        import torch
        n = self.GetNumberOfSamples() if count is None else count
        return torch.as_tensor(_DeviceArray(self.GetSampleCoordinatesPtr(), (n, self.dim)), device="cuda")

    def GetSampleValues(self, count: int | None = None):
        """Device view (torch CUDA tensor [count, 3]) of the value buffer (float3)."""
        import torch
        n = self.GetNumberOfSamples() if count is None else count
        return torch.as_tensor(_DeviceArray(self.GetSampleValuesPtr(), (n, 3)), device="cuda")

    # ---- state (checkpoint / parity)
    def dump_state(self) -> dict:
        n, _, l, _ = self._counts()
        st = dict(N=n, L=l,
                  coords=np.empty((n, self.dim), np.float32), values=np.empty((n, 3), np.float32),
                  nodes=np.empty((l, 4), np.int32), boxes=np.empty((l, 2 * self.dim), np.float32),
                  errors=np.empty(l, np.float32), seeds=np.empty(l, np.uint32))
        N.check(self._lib.mdas_dump_state(self._h, _ptr(st["coords"]), _ptr(st["values"]), _ptr(st["nodes"]),
                                          _ptr(st["boxes"]), _ptr(st["errors"]), _ptr(st["seeds"])), "dump_state")
        return st

    def load_state(self, st: dict):
        arrs = {}
        for k, dt in (("coords", np.float32), ("values", np.float32), ("nodes", np.int32), ("boxes", np.float32),
                      ("errors", np.float32), ("seeds", np.uint32)):
            arrs[k] = np.ascontiguousarray(st[k], dtype=dt)
        N.check(self._lib.mdas_load_state(self._h, int(st["N"]), int(st["L"]), _ptr(arrs["coords"]),
                                          _ptr(arrs["values"]), _ptr(arrs["nodes"]), _ptr(arrs["boxes"]),
                                          _ptr(arrs["errors"]), _ptr(arrs["seeds"])), "load_state")

    # ---- timing / accounting
    def set_timing(self, on: bool = True):
        N.check(self._lib.mdas_set_timing(self._h, 1 if on else 0), "set_timing")

    def stage_times(self, reset: bool = False) -> list:
        """Per-stage ms since the last reset: init, errors, adaptive (kernels),
        integrate, integrand, and the adaptive pass until the host holds its counts."""
        a = (C.c_double * 6)()
        N.check(self._lib.mdas_get_stage_times_ex(self._h, a, 6, 1 if reset else 0), "stage_times")
        return list(a)

    def pass_stats(self) -> dict:
        """Tallies of the last pass: recomputed errors, accepted leaves, splits, gathered samples."""
        r, s, p, g = C.c_int(), C.c_int(), C.c_int(), C.c_int64()
        N.check(self._lib.mdas_get_pass_stats(self._h, C.byref(r), C.byref(s), C.byref(p), C.byref(g)), "stats")
        return dict(recomputed=r.value, selected=s.value, splits=p.value, gathered=g.value)

    def launch_count(self) -> int:
        v = C.c_uint64()
        N.check(self._lib.mdas_get_launch_count(self._h, C.byref(v)), "launch_count")
        return v.value

    # ---- leaf order and hierarchy (no reference counterpart)
    def LeafOrder(self, fineBits: int = -1):
        """(sorted keys, leaf slots in key order) as torch CUDA tensors (int64 holding
        uint64 keys, int32 holding uint32 slots)."""
        import torch
        n = self.GetNumberOfNodes()
        keys = torch.empty(max(n, 1), dtype=torch.int64, device="cuda")
        order = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
        N.check(self._lib.mdas_leaf_order(self._h, fineBits, _ptr(keys), _ptr(order)), "leaf_order")
        return keys[:n], order[:n]

    def BuildHierarchy(self, fineBits: int = -1):
        N.check(self._lib.mdas_build_hierarchy(self._h, fineBits), "build_hierarchy")

    def Hierarchy(self) -> dict:
        """Host copy of the hierarchy: keys (uint64), order (uint32), children
        [n-1, 2], parents [2n-1], boxes [n-1, 2*dim]."""
        n = self.GetNumberOfNodes()
        h = dict(keys=np.empty(n, np.uint64), order=np.empty(n, np.uint32),
                 children=np.empty((max(n - 1, 0), 2), np.int32), parents=np.empty(max(2 * n - 1, 0), np.int32),
                 boxes=np.empty((max(n - 1, 0), 2 * self.dim), np.float32))
        cnt = C.c_int()
        N.check(self._lib.mdas_get_hierarchy(self._h, C.byref(cnt), _ptr(h["keys"]), _ptr(h["order"]),
                                             _ptr(h["children"]), _ptr(h["parents"]), _ptr(h["boxes"])), "hierarchy")
        return h

    def Locate(self, points):
        """Leaf slot holding each point (torch CUDA float32 [n, dim]) -> int32 [n], -1 outside."""
        import torch
        pts = points.contiguous()
        out = torch.empty(max(pts.shape[0], 1), dtype=torch.int32, device="cuda")
        N.check(self._lib.mdas_locate(self._h, _ptr(pts), int(pts.shape[0]), _ptr(out)), "locate")
        return out[:pts.shape[0]]

    # ---- learned acceptance (no reference counterpart)
    def LearnedEnable(self, on: bool = True, params=None, tolerance: float = 0.05, seed: int = 1):
        """Learned mode on (trained `params`, MDAS_MLP_PARAMS floats, or seeded initial weights) or off."""
        if not on:
            N.check(self._lib.mdas_learned_enable(self._h, None), "learned_enable")
            return
        c = N.LearnedConfig()
        N.check(self._lib.mdas_learned_defaults(C.byref(c)), "learned_defaults")
        c.tolerance = tolerance
        c.seed = seed
        keep = None
        if params is not None:
            keep = np.ascontiguousarray(params, np.float32)
            assert keep.size == N.MLP_PARAMS
            c.params = keep.ctypes.data
        N.check(self._lib.mdas_learned_enable(self._h, C.byref(c)), "learned_enable")

    def LearnedUpdate(self):
        """Predict every leaf and judge the pass (after ComputeErrors)."""
        N.check(self._lib.mdas_learned_update(self._h), "learned_update")

    def LearnedStats(self) -> dict:
        j, p, lp, ul, up = C.c_int(), C.c_int(), C.c_int(), C.c_double(), C.c_double()
        N.check(self._lib.mdas_learned_stats(self._h, C.byref(j), C.byref(p), C.byref(lp), C.byref(ul), C.byref(up)),
                "stats")
        return dict(judged=j.value, plain=p.value, last_plain=lp.value, unrefined_learned=ul.value,
                    unrefined_plain=up.value)

    def LeafTrueErrors(self, scene, samples: int = 64, seed: int = 1, leaves=None):
        """Training targets: the true reconstruction error of every leaf, or of the
        leaf slots in `leaves` (torch CUDA int32) -> torch CUDA float32."""
        import torch
        n = self.GetNumberOfNodes() if leaves is None else int(leaves.shape[0])
        out = torch.empty(max(n, 1), dtype=torch.float32, device="cuda")
        idx = None if leaves is None else leaves.contiguous()
        N.check(self._lib.mdas_leaf_true_errors(self._h, scene.handle, samples, seed, _ptr(idx), n, _ptr(out)),
                "leaf_true_errors")
        return out[:n]

    def LearnedPredict(self):
        N.check(self._lib.mdas_learned_predict(self._h), "learned_predict")

    def LearnedParams(self) -> np.ndarray:
        p = np.empty(N.MLP_PARAMS, np.float32)
        N.check(self._lib.mdas_learned_get_params(self._h, _ptr(p)), "learned_get_params")
        return p

    def SetLearnedParams(self, p: np.ndarray):
        q = np.ascontiguousarray(p, np.float32)
        assert q.size == N.MLP_PARAMS
        N.check(self._lib.mdas_learned_set_params(self._h, _ptr(q)), "learned_set_params")

    def LearnedPredMax(self) -> float:
        """The largest priority the last learned update used."""
        v = C.c_float()
        N.check(self._lib.mdas_learned_pred_max(self._h, C.byref(v)), "learned_pred_max")
        return v.value

    def LearnedPredictions(self):
        import torch
        n = self.GetNumberOfNodes()
        out = torch.empty(max(n, 1), dtype=torch.float32, device="cuda")
        N.check(self._lib.mdas_learned_predictions(self._h, _ptr(out)), "learned_predictions")
        return out[:n]

    def LeafFeatures(self):
        import torch
        n = self.GetNumberOfNodes()
        out = torch.empty((max(n, 1), 16), dtype=torch.float32, device="cuda")
        N.check(self._lib.mdas_leaf_features(self._h, _ptr(out)), "leaf_features")
        return out[:n]


def mlp_forward(params, features):
    """pred [m] of the MLP (params: torch CUDA float32 [MDAS_MLP_PARAMS], features [m, 16])."""
    import torch
    p, f = params.contiguous(), features.contiguous()
    m = f.shape[0]
    out = torch.empty(max(m, 1), dtype=torch.float32, device="cuda")
    N.check(N.load().mdas_mlp_forward(_ptr(p), _ptr(f), m, _ptr(out), None), "mlp_forward")
    return out[:m]


def mlp_adam(params, m1, m2, grads, step: int, lr: float):
    """One Adam step on torch CUDA float32 [MDAS_MLP_PARAMS] tensors, in place (grads zeroed)."""
    N.check(N.load().mdas_mlp_adam(_ptr(params), _ptr(m1), _ptr(m2), _ptr(grads), int(step), float(lr), None),
            "mlp_adam")


def mlp_gradients(params, features, targets):
    """(grads [MDAS_MLP_PARAMS], loss) of mean((pred - targets)^2)."""
    import torch
    p, f, t = params.contiguous(), features.contiguous(), targets.contiguous()
    g = torch.empty(N.MLP_PARAMS, dtype=torch.float32, device="cuda")
    loss = C.c_float()
    N.check(N.load().mdas_mlp_gradients(_ptr(p), _ptr(f), _ptr(t), f.shape[0], _ptr(g), C.byref(loss), None),
            "mlp_gradients")
    return g, loss.value


def morton_key_bits(dim: int, bitsPerDim: int, extraImgBits: int, fineBits: int) -> int:
    return N.load().mdas_morton_key_bits(dim, bitsPerDim, extraImgBits, fineBits)


def morton_encode(points, bitsPerDim: int, extraImgBits: int, fineBits: int, scaleX: float, scaleY: float):
    """Keys (torch int64 holding uint64) of points (torch CUDA float32 [n, dim])."""
    import torch
    pts = points.contiguous()
    n, dim = pts.shape
    keys = torch.empty(max(n, 1), dtype=torch.int64, device="cuda")
    N.check(N.load().mdas_morton_encode(dim, bitsPerDim, extraImgBits, fineBits, float(scaleX), float(scaleY),
                                        _ptr(pts), n, _ptr(keys), None), "morton_encode")
    torch.cuda.synchronize()
    return keys[:n]


def morton_decode(cells, dim: int, bitsPerDim: int, extraImgBits: int, scaleX: float, scaleY: float):
    """Boxes [n, 2*dim] (mn, mx) of cells (torch CUDA int64 holding uint64)."""
    import torch
    c = cells.contiguous()
    n = c.shape[0]
    boxes = torch.empty((max(n, 1), 2 * dim), dtype=torch.float32, device="cuda")
    N.check(N.load().mdas_morton_decode(dim, bitsPerDim, extraImgBits, float(scaleX), float(scaleY), _ptr(c), n,
                                        _ptr(boxes), None), "morton_decode")
    torch.cuda.synchronize()
    return boxes[:n]


def radix_sort_pairs(keys, values=None, beginBit: int = 0, endBit: int = 64):
    """Stable sort of (keys, values) on key bits [beginBit, endBit): torch CUDA int64
    keys (read as uint64) and int32 values (uint32; None = 0..n-1)."""
    import torch
    lib = N.load()
    k = keys.contiguous()
    n = k.shape[0]
    v = values.contiguous() if values is not None else None
    need = C.c_size_t(0)
    N.check(lib.mdas_radix_sort_pairs(None, C.byref(need), None, None, None, None, n, beginBit, endBit, None),
            "radix_sort_pairs")
    temp = torch.empty(max(need.value, 1), dtype=torch.uint8, device="cuda")
    ko = torch.empty(max(n, 1), dtype=torch.int64, device="cuda")
    vo = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
    N.check(lib.mdas_radix_sort_pairs(_ptr(temp), C.byref(need), _ptr(k), _ptr(ko), _ptr(v), _ptr(vo), n, beginBit,
                                      endBit, None), "radix_sort_pairs")
    return ko[:n], vo[:n]


@dataclass
class SceneDesc:
    kind: int
    dim: int
    count: int
    desc_bytes: bytes
    prims: np.ndarray


class Scene:
    """A seeded analytic integrand (stands in for the OptiX ray generation programs)."""

    def __init__(self, kind: int, seed: int, count: int, scaleX: float, scaleY: float, width: int, height: int):
        lib = N.load()
        h = C.c_void_p()
        N.check(lib.mdas_scene_create(C.byref(h), kind, seed, count, float(scaleX), float(scaleY), width, height),
                "mdas_scene_create")
        self._lib = lib
        self._h = h
        self.kind = kind

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            self._lib.mdas_scene_destroy(self._h)
            self._h = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass

    def export(self) -> SceneDesc:
        size = self._lib.mdas_scene_desc_size()
        desc = C.create_string_buffer(size)
        dim, count = C.c_int(), C.c_int()
        N.check(self._lib.mdas_scene_export(self._h, None, 0, None, 0, C.byref(dim), C.byref(count)), "export")
        prims = np.zeros((max(count.value, 1), N.PRIM_STRIDE), np.float32)
        N.check(self._lib.mdas_scene_export(self._h, desc, size, prims.ctypes.data, count.value, C.byref(dim),
                                            C.byref(count)), "export")
        return SceneDesc(self.kind, dim.value, count.value, desc.raw, prims[:count.value].copy())

    def evaluate_buffers(self, coords_ptr: int, values_ptr: int, dim: int, offset: int, count: int,
                         stream: int | None = None):
        """Evaluate samples [offset, offset+count) of any device coordinate buffer into a value buffer."""
        N.check(self._lib.mdas_scene_evaluate(self._h, coords_ptr, values_ptr, dim, offset, count, stream or 0),
                "mdas_scene_evaluate")

    def reference_image(self, width: int, height: int, spp: int = 4096, seed: int = 12345):
        """FP64-accumulated reference image (torch CUDA float64 tensor [H, W, 3])."""
        import torch
        out = torch.empty(height, width, 3, dtype=torch.float64, device="cuda")
        N.check(self._lib.mdas_scene_reference_image(self._h, width, height, spp, seed, out.data_ptr(), 0),
                "mdas_scene_reference_image")
        return out

    def evaluate(self, grid: KDGrid, offset: int, count: int):
        """launchSubframe: evaluate samples [offset, offset+count) of `grid` in place."""
        N.check(self._lib.mdas_evaluate(grid.handle, self._h, offset, count), "mdas_evaluate")


def save_image(path: str, pixels) -> None:
    """Write an (H, W, 4) image held in host memory (numpy) or on the device
    (torch; copied to the host first) to `path`: float32 as a Portable Float
    Map, uint8 (after ConvertToBytes) as a binary PPM — the headless stand-ins
    for the sample apps' EXR and PPM output (optixMotionBlur.cpp:795-840)."""
    a = pixels.detach().cpu().numpy() if hasattr(pixels, "detach") else np.asarray(pixels)
    if a.ndim != 3 or a.shape[2] != 4:
        raise ValueError(f"expected an (H, W, 4) image, got shape {a.shape}")
    if a.dtype == np.float32:
        fmt = N.IMAGE_FLOAT4
    elif a.dtype == np.uint8:
        fmt = N.IMAGE_UCHAR4
    else:
        raise ValueError(f"expected float32 or uint8 pixels, got {a.dtype}")
    a = np.ascontiguousarray(a)
    N.check(N.load().mdas_save_image(path.encode(), a.ctypes.data, a.shape[1], a.shape[0], fmt), "mdas_save_image")


def read_image(path: str) -> np.ndarray:
    """Read a PFM (as (H, W, 3) float32, top row first) or a binary PPM (as
    (H, W, 3) uint8) written by save_image."""
    with open(path, "rb") as f:
        data = f.read()
    parts, pos = [], 0
    while len(parts) < 4:  # magic, width, height, scale or maxval
        while data[pos:pos + 1].isspace():
            pos += 1
        end = pos
        while not data[end:end + 1].isspace():
            end += 1
        parts.append(data[pos:end].decode())
        pos = end
    pos += 1  # the single whitespace byte after the header
    magic, w, h = parts[0], int(parts[1]), int(parts[2])
    if magic == "PF":
        dt = "<f4" if float(parts[3]) < 0 else ">f4"
        img = np.frombuffer(data, dtype=dt, count=w * h * 3, offset=pos).reshape(h, w, 3)
        return img[::-1].astype(np.float32)
    if magic == "P6":
        return np.frombuffer(data, dtype=np.uint8, count=w * h * 3, offset=pos).reshape(h, w, 3).copy()
    raise ValueError(f"{path}: not a PFM or binary PPM file")


def render(grid: KDGrid, scene: Scene, budget: int, pixels, width: int, height: int) -> N.RenderStats:
    """The headless budget loop of the sample apps (optixMotionBlur.cpp:768-793)."""
    st = N.RenderStats()
    N.check(grid._lib.mdas_render(grid.handle, scene.handle, int(budget), _ptr(pixels), width, height,
                                  C.byref(st)), "mdas_render")
    return st


def render_graph(grid: KDGrid, scene: Scene, budget: int, pixels, width: int, height: int) -> N.RenderStats:
    """The budget loop as one CUDA graph with a device-side loop (no host sync per pass)."""
    st = N.RenderStats()
    N.check(grid._lib.mdas_render_graph(grid.handle, scene.handle, int(budget), _ptr(pixels), width, height,
                                        C.byref(st)), "mdas_render_graph")
    return st


def render_host(grid: KDGrid, scene: Scene, budget: int, host_pixels: np.ndarray, width: int, height: int,
                host_prims: np.ndarray | None = None) -> N.RenderStats:
    """The budget loop with host input (scene primitives) and host output (float4 image)."""
    assert host_pixels.dtype == np.float32 and host_pixels.size >= width * height * 4
    st = N.RenderStats()
    N.check(grid._lib.mdas_render_host(grid.handle, scene.handle, _ptr(host_prims), int(budget), _ptr(host_pixels),
                                       width, height, C.byref(st)), "mdas_render_host")
    return st


class Batch:
    """Many images rendered together: one CUDA graph, one launch per stage and
    point dimension, a device-side loop until every image reached its budget."""

    def __init__(self, grids, scenes, budgets, pixels, widths, heights):
        lib = N.load()
        n = len(grids)
        self._keep = (list(grids), list(scenes), list(pixels))
        G = (C.c_void_p * n)(*[g.handle.value for g in grids])
        S = (C.c_void_p * n)(*[sc.handle.value for sc in scenes])
        B = (C.c_int * n)(*[int(b) for b in budgets])
        Pp = (C.c_void_p * n)(*[_ptr(p) for p in pixels])
        W = (C.c_int * n)(*[int(w) for w in widths])
        H = (C.c_int * n)(*[int(h) for h in heights])
        h = C.c_void_p()
        N.check(lib.mdas_batch_create(C.byref(h), n, G, S, B, Pp, W, H), "mdas_batch_create")
        self._lib = lib
        self._h = h
        self.n = n

    def close(self):
        if getattr(self, "_h", None):
            self._lib.mdas_batch_destroy(self._h)
            self._h = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass

    def render(self):
        st = (N.RenderStats * self.n)()
        N.check(self._lib.mdas_batch_render(self._h, st), "mdas_batch_render")
        return list(st)

    def render_stepped(self):
        """The same render with the pass loop on the host (kernels visible to profilers)."""
        st = (N.RenderStats * self.n)()
        N.check(self._lib.mdas_batch_render_stepped(self._h, st), "mdas_batch_render_stepped")
        return list(st)

    def set_tuning(self, ctas_per_sm):
        a = (C.c_int * 4)(*ctas_per_sm)
        N.check(self._lib.mdas_batch_set_tuning(self._h, a), "mdas_batch_set_tuning")

    def set_tiling(self, ctas_per_sm, leaves_per_tile: int):
        """Per-stage CTAs per SM plus the decide tile size (1024 or 2048 leaves)."""
        a = (C.c_int * 4)(*ctas_per_sm)
        N.check(self._lib.mdas_batch_set_tiling(self._h, a, int(leaves_per_tile)), "mdas_batch_set_tiling")

    def autotune(self, repeats: int = 2):
        a = (C.c_int * 4)()
        ms = C.c_double()
        N.check(self._lib.mdas_batch_autotune(self._h, repeats, a, C.byref(ms)), "mdas_batch_autotune")
        return list(a), ms.value

    def autotune_ex(self, repeats: int = 2):
        """Coordinate-descent autotune over the decide tile size and every stage's
        CTAs per SM: returns (ctas_per_sm, leaves_per_tile, ms_per_render, evaluated)."""
        a = (C.c_int * 4)()
        tile = C.c_int()
        ms = C.c_double()
        ev = C.c_int()
        N.check(self._lib.mdas_batch_autotune_ex(self._h, repeats, a, C.byref(tile), C.byref(ms), C.byref(ev)),
                "mdas_batch_autotune_ex")
        return list(a), tile.value, ms.value, ev.value
