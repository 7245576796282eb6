"""ctypes wrapper of the CPU oracle (oracle/mdas_oracle.cpp) and of the
reference harness (oracle/ref_harness.cu).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as
the checker, and by bench.py for the CPU baseline.  The product never imports
this module.
"""
from __future__ import annotations

import ctypes as C
import os
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "_build", "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libmdas_ref.so")

_P = C.c_void_p
_I = C.c_int
_F = C.c_float

_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_LIB):
            from oracle import build as _build
            _build.build_oracle()
        lib = C.CDLL(ORACLE_LIB)
        sig = {
            "orc_set_threads": (_I, [_I]),
            "orc_initial_sampling": (_I, [_I, _I, _I, _F, _F, _I, _P, _P, _P, _P, _P, C.POINTER(_I), C.POINTER(_I)]),
            "orc_compute_errors": (_F, [_I, _I, _P, _P, _P, _P]),
            "orc_adaptive_sampling": (_I, [_I, _I, _I, _I, _I, _F, _F, _P, _P, _P, _P, _P, C.POINTER(_I),
                                           C.POINTER(_I), _P]),
            "orc_integrate": (_I, [_I, _I, _I, _I, _F, _F, _P, _P, _P, _P, _I]),
            "orc_convert_to_bytes": (_I, [_I, _P, _P]),
            "orc_sampling_density": (_I, [_I, _I, _F, _F, _P, _P, _I, _I]),
            "orc_validate": (_I, [_I, _I, _I, _F, _F, _P, _P, _P]),
            "orc_evaluate": (_I, [_P, _P, _I, _P, _P, _I, _I]),
            "orc_powf": (_F, [_F, _F]),
            "orc_log2f": (_F, [_F]),
            "orc_exp2f": (_F, [_F]),
            "orc_sincos": (None, [_F, C.POINTER(_F), C.POINTER(_F)]),
            "orc_render": (_I, [_I, _I, _I, _I, _F, _F, _F, _I, _I, _I, _P, _P, _I, _I, _P, _P, _P, _P, _P, _P, _P,
                                _I, C.POINTER(_I), C.POINTER(_I), C.POINTER(_I), C.POINTER(C.c_double)]),
            "orc_morton_encode": (_I, [_I, _I, _I, _I, _F, _F, _P, _I, _P]),
            "orc_morton_decode": (_I, [_I, _I, _I, _F, _F, _P, _I, _P]),
            "orc_leaf_keys": (_I, [_I, _I, _I, _I, _F, _F, _P, _I, _P]),
            "orc_sort_pairs": (_I, [_P, _I, _I, _I, _P, _P]),
            "orc_karras": (_I, [_P, _I, _P, _P]),
            "orc_refit": (_I, [_I, _P, _P, _I, _P, _P]),
            "orc_locate": (_I, [_I, _P, _P, _I, _P, _I, _P]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def set_threads(n: int) -> int:
    return load().orc_set_threads(n)


def _p(a):
    return None if a is None else a.ctypes.data


class OracleGrid:
    """The sampler state in host numpy arrays, advanced by the CPU oracle."""

    def __init__(self, dim, maxSamples, candidatesNum, bitsPerDim, extraImgBits, alpha, scaleX, scaleY):
        self.dim = dim
        self.maxSamples = maxSamples
        self.candidatesNum = candidatesNum
        self.bpd = bitsPerDim
        self.eib = extraImgBits
        self.alpha = np.float32(alpha)
        self.sx = np.float32(scaleX)
        self.sy = np.float32(scaleY)
        self.capSamples = (maxSamples + 127) // 128 * 128
        self.capNodes = 2 * maxSamples - 1
        self.coords = np.zeros((self.capSamples, dim), np.float32)
        self.values = np.zeros((self.capSamples, 3), np.float32)
        self.nodes = np.zeros((self.capNodes, 4), np.int32)
        self.boxes = np.zeros((self.capNodes, 2 * dim), np.float32)
        self.errors = np.zeros(self.capNodes, np.float32)
        self.seeds = np.zeros(self.capNodes, np.uint32)
        self.N = self.L = self.newN = self.newL = 0
        self.gerr = np.float32(0)

    def initial_sampling(self):
        n, l = C.c_int(), C.c_int()
        rc = load().orc_initial_sampling(self.dim, self.bpd, self.eib, self.sx, self.sy, self.capNodes,
                                         _p(self.coords), _p(self.nodes), _p(self.boxes), _p(self.errors),
                                         _p(self.seeds), C.byref(n), C.byref(l))
        assert rc == 0, rc
        self.N, self.L = n.value, l.value
        assert self.N <= self.maxSamples

    def compute_errors(self) -> np.float32:
        self.gerr = np.float32(load().orc_compute_errors(self.dim, self.L, _p(self.errors), _p(self.nodes),
                                                         _p(self.boxes), _p(self.values)))
        return self.gerr

    def adaptive_sampling(self, gerr=None):
        g = self.gerr if gerr is None else np.float32(gerr)
        assert self.N + self.L <= self.maxSamples and 2 * self.L <= self.capNodes
        nn, nl = C.c_int(), C.c_int()
        mask = np.zeros(self.L, np.uint8)
        rc = load().orc_adaptive_sampling(self.dim, self.N, self.L, 4, self.candidatesNum, self.alpha, g,
                                          _p(self.errors), _p(self.nodes), _p(self.boxes), _p(self.coords),
                                          _p(self.seeds), C.byref(nn), C.byref(nl), _p(mask))
        assert rc == 0
        self.newN, self.newL = nn.value, nl.value
        self.N += self.newN
        self.L += self.newL
        return mask

    def sampling_pass(self):
        self.compute_errors()
        return self.adaptive_sampling()

    def evaluate(self, scene, offset, count):
        desc = C.create_string_buffer(scene.desc_bytes, len(scene.desc_bytes))
        prims = np.ascontiguousarray(scene.prims, np.float32)
        load().orc_evaluate(desc, prims.ctypes.data if prims.size else None, self.dim, _p(self.coords),
                            _p(self.values), offset, count)

    def integrate(self, width, height, threads=1) -> np.ndarray:
        px = np.zeros((height, width, 4), np.float32)
        load().orc_integrate(self.dim, self.L, width, height, self.sx, self.sy, _p(self.nodes), _p(self.boxes),
                             _p(self.values), _p(px), threads)
        return px

    def sampling_density(self, width, height) -> np.ndarray:
        px = np.zeros((height, width, 4), np.float32)
        load().orc_sampling_density(self.dim, self.N, self.sx, self.sy, _p(self.coords), _p(px), width, height)
        return px

    def validate(self) -> int:
        return load().orc_validate(self.dim, self.N, self.L, self.sx, self.sy, _p(self.coords), _p(self.nodes),
                                   _p(self.boxes))

    def dump_state(self) -> dict:
        n, l = self.N, self.L
        return dict(N=n, L=l, coords=self.coords[:n].copy(), values=self.values[:n].copy(),
                    nodes=self.nodes[:l].copy(), boxes=self.boxes[:l].copy(), errors=self.errors[:l].copy(),
                    seeds=self.seeds[:l].copy())

    def load_state(self, st: dict):
        n, l = int(st["N"]), int(st["L"])
        self.coords[:n] = st["coords"]
        self.values[:n] = st["values"]
        self.nodes[:l] = st["nodes"]
        self.boxes[:l] = st["boxes"]
        self.errors[:l] = st["errors"]
        self.seeds[:l] = st["seeds"]
        self.seeds[l:] = 0
        self.N, self.L = n, l


def evaluate_points(scene, points) -> np.ndarray:
    """The integrand at arbitrary points (rows of `dim` floats) -> [n, 3] values."""
    pts = np.ascontiguousarray(points, np.float32)
    n, dim = pts.shape
    vals = np.zeros((max(n, 1), 3), np.float32)
    desc = C.create_string_buffer(scene.desc_bytes, len(scene.desc_bytes))
    prims = np.ascontiguousarray(scene.prims, np.float32)
    load().orc_evaluate(desc, prims.ctypes.data if prims.size else None, dim, _p(pts), _p(vals), 0, n)
    return vals[:n]


def convert_to_bytes(pixels: np.ndarray) -> np.ndarray:
    px = np.ascontiguousarray(pixels, np.float32)
    out = np.zeros(px.shape[:-1] + (4,), np.uint8)
    load().orc_convert_to_bytes(px.size // 4, px.ctypes.data, out.ctypes.data)
    return out


def powf(x, y) -> np.float32:
    return np.float32(load().orc_powf(np.float32(x), np.float32(y)))


def render(dim, bpd, eib, cand, alpha, sx, sy, budget, maxSamples, scene, width, height, threads=1):
    """The whole CPU budget loop; returns (pixels, N, L, passes, times_ms[5], wall_s)."""
    capS = (maxSamples + 127) // 128 * 128
    capN = 2 * maxSamples - 1
    coords = np.empty((capS, dim), np.float32)
    values = np.empty((capS, 3), np.float32)
    nodes = np.empty((capN, 4), np.int32)
    boxes = np.empty((capN, 2 * dim), np.float32)
    errors = np.empty(capN, np.float32)
    seeds = np.empty(capN, np.uint32)
    px = np.zeros((height, width, 4), np.float32)
    desc = C.create_string_buffer(scene.desc_bytes, len(scene.desc_bytes))
    prims = np.ascontiguousarray(scene.prims, np.float32)
    n, l, p = C.c_int(), C.c_int(), C.c_int()
    t = (C.c_double * 5)()
    set_threads(threads)
    t0 = time.perf_counter()
    rc = load().orc_render(dim, bpd, eib, cand, np.float32(alpha), np.float32(sx), np.float32(sy), budget, capS,
                           capN, desc, prims.ctypes.data if prims.size else None, width, height, _p(coords),
                           _p(values), _p(nodes), _p(boxes), _p(errors), _p(seeds), _p(px), threads, C.byref(n),
                           C.byref(l), C.byref(p), t)
    wall = time.perf_counter() - t0
    assert rc == 0, rc
    return px, n.value, l.value, p.value, list(t), wall


# ---- leaf ordering (Morton keys, stable sort, radix tree, point location) -----------
def morton_encode(points, bpd, eib, fine, sx, sy) -> np.ndarray:
    pts = np.ascontiguousarray(points, np.float32)
    n, dim = pts.shape
    keys = np.zeros(max(n, 1), np.uint64)
    assert load().orc_morton_encode(dim, bpd, eib, fine, np.float32(sx), np.float32(sy), _p(pts), n, _p(keys)) == 0
    return keys[:n]


def morton_decode(cells, dim, bpd, eib, sx, sy) -> np.ndarray:
    c = np.ascontiguousarray(cells, np.uint64)
    boxes = np.zeros((max(c.size, 1), 2 * dim), np.float32)
    assert load().orc_morton_decode(dim, bpd, eib, np.float32(sx), np.float32(sy), _p(c), c.size, _p(boxes)) == 0
    return boxes[:c.size]


def leaf_keys(boxes, dim, bpd, eib, fine, sx, sy) -> np.ndarray:
    b = np.ascontiguousarray(boxes, np.float32)
    L = b.shape[0]
    keys = np.zeros(max(L, 1), np.uint64)
    assert load().orc_leaf_keys(dim, bpd, eib, fine, np.float32(sx), np.float32(sy), _p(b), L, _p(keys)) == 0
    return keys[:L]


def sort_pairs(keys, begin=0, end=64):
    """(sorted keys, permutation) of a stable sort on key bits [begin, end)."""
    k = np.ascontiguousarray(keys, np.uint64)
    n = k.size
    sk = np.zeros(max(n, 1), np.uint64)
    order = np.zeros(max(n, 1), np.uint32)
    assert load().orc_sort_pairs(_p(k), n, begin, end, _p(sk), _p(order)) == 0
    return sk[:n], order[:n]


def karras(sorted_keys):
    """(children [n-1, 2], parents [2n-1]) of the radix tree over sorted keys."""
    k = np.ascontiguousarray(sorted_keys, np.uint64)
    n = k.size
    children = np.zeros((max(n - 1, 1), 2), np.int32)
    parents = np.zeros(max(2 * n - 1, 1), np.int32)
    assert load().orc_karras(_p(k), n, _p(children), _p(parents)) == 0
    return children[:max(n - 1, 0)], parents[:max(2 * n - 1, 0)]


def refit(leaf_boxes, order, children):
    b = np.ascontiguousarray(leaf_boxes, np.float32)
    o = np.ascontiguousarray(order, np.uint32)
    ch = np.ascontiguousarray(children, np.int32)
    n = o.size
    dim = b.shape[1] // 2
    boxes = np.zeros((max(n - 1, 1), 2 * dim), np.float32)
    assert load().orc_refit(dim, _p(b), _p(o), n, _p(ch) if ch.size else None, _p(boxes)) == 0
    return boxes[:max(n - 1, 0)]


def locate(leaf_boxes, order, points) -> np.ndarray:
    b = np.ascontiguousarray(leaf_boxes, np.float32)
    o = np.ascontiguousarray(order, np.uint32)
    pts = np.ascontiguousarray(points, np.float32)
    m = pts.shape[0]
    out = np.zeros(max(m, 1), np.int32)
    assert load().orc_locate(b.shape[1] // 2, _p(b), _p(o), o.size, _p(pts), m, _p(out)) == 0
    return out[:m]


# ---- the reference's own kernels (patched copy built into oracle/_ref) ---------------
class RefGrid:
    """mdas::KDGrid of the reference, driven through oracle/ref_harness.cu (GPU)."""

    _lib = None

    @classmethod
    def available(cls) -> bool:
        return os.path.exists(REF_LIB)

    @classmethod
    def lib(cls):
        if cls._lib is None:
            lib = C.CDLL(REF_LIB)
            sig = {
                "ref_create": (_P, [_I, _I, _I, _I, _I, _F, _F, _F]),
                "ref_destroy": (_I, [_P]),
                "ref_sync": (_I, []),
                "ref_initial_sampling": (_I, [_P]),
                "ref_compute_errors": (_I, [_P]),
                "ref_adaptive_sampling": (_I, [_P]),
                "ref_initial_sampling_async": (_I, [_P]),
                "ref_compute_errors_async": (_I, [_P]),
                "ref_adaptive_sampling_async": (_I, [_P]),
                "ref_adaptive_sampling_kernel_timed": (_I, [_P, C.POINTER(_F)]),
                "ref_integrate_async": (_I, [_P, _P, _I, _I]),
                "ref_integrate": (_I, [_P, _P, _I, _I]),
                "ref_convert_to_bytes": (_I, [_P, _P, _P, _I, _I]),
                "ref_sampling_density": (_I, [_P, _P, _I, _I]),
                "ref_get_counts": (_I, [_P, C.POINTER(_I), C.POINTER(_I), C.POINTER(_I), C.POINTER(_I)]),
                "ref_set_counts": (_I, [_P, _I, _I]),
                "ref_get_gerror": (_F, []),
                "ref_ptr": (_P, [_P, _I]),
                "ref_set_log": (_I, [_P, C.c_char_p]),
            }
            for name, (res, args) in sig.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            cls._lib = lib
        return cls._lib

    def __init__(self, dim, maxSamples, candidatesNum, bitsPerDim, extraImgBits, alpha, scaleX, scaleY):
        self.dim = dim
        self.maxSamples = maxSamples
        self.h = self.lib().ref_create(dim, maxSamples, candidatesNum, bitsPerDim, extraImgBits, float(alpha),
                                       float(scaleX), float(scaleY))
        assert self.h

    def close(self):
        if self.h:
            self.lib().ref_destroy(self.h)
            self.h = None

    def counts(self):
        a, b, c, d = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        self.lib().ref_get_counts(self.h, C.byref(a), C.byref(b), C.byref(c), C.byref(d))
        return a.value, b.value, c.value, d.value

    def ptr(self, which: int) -> int:
        return self.lib().ref_ptr(self.h, which)

    def _view(self, which, count, cols, dtype):
        n = count * cols
        buf = (C.c_byte * (n * np.dtype(dtype).itemsize)).from_address(self.ptr(which))
        return np.frombuffer(buf, dtype=dtype, count=n).reshape(count, cols) if cols > 1 else \
            np.frombuffer(buf, dtype=dtype, count=n)

    def dump_state(self) -> dict:
        self.lib().ref_sync()
        n, _, l, _ = self.counts()
        d = self.dim
        return dict(N=n, L=l, coords=self._view(0, n, d, np.float32).copy(),
                    values=self._view(1, n, 3, np.float32).copy(), nodes=self._view(2, l, 4, np.int32).copy(),
                    boxes=self._view(3, l, 2 * d, np.float32).copy(), errors=self._view(4, l, 1, np.float32).copy(),
                    seeds=self._view(5, l, 1, np.uint32).copy())

    def load_state(self, st: dict):
        self.lib().ref_sync()
        n, l, d = int(st["N"]), int(st["L"]), self.dim
        self._view(0, n, d, np.float32)[:] = st["coords"]
        self._view(1, n, 3, np.float32)[:] = st["values"]
        self._view(2, l, 4, np.int32)[:] = st["nodes"]
        self._view(3, l, 2 * d, np.float32)[:] = st["boxes"]
        self._view(4, l, 1, np.float32)[:] = st["errors"]
        seeds = self._view(5, self.maxSamples, 1, np.uint32)
        seeds[:] = 0
        seeds[:l] = st["seeds"]
        self.lib().ref_set_counts(self.h, n, l)

    def initial_sampling(self):
        assert self.lib().ref_initial_sampling(self.h) == 0

    def compute_errors(self):
        assert self.lib().ref_compute_errors(self.h) == 0
        return np.float32(self.lib().ref_get_gerror())

    def adaptive_sampling(self):
        assert self.lib().ref_adaptive_sampling(self.h) == 0
        return self.counts()
