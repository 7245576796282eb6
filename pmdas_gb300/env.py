"""The `.env` configuration surface (``Sampler { mdas, samples }``,
``Mdas { scaleFactor, alpha, bitsPerDim, extraImgBits, candidatesNum }``,
``Film``, ``Camera`` ...) parsed by the library's C++ reader, which follows the
reference's Environment rules (SDK/sutil/Environment.cpp)."""
from __future__ import annotations

import ctypes as C

from . import _native as N

FIELDS = [f for f, _ in N.Config._fields_]


def _to_dict(cfg: N.Config) -> dict:
    d = {f: getattr(cfg, f) for f in FIELDS}
    d["filmFilename"] = cfg.filmFilename.decode()
    return d


def defaults() -> dict:
    cfg = N.Config()
    N.check(N.load().mdas_config_defaults(C.byref(cfg)), "mdas_config_defaults")
    return _to_dict(cfg)


def read_env(path: str) -> dict:
    """Parse an .env file; raises ValueError with the reader's message on error."""
    cfg = N.Config()
    err = C.create_string_buffer(512)
    rc = N.load().mdas_config_read(path.encode(), C.byref(cfg), err, 512)
    if rc != N.MDAS_OK:
        raise ValueError(err.value.decode() or N.status_string(rc))
    return _to_dict(cfg)
