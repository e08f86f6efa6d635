"""ctypes wrapper of oracle/ref_binning.c, the CPU restatement of the reference CUDA rasterizer's
binning (TEST INFRASTRUCTURE ONLY). Built by ``make -C oracle lib``."""

from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_build", "libref_binning.so")
_lib = None


def build():
    subprocess.run(["make", "-s", "-C", _HERE, "lib"], check=True)
    return _LIB


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB):
            build()
        lib = ctypes.CDLL(_LIB)
        f = lib.ref_binning
        f.restype = ctypes.c_int64
        f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float] + [ctypes.c_void_p] * 5 + \
            [ctypes.c_float, ctypes.c_float] + [ctypes.c_void_p] * 4 + [ctypes.c_int64, ctypes.c_void_p]
        _lib = lib
    return _lib


def _f32(a, n):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(-1))
    assert a.size == n, (a.size, n)
    return a


def ref_binning(means, scales, rots, view, proj, height, width, tan_fovx, tan_fovy, n_std):
    """Returns dict(radii, means2d, tiles_touched (inclusive), keys (sorted uint64), ranges (T,2))."""
    lib = _load()
    P = int(np.asarray(means).reshape(-1, 3).shape[0])
    m, s, r = _f32(means, 3 * P), _f32(scales, 3 * P), _f32(rots, 4 * P)
    v, pj = _f32(view, 16), _f32(proj, 16)
    gx, gy = (width + 7) // 8, (height + 7) // 8
    T = gx * gy
    radii = np.zeros(max(P, 1), np.int32)
    means2d = np.zeros(2 * max(P, 1), np.float32)
    touched = np.zeros(max(P, 1), np.uint32)
    ranges = np.zeros(2 * T, np.uint32)
    cap = 1 << 16
    while True:
        keys = np.zeros(cap, np.uint64)
        k = lib.ref_binning(P, int(height), int(width), float(n_std), m.ctypes.data, s.ctypes.data,
                            r.ctypes.data, v.ctypes.data, pj.ctypes.data, float(tan_fovx),
                            float(tan_fovy), radii.ctypes.data, means2d.ctypes.data,
                            touched.ctypes.data, keys.ctypes.data, cap, ranges.ctypes.data)
        if k == -1:
            cap = int(touched[P - 1]) + 1
            continue
        if k < 0:
            raise MemoryError("ref_binning failed")
        break
    return {"radii": radii[:P], "means2d": means2d[:2 * P].reshape(P, 2), "tiles_touched": touched[:P],
            "keys": keys[:k], "ranges": ranges.reshape(T, 2), "num_keys": int(k)}
