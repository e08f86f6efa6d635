"""ctypes binding of the native library ``_lib/libfuzzy_ellipses.so`` (C ABI: include/fuzzy_ellipses.h).

The library is built in-tree by ``fuzzy-ellipses_gb300/build.py``. There is no fallback: if the
library is missing, every render entry point raises ``NativeLibraryMissing``.
"""

from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libfuzzy_ellipses.so")

FE_DESC_MAGIC = 0x31644546
FE_DESC_VERSION = 1
FE_PIXLIST_DESC_VERSION = 2
FE_RAYS_POSE_INDEXED = 0
FE_RAYS_QUAT_CAM = 1
FE_CULL_EPS = 0
FE_CULL_NSTD = 1
FE_DEVERR_CAPACITY = 1
FE_DEVERR_TIMEOUT = 2
FE_FLAG_EXACT_KEYS = 2
FE_FLAG_KEEP_BINNING = 4
FE_FLAG_RADIX_BINNING = 8
FE_FLAG_HEAVY_TILES_FIRST = 0x10000
FE_FLAG_RECT_BINNING = 0x20000
FE_VIEW_NO_GRAD = 1
FE_ERR_OUT_OF_MEMORY = 4


def flag_chunk(pairs):
    return (int(pairs) & 0xFF) << 8

STATUS_NAMES = {
    0: "FE_OK", 1: "FE_ERR_INVALID_ARGUMENT", 2: "FE_ERR_DESCRIPTOR", 3: "FE_ERR_CUDA",
    4: "FE_ERR_OUT_OF_MEMORY", 5: "FE_ERR_CAPACITY", 6: "FE_ERR_DEVICE_TIMEOUT",
    7: "FE_ERR_UNSUPPORTED", 8: "FE_ERR_SCRATCH_LIMIT",
}


class NativeLibraryMissing(ImportError):
    pass


class FEError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class RenderDesc(ctypes.Structure):
    """Mirror of ``fe_render_desc``."""
    _fields_ = [
        ("magic", ctypes.c_uint32), ("version", ctypes.c_uint32),
        ("n_gaussians", ctypes.c_int32), ("height", ctypes.c_int32), ("width", ctypes.c_int32),
        ("fx", ctypes.c_float), ("fy", ctypes.c_float), ("cx", ctypes.c_float), ("cy", ctypes.c_float),
        ("beta2", ctypes.c_float), ("beta3", ctypes.c_float),
        ("cull_mode", ctypes.c_int32), ("cull_param", ctypes.c_float),
        ("tile_w", ctypes.c_int32), ("tile_h", ctypes.c_int32),
        ("flags", ctypes.c_uint32), ("px_per_thread", ctypes.c_int32),
    ]


class LegacyDesc(ctypes.Structure):
    """Mirror of ``fe_legacy_desc`` (byte-compatible with the reference's RasterizeDescriptor,
    rasterize_main.h:14-20)."""
    _fields_ = [("image_height", ctypes.c_int32), ("image_width", ctypes.c_int32),
                ("P", ctypes.c_int32), ("tan_fovx", ctypes.c_float), ("tan_fovy", ctypes.c_float)]


class View(ctypes.Structure):
    """Mirror of ``fe_view``."""
    _fields_ = [("scene", ctypes.c_int32), ("height", ctypes.c_int32), ("width", ctypes.c_int32),
                ("fx", ctypes.c_float), ("fy", ctypes.c_float), ("cx", ctypes.c_float),
                ("cy", ctypes.c_float), ("quat", ctypes.c_float * 4), ("trans", ctypes.c_float * 3),
                ("flags", ctypes.c_uint32), ("pixel_offset", ctypes.c_int64)]


# numpy mirror of fe_view: a structured array of this dtype is passed to the library as is.
VIEW_DTYPE = np.dtype(View)


class SceneEntry(ctypes.Structure):
    """Mirror of ``fe_scene``."""
    _fields_ = [("gauss_offset", ctypes.c_int64), ("n", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class PixlistDesc(ctypes.Structure):
    """Mirror of ``fe_pixlist_desc``."""
    _fields_ = [("magic", ctypes.c_uint32), ("version", ctypes.c_uint32),
                ("n_gaussians", ctypes.c_int32), ("n_poses", ctypes.c_int32),
                ("n_rays", ctypes.c_int64), ("inv_f", ctypes.c_float), ("beta2", ctypes.c_float),
                ("beta3", ctypes.c_float), ("cull_mode", ctypes.c_int32),
                ("cull_param", ctypes.c_float), ("n_features", ctypes.c_int32),
                ("ray_mode", ctypes.c_int32), ("aspect", ctypes.c_float),
                ("shift_x", ctypes.c_float), ("shift_y", ctypes.c_float)]


class ServerConfig(ctypes.Structure):
    """Mirror of ``fe_server_config``."""
    _fields_ = [("lanes", ctypes.c_int32), ("max_batch_views", ctypes.c_int32),
                ("max_batch_pixels", ctypes.c_int64), ("hbm_budget_bytes", ctypes.c_int64),
                ("desc", RenderDesc)]


class Request(ctypes.Structure):
    """Mirror of ``fe_request``."""
    _fields_ = [("n_gaussians", ctypes.c_int32), ("n_views", ctypes.c_int32),
                ("means", ctypes.c_void_p), ("prec", ctypes.c_void_p), ("logw", ctypes.c_void_p),
                ("views", ctypes.c_void_p), ("targets", ctypes.c_void_p),
                ("depth", ctypes.c_void_p), ("alpha", ctypes.c_void_p),
                ("grad_means", ctypes.c_void_p), ("grad_prec", ctypes.c_void_p),
                ("grad_logw", ctypes.c_void_p), ("loss", ctypes.c_void_p),
                ("user_tag", ctypes.c_uint64)]


class Completion(ctypes.Structure):
    """Mirror of ``fe_completion``."""
    _fields_ = [("id", ctypes.c_uint64), ("user_tag", ctypes.c_uint64), ("status", ctypes.c_int32),
                ("n_views", ctypes.c_int32), ("submitted_s", ctypes.c_double),
                ("started_s", ctypes.c_double), ("finished_s", ctypes.c_double),
                ("message", ctypes.c_char * 160)]


class ServerStats(ctypes.Structure):
    """Mirror of ``fe_server_stats``."""
    _fields_ = [("submitted", ctypes.c_int64), ("completed", ctypes.c_int64),
                ("renders", ctypes.c_int64), ("batches", ctypes.c_int64),
                ("queued", ctypes.c_int64), ("p50_latency_s", ctypes.c_double),
                ("p99_latency_s", ctypes.c_double), ("busy_s", ctypes.c_double),
                ("phase_s", ctypes.c_double * 6)]


P = ctypes.c_void_p
I32 = ctypes.c_int32
I64 = ctypes.c_int64
F32 = ctypes.c_float

# name -> (restype, argtypes); every symbol the public header declares.
PROTOTYPES = {
    "fe_version": (ctypes.c_char_p, []),
    "fe_last_error_message": (ctypes.c_char_p, []),
    "fe_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "fe_render_desc_init": (None, [ctypes.POINTER(RenderDesc), I32, I32, I32, F32, F32, F32, F32]),
    "fe_render_fwd": (ctypes.c_int, [ctypes.POINTER(RenderDesc)] + [P] * 8 + [P]),
    "fe_render_fwd_noalloc": (ctypes.c_int, [ctypes.POINTER(RenderDesc)] + [P] * 9 + [P]),
    "fe_render_features": (ctypes.c_int, [ctypes.POINTER(RenderDesc)] + [P] * 7 + [I32, P, P]),
    "fe_silhouette_bce": (ctypes.c_int, [P, P, P, I32, I64, P, P, P]),
    "fe_gmm_log_likelihood": (ctypes.c_int, [P, P, P, I32, P, I64, P, P, P, P]),
    "fe_pixlist_desc_init": (None, [ctypes.POINTER(PixlistDesc), I32, I32, I64, F32]),
    "fe_render_pixels": (ctypes.c_int, [ctypes.POINTER(PixlistDesc)] + [P] * 12 + [P]),
    "fe_prec_from_scale_rot": (ctypes.c_int, [P, P, I64, P, P]),
    "fe_prec_from_scale_rot_bwd": (ctypes.c_int, [P, P, I64, P, P, P, P]),
    "fe_transform_points": (ctypes.c_int, [P, I64, P, I32, P, P]),
    "fe_transform_points_bwd": (ctypes.c_int, [P, I64, P, I32, P, P, P, P]),
    "fe_render_bwd": (ctypes.c_int, [ctypes.POINTER(RenderDesc)] + [P] * 13 + [P]),
    "fe_render_binning": (ctypes.c_int, [ctypes.POINTER(RenderDesc)] + [P] * 6 + [I64, P,
                                                                                ctypes.POINTER(I64), P]),
    "fe_render_fwd_xla": (None, [P, P, P, ctypes.c_size_t, P]),
    "fe_render_bwd_xla": (None, [P, P, P, ctypes.c_size_t, P]),
    "fe_rasterize_legacy_xla": (None, [P, P, P, ctypes.c_size_t, P]),
    "fe_rasterize_legacy": (ctypes.c_int, [ctypes.POINTER(LegacyDesc)] + [P] * 11 + [P]),
    "fe_reference_binning": (ctypes.c_int, [I32, I32, I32, F32, P, P, P, P, P, F32, F32,
                                            P, P, P, P, I64, P, ctypes.POINTER(I64), P]),
    "fe_batch_create": (ctypes.c_int, [ctypes.POINTER(RenderDesc), ctypes.POINTER(SceneEntry), I32,
                                       ctypes.POINTER(View), I32, ctypes.POINTER(P)]),
    "fe_batch_destroy": (None, [P]),
    "fe_batch_reset": (ctypes.c_int, [P, ctypes.POINTER(SceneEntry), I32, ctypes.POINTER(View), I32, P]),
    "fe_batch_pixels": (I64, [P]),
    "fe_batch_scratch_bytes": (I64, [P]),
    "fe_batch_fwd": (ctypes.c_int, [P] + [P] * 6 + [P]),
    "fe_batch_fwd_host": (ctypes.c_int, [P] + [P] * 5 + [P]),
    "fe_batch_bwd": (ctypes.c_int, [P] + [P] * 11 + [P]),
    "fe_batch_status": (ctypes.c_int, [P, P, ctypes.POINTER(I64), ctypes.POINTER(I64),
                                       ctypes.POINTER(ctypes.c_uint32)]),
    "fe_check_device_status": (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_uint32)]),
    "fe_batch_fwd_timed": (ctypes.c_int, [P] + [P] * 6 + [ctypes.POINTER(ctypes.c_float), P]),
    "fe_batch_launch_count": (ctypes.c_int, [P]),
    "fe_bench_peak": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double), P]),
    "fe_selftest_bounded_wait": (ctypes.c_int, [ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint32),
                                                ctypes.POINTER(ctypes.c_uint64), P]),
    "fe_server_config_init": (None, [ctypes.POINTER(ServerConfig)]),
    "fe_server_create": (ctypes.c_int, [ctypes.POINTER(ServerConfig), ctypes.c_int, ctypes.POINTER(P)]),
    "fe_server_submit": (ctypes.c_int, [P, ctypes.POINTER(Request), ctypes.POINTER(ctypes.c_uint64)]),
    "fe_server_wait": (ctypes.c_int, [P, ctypes.POINTER(Completion), I32, I32, ctypes.POINTER(I32)]),
    "fe_server_stats_get": (ctypes.c_int, [P, ctypes.POINTER(ServerStats)]),
    "fe_server_stats_reset": (None, [P]),
    "fe_server_close": (ctypes.c_int, [P]),
    "fe_server_destroy": (None, [P]),
    "fe_request_footprint": (I64, [ctypes.POINTER(Request), I32, I32]),
}

_lib = None
_lock = threading.Lock()


def load(path: str | None = None):
    """Load (once) and return the native library; raises NativeLibraryMissing if absent."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise NativeLibraryMissing(
                f"{p} is missing: build it with `python fuzzy-ellipses_gb300/build.py` "
                "(or __graft_entry__.build()); there is no non-CUDA fallback")
        lib = ctypes.CDLL(p)
        for name, (res, args) in PROTOTYPES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(status: int):
    if status != 0:
        msg = load().fe_last_error_message().decode(errors="replace")
        raise FEError(status, msg)


def make_desc(n, height, width, fx, fy, cx, cy, beta2=21.4, beta3=2.66, cull="eps",
              cull_param=None, tile=(16, 16), flags=0, px=0) -> RenderDesc:
    d = RenderDesc()
    load().fe_render_desc_init(ctypes.byref(d), int(n), int(height), int(width), float(fx),
                               float(fy), float(cx), float(cy))
    d.beta2 = float(beta2)
    d.beta3 = float(beta3)
    if cull == "eps":
        d.cull_mode = FE_CULL_EPS
        d.cull_param = 1e-7 if cull_param is None else float(cull_param)
    elif cull == "nstd":
        d.cull_mode = FE_CULL_NSTD
        d.cull_param = 3.0 if cull_param is None else float(cull_param)
    else:
        raise ValueError("cull must be 'eps' or 'nstd'")
    d.tile_w, d.tile_h = int(tile[0]), int(tile[1])
    d.flags = int(flags)
    d.px_per_thread = int(px)
    return d
