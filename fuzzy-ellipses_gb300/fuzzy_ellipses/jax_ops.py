"""JAX binding of the render path: the library's XLA custom-call targets behind ``jax.custom_vjp``.

The reference registers its CUDA custom call from a pybind capsule (``ext.cpp:23-33``,
``fuzzy_ellipses/__init__.py:22-23``) and lowers ``rasterize`` to it
(``fuzzy_ellipses/__init__.py:111-166``). This module does the same for this library's targets:
``fe_render_fwd_xla`` / ``fe_render_bwd_xla`` (api_version 2, status-returning; the opaque payload
is an ``fe_render_desc``) and the reference-signature ``fe_rasterize_legacy_xla``, and defines
``render`` as a ``jax.custom_vjp`` whose backward is the library's recompute backward.

Importing this module requires JAX with the ``jax.ffi`` API (``register_ffi_target`` with
``api_version=0`` for classic custom calls and ``ffi_call`` with ``custom_call_api_version`` /
``legacy_backend_config``); without JAX it raises ImportError with that reason. JAX is not
installed on the machines this package was built and tested on, so this module has not been
executed there.
"""

from __future__ import annotations

import ctypes

try:
    import jax
    import jax.numpy as jnp
    from jax import ffi as _ffi
except ImportError as e:  # pragma: no cover - depends on the environment
    raise ImportError(f"fuzzy_ellipses.jax_ops needs JAX with jax.ffi: {e}") from e

import numpy as np

from . import _native as N

__all__ = ["register", "render", "rasterize"]

_REGISTERED = False
_TARGETS = {"fe_render_fwd": "fe_render_fwd_xla", "fe_render_bwd": "fe_render_bwd_xla",
            "rasterize_gaussians_fwd": "fe_rasterize_legacy_xla"}


def _capsule(fn):
    make = ctypes.pythonapi.PyCapsule_New
    make.restype = ctypes.py_object
    make.argtypes = (ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p)
    return make(ctypes.cast(fn, ctypes.c_void_p).value, b"xla._CUSTOM_CALL_TARGET", None)


def register():
    """Register the library's targets with XLA for the CUDA platform (once)."""
    global _REGISTERED
    if _REGISTERED:
        return
    lib = N.load()
    for name, symbol in _TARGETS.items():
        _ffi.register_ffi_target(name, _capsule(getattr(lib, symbol)), platform="CUDA",
                                 api_version=0)
    _REGISTERED = True


def _desc_bytes(n, height, width, fx, fy, cx, cy, beta2, beta3, cull, cull_param, tile):
    d = N.make_desc(n, height, width, fx, fy, cx, cy, beta2, beta3, cull, cull_param, tile)
    return bytes(d)


def _fwd_call(opaque, means, prec, logw, quat, t, height, width):
    f32 = jnp.float32
    out = (jax.ShapeDtypeStruct((height, width), f32), jax.ShapeDtypeStruct((height, width), f32),
           jax.ShapeDtypeStruct((3, height, width), f32))
    call = _ffi.ffi_call("fe_render_fwd", out, custom_call_api_version=2,
                         legacy_backend_config=opaque)
    return call(means, prec, logw, quat, t)


def _bwd_call(opaque, means, prec, logw, quat, t, depth, alpha, stats, g_depth, g_alpha):
    f32 = jnp.float32
    n = means.shape[0]
    out = (jax.ShapeDtypeStruct((n, 3), f32), jax.ShapeDtypeStruct((n, 3, 3), f32),
           jax.ShapeDtypeStruct((n,), f32))
    call = _ffi.ffi_call("fe_render_bwd", out, custom_call_api_version=2,
                         legacy_backend_config=opaque)
    return call(means, prec, logw, quat, t, depth, alpha, stats, g_depth, g_alpha)


def render(means, prec, logw, fx, fy, cx, cy, quat, t, height, width, beta2=21.4, beta3=2.66, *,
           cull="eps", cull_param=None, tile=(16, 16)):
    """Depth and alpha (H, W) of one pinhole camera, differentiable in means (N,3), prec (N,3,3)
    (upper triangle read; Sigma^-1 = U U^T, fm_render's prec_full) and logw (N,). Camera
    intrinsics, pose and sizes are static."""
    register()
    means = jnp.asarray(means, jnp.float32)
    prec = jnp.asarray(prec, jnp.float32)
    logw = jnp.asarray(logw, jnp.float32)
    quat = jnp.asarray(quat, jnp.float32).reshape(4)
    t = jnp.asarray(t, jnp.float32).reshape(3)
    opaque = _desc_bytes(means.shape[0], height, width, fx, fy, cx, cy, beta2, beta3, cull,
                         cull_param, tile)

    @jax.custom_vjp
    def _render(m, p, w):
        d, a, _ = _fwd_call(opaque, m, p, w, quat, t, height, width)
        return d, a

    def _fwd(m, p, w):
        d, a, stats = _fwd_call(opaque, m, p, w, quat, t, height, width)
        return (d, a), (m, p, w, d, a, stats)

    def _bwd(res, cot):
        m, p, w, d, a, stats = res
        gd, ga = cot
        return _bwd_call(opaque, m, p, w, quat, t, d, a, stats, gd.astype(jnp.float32),
                         ga.astype(jnp.float32))

    _render.defvjp(_fwd, _bwd)
    return _render(means, prec, logw)


def rasterize(means3D, scales, rotations, weights, camera_rays, camera_rot, camera_trans,
              viewmatrix, projmatrix, image_height, image_width, tan_fovx, tan_fovy):
    """The reference's ``rasterize`` operand list (``fuzzy_ellipses/__init__.py:136-146``)
    through ``fe_rasterize_legacy_xla``: returns (z, alpha) of shape (H, W), forward only."""
    register()
    P = int(np.shape(means3D)[0])
    opaque = bytes(N.LegacyDesc(int(image_height), int(image_width), P, float(tan_fovx),
                                float(tan_fovy)))
    f32 = jnp.float32
    out = (jax.ShapeDtypeStruct((image_height, image_width), f32),
           jax.ShapeDtypeStruct((image_height, image_width), f32))
    call = _ffi.ffi_call("rasterize_gaussians_fwd", out, custom_call_api_version=2,
                         legacy_backend_config=opaque)
    args = [jnp.asarray(x, f32) for x in (means3D, weights, scales, rotations, camera_rays,
                                           camera_rot, camera_trans, viewmatrix, projmatrix)]
    return call(*args)
