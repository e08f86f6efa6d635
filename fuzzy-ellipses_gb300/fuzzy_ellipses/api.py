"""torch-facing render API over the native C ABI.

``render`` is the drop-in for the reference's render entry point, re-specified as in
``baseline/fm_render.py:113-126`` (``render_func_quat``): precision factor in fm_render's
``prec_full`` convention, camera given by pinhole intrinsics and a (quaternion, translation) pose.
It is differentiable with respect to means, precisions and log-weights through a
``torch.autograd.Function`` whose backward is the native recompute-based backward kernel.

``rasterize`` mirrors the reference's legacy ``fuzzy_ellipses.rasterize``
(``fuzzy_ellipses/__init__.py:189-236``): same arguments, same conventions (full-angle
``tan_fov``, identity view matrix, ``getNumStds`` cut-off, 8x8 tiles), same
``nan_to_num`` post-processing.

All work is enqueued on torch's current CUDA stream; there is no CPU path.
"""

from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import _native as N

__all__ = ["render", "render_forward", "render_binning", "rasterize", "reference_binning", "Batch", "bench_peak",
           "projection_matrix", "reference_num_stds", "device_status"]


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


def _as_dev(x, device, shape=None, name="tensor"):
    if not torch.is_tensor(x):
        x = torch.as_tensor(np.asarray(x, dtype=np.float32))
    x = x.to(device=device, dtype=torch.float32).contiguous()
    if shape is not None and tuple(x.shape) != tuple(shape):
        x = x.reshape(shape)
    return x


def _check_inputs(means, prec, logw):
    if not (torch.is_tensor(means) and means.is_cuda):
        raise TypeError("means must be a CUDA tensor (the renderer has no CPU path)")
    n = means.shape[0]
    if means.shape != (n, 3) or prec.shape != (n, 3, 3) or logw.shape != (n,):
        raise ValueError(f"expected means (N,3), prec (N,3,3), logw (N,); got {tuple(means.shape)}, "
                         f"{tuple(prec.shape)}, {tuple(logw.shape)}")
    return n


class _RenderFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, means, prec, logw, quat, trans, desc):
        lib = N.load()
        dev = means.device
        means = means.detach().contiguous().float()
        prec = prec.detach().contiguous().float()
        logw = logw.detach().contiguous().float()
        H, W = desc.height, desc.width
        depth = torch.empty((H, W), device=dev, dtype=torch.float32)
        alpha = torch.empty((H, W), device=dev, dtype=torch.float32)
        need = any(ctx.needs_input_grad[:3])
        stats = torch.empty((3, H, W), device=dev, dtype=torch.float32) if need else None
        N.check(lib.fe_render_fwd(ctypes.byref(desc), _ptr(means), _ptr(prec), _ptr(logw),
                                  _ptr(quat), _ptr(trans), _ptr(depth), _ptr(alpha), _ptr(stats),
                                  _stream()))
        ctx.desc = desc
        if need:
            ctx.save_for_backward(means, prec, logw, quat, trans, depth, alpha, stats)
        return depth, alpha

    @staticmethod
    def backward(ctx, gdepth, galpha):
        lib = N.load()
        means, prec, logw, quat, trans, depth, alpha, stats = ctx.saved_tensors
        gm = torch.empty_like(means)
        gp = torch.empty_like(prec)
        gw = torch.empty_like(logw)
        gd = gdepth.contiguous().float() if gdepth is not None else None
        ga = galpha.contiguous().float() if galpha is not None else None
        N.check(lib.fe_render_bwd(ctypes.byref(ctx.desc), _ptr(means), _ptr(prec), _ptr(logw),
                                  _ptr(quat), _ptr(trans), _ptr(depth), _ptr(alpha), _ptr(stats),
                                  _ptr(gd), _ptr(ga), _ptr(gm), _ptr(gp), _ptr(gw), _stream()))
        return gm, gp, gw, None, None, None


def render(means, prec, logw, fx, fy, cx, cy, quat, t, height, width, beta2=21.4, beta3=2.66, *,
           cull="eps", cull_param=None, tile=(16, 16)):
    """Render depth and alpha (H, W) of one pinhole camera; differentiable in means/prec/logw.

    means (N,3), prec (N,3,3) (upper triangle read, precision U U^T), logw (N,): CUDA float32.
    quat (4,) scalar-first and t (3,): camera rotation (rays_world = rays_cam @ quat_to_rot(quat))
    and centre. ``cull='eps'`` drops a Gaussian where its peak density along a ray is below
    ``cull_param`` (default 1e-7); ``cull='nstd'`` uses a fixed ``cull_param`` sigma radius.
    """
    n = _check_inputs(means, prec, logw)
    dev = means.device
    q = _as_dev(quat, dev, (4,))
    tt = _as_dev(t, dev, (3,))
    desc = N.make_desc(n, height, width, fx, fy, cx, cy, beta2, beta3, cull, cull_param, tile)
    return _RenderFn.apply(means, prec, logw, q, tt, desc)


def render_forward(means, prec, logw, fx, fy, cx, cy, quat, t, height, width, beta2=21.4,
                   beta3=2.66, *, cull="eps", cull_param=None, tile=(16, 16), out=None,
                   stats=None, binning="tiles"):
    """Non-differentiable forward into optional preallocated ``out=(depth, alpha)``."""
    lib = N.load()
    n = _check_inputs(means, prec, logw)
    dev = means.device
    q = _as_dev(quat, dev, (4,))
    tt = _as_dev(t, dev, (3,))
    desc = N.make_desc(n, height, width, fx, fy, cx, cy, beta2, beta3, cull, cull_param, tile,
                       flags=_binning_flag(binning))
    if out is None:
        out = (torch.empty((height, width), device=dev), torch.empty((height, width), device=dev))
    N.check(lib.fe_render_fwd(ctypes.byref(desc), _ptr(means), _ptr(prec), _ptr(logw), _ptr(q),
                              _ptr(tt), _ptr(out[0]), _ptr(out[1]), _ptr(stats), _stream()))
    return out


def render_features(means, prec, logw, features, fx, fy, cx, cy, quat, t, height, width,
                    beta2=21.4, beta3=2.66, *, cull="eps", cull_param=None, tile=(16, 16)):
    """Depth, alpha (H, W) and the softmax-weighted features (H, W, F) of one pinhole camera:
    feature(pixel) = sum_i w_i f_i with fm_render's normalised weights w (fm_render.py:95-109).
    ``features`` (N, F) float32. Forward only."""
    lib = N.load()
    n = _check_inputs(means, prec, logw)
    dev = means.device
    feats = features.to(device=dev, dtype=torch.float32).contiguous()
    if feats.dim() != 2 or feats.shape[0] != n or feats.shape[1] < 1:
        raise ValueError("features must be (N, F) with F >= 1")
    q = _as_dev(quat, dev, (4,))
    tt = _as_dev(t, dev, (3,))
    desc = N.make_desc(n, height, width, fx, fy, cx, cy, beta2, beta3, cull, cull_param, tile)
    depth = torch.empty((height, width), device=dev)
    alpha = torch.empty((height, width), device=dev)
    stats = torch.empty((3, height, width), device=dev)
    out = torch.empty((height, width, feats.shape[1]), device=dev)
    N.check(lib.fe_render_fwd(ctypes.byref(desc), _ptr(means), _ptr(prec), _ptr(logw), _ptr(q),
                              _ptr(tt), _ptr(depth), _ptr(alpha), _ptr(stats), _stream()))
    N.check(lib.fe_render_features(ctypes.byref(desc), _ptr(means), _ptr(prec), _ptr(logw),
                                   _ptr(q), _ptr(tt), _ptr(stats), _ptr(feats), feats.shape[1],
                                   _ptr(out), _stream()))
    return depth, alpha, out


def _binning_flag(binning, footprint="ellipse"):
    if binning not in ("tiles", "radix"):
        raise ValueError("binning must be 'tiles' or 'radix'")
    if footprint not in ("ellipse", "rect"):
        raise ValueError("footprint must be 'ellipse' or 'rect'")
    return ((N.FE_FLAG_RADIX_BINNING if binning == "radix" else 0)
            | (N.FE_FLAG_RECT_BINNING if footprint == "rect" else 0))


def render_binning(means, prec, logw, fx, fy, cx, cy, quat, t, height, width, *, cull="eps",
                   cull_param=None, tile=(16, 16), key_capacity=None, binning="tiles",
                   footprint="ellipse"):
    """The tile binning ``render`` uses: returns (keys (K,) int64 holding (tile << 32 | gaussian),
    ranges (T, 2) int64). Synchronises once. ``binning="radix"`` forces key emission + radix sort
    instead of the tile-major binning (same result). ``footprint="rect"`` bins each Gaussian to
    every tile of its footprint's bounding rectangle (FE_FLAG_RECT_BINNING) instead of the tiles
    its footprint ellipse reaches in each tile row."""
    lib = N.load()
    n = _check_inputs(means, prec, logw)
    dev = means.device
    q = _as_dev(quat, dev, (4,))
    tt = _as_dev(t, dev, (3,))
    desc = N.make_desc(n, height, width, fx, fy, cx, cy, 21.4, 2.66, cull, cull_param, tile,
                       flags=_binning_flag(binning, footprint))
    gx = (width + tile[0] - 1) // tile[0]
    gy = (height + tile[1] - 1) // tile[1]
    cap = int(key_capacity) if key_capacity is not None else max(1, n * gx * gy)
    keys = torch.empty(cap, dtype=torch.int64, device=dev)
    ranges = torch.empty((gx * gy, 2), dtype=torch.int32, device=dev)
    nk = ctypes.c_int64(0)
    N.check(lib.fe_render_binning(ctypes.byref(desc), _ptr(means), _ptr(prec), _ptr(logw), _ptr(q),
                                  _ptr(tt), _ptr(keys), cap, _ptr(ranges), ctypes.byref(nk),
                                  _stream()))
    return keys[:nk.value], ranges.to(torch.int64) & 0xFFFFFFFF


def silhouette_bce(alpha, target, seg_end, galpha=None, loss=None):
    """Per-render mean silhouette BCE and its alpha cotangent in one kernel.

    ``alpha``/``target``: flat float32 device buffers of the renders stored back to back;
    ``seg_end``: int64 device tensor of each render's end pixel (the last equals alpha's size).
    Returns ``(loss (R,) float64, galpha)`` with galpha = dL_r/dalpha per pixel (the loss of the
    reference's shape-from-silhouette loop, shape_from_silhouette.ipynb cell 12)."""
    lib = N.load()
    n_pix = alpha.numel()
    if target.numel() != n_pix or not (alpha.is_contiguous() and target.is_contiguous()):
        raise ValueError("alpha and target must be contiguous with the same size")
    if alpha.dtype != torch.float32 or target.dtype != torch.float32:
        raise ValueError("alpha and target must be float32")
    if seg_end.dtype != torch.int64 or not seg_end.is_contiguous():
        raise ValueError("seg_end must be a contiguous int64 tensor")
    if galpha is None:
        galpha = torch.empty_like(alpha)
    if loss is None:
        loss = torch.empty(seg_end.numel(), dtype=torch.float64, device=alpha.device)
    N.check(lib.fe_silhouette_bce(_ptr(alpha), _ptr(target), _ptr(seg_end), seg_end.numel(),
                                  n_pix, _ptr(galpha), _ptr(loss), _stream()))
    return loss, galpha


def render_pixels(means, prec, logw, pixel_posei, inv_f, poses, beta2=21.4, beta3=2.66, *,
                  flow=False, weights=False, features=None, cull="eps", cull_param=None):
    """Multi-pose pixel-list render (baseline/fm_render.py:151-224 ``render_func_idx_quattrans``
    and, with ``flow=True``, ``render_func_idx_quattrans_flow``).

    ``pixel_posei`` (P, 4): rows (x, y, c, pose) -- the camera ray is (x inv_f, y inv_f, c) of
    pose ``pose``; ``poses`` (n_poses, 7): quaternion (scalar first) and translation.
    Returns ``(depth, alpha, None, w)`` or, with ``flow=True``, ``(depth, alpha, None, w, flowp,
    flowm)`` as the reference does; ``w`` is the dense (N, P) softmax weight matrix when
    ``weights=True``, else None. With ``features`` (N, F), F <= 16, the softmax-weighted features
    (P, F) are appended to the tuple. Forward only."""
    lib = N.load()
    n = _check_inputs(means, prec, logw)
    dev = means.device
    rays = pixel_posei.to(device=dev, dtype=torch.float32).contiguous()
    ps = poses.to(device=dev, dtype=torch.float32).contiguous()
    if rays.dim() != 2 or rays.shape[1] != 4 or ps.dim() != 2 or ps.shape[1] != 7:
        raise ValueError("pixel_posei must be (P, 4) and poses (n_poses, 7)")
    P = rays.shape[0]
    d = N.PixlistDesc()
    lib.fe_pixlist_desc_init(ctypes.byref(d), n, ps.shape[0], P, float(inv_f))
    d.beta2, d.beta3 = float(beta2), float(beta3)
    if cull == "eps":
        d.cull_mode, d.cull_param = N.FE_CULL_EPS, (1e-7 if cull_param is None else float(cull_param))
    else:
        d.cull_mode, d.cull_param = N.FE_CULL_NSTD, (3.0 if cull_param is None else float(cull_param))
    feats = None
    if features is not None:
        feats = features.to(device=dev, dtype=torch.float32).contiguous()
        if feats.dim() != 2 or feats.shape[0] != n:
            raise ValueError("features must be (N, F)")
        d.n_features = feats.shape[1]
    depth = torch.empty(P, device=dev)
    alpha = torch.empty(P, device=dev)
    fp = torch.empty((P, 2), device=dev) if flow else None
    fm = torch.empty((P, 2), device=dev) if flow else None
    of = torch.empty((P, d.n_features), device=dev) if feats is not None else None
    w = torch.empty((n, P), device=dev) if weights else None
    N.check(lib.fe_render_pixels(ctypes.byref(d), _ptr(means), _ptr(prec), _ptr(logw), _ptr(ps),
                                 _ptr(rays), _ptr(feats), _ptr(depth), _ptr(alpha), _ptr(fp),
                                 _ptr(fm), _ptr(of), _ptr(w), _stream()))
    out = (depth, alpha, None, w) + ((fp, fm) if flow else ())
    return out + ((of,) if feats is not None else ())


def render_pixels_cam(means, prec, logw, pixel_list, aspect, inv_f, quat, t, beta2=21.4,
                      beta3=2.66, *, weights=False, features=None, cull="eps", cull_param=None,
                      shift=(0.5, 0.5)):
    """Pixel-list render of one pose with a single inverse focal length and an aspect ratio
    (baseline/fm_render.py:130-144 ``render_func_quat_cam``).

    ``pixel_list`` (P, 3): rows (x, y, c); the camera ray is ((x - 0.5) inv_f,
    (y - 0.5) aspect inv_f, c), rotated by ``quat_to_rot(quat)`` and starting at ``t``. Returns
    ``(depth, alpha, None, w)`` like the reference (``w`` the dense (N, P) weights when
    ``weights=True``, else None), with the softmax-weighted features (P, F) appended when
    ``features`` (N, F) is given. Forward only."""
    lib = N.load()
    n = _check_inputs(means, prec, logw)
    dev = means.device
    rays = torch.as_tensor(pixel_list).to(device=dev, dtype=torch.float32).contiguous()
    if rays.dim() != 2 or rays.shape[1] != 3:
        raise ValueError("pixel_list must be (P, 3)")
    pose = torch.cat([torch.as_tensor(quat, dtype=torch.float32).reshape(4),
                      torch.as_tensor(t, dtype=torch.float32).reshape(3)]).to(dev).reshape(1, 7)
    P = rays.shape[0]
    d = N.PixlistDesc()
    lib.fe_pixlist_desc_init(ctypes.byref(d), n, 1, P, float(inv_f))
    d.ray_mode = N.FE_RAYS_QUAT_CAM
    d.aspect = float(aspect)
    d.shift_x, d.shift_y = float(shift[0]), float(shift[1])
    d.beta2, d.beta3 = float(beta2), float(beta3)
    if cull == "eps":
        d.cull_mode, d.cull_param = N.FE_CULL_EPS, (1e-7 if cull_param is None else float(cull_param))
    else:
        d.cull_mode, d.cull_param = N.FE_CULL_NSTD, (3.0 if cull_param is None else float(cull_param))
    feats = None
    if features is not None:
        feats = features.to(device=dev, dtype=torch.float32).contiguous()
        if feats.dim() != 2 or feats.shape[0] != n:
            raise ValueError("features must be (N, F)")
        d.n_features = feats.shape[1]
    depth = torch.empty(P, device=dev)
    alpha = torch.empty(P, device=dev)
    of = torch.empty((P, d.n_features), device=dev) if feats is not None else None
    w = torch.empty((n, P), device=dev) if weights else None
    N.check(lib.fe_render_pixels(ctypes.byref(d), _ptr(means), _ptr(prec), _ptr(logw), _ptr(pose),
                                 _ptr(rays), _ptr(feats), _ptr(depth), _ptr(alpha), None, None,
                                 _ptr(of), _ptr(w), _stream()))
    out = (depth, alpha, None, w)
    return out + ((of,) if feats is not None else ())


def gmm_log_likelihood(means, prec, logw, points, *, return_matrix=False):
    """Log-likelihood of points (P, 3) under the mixture (the reference's ``log_likelihood``,
    baseline/fm_render.py:231-259): returns ``(nll, point_ll)`` -- the mean negative
    log-likelihood (float64 scalar tensor, the reference's first output) and the per-point
    log-likelihoods (P,) -- plus, with ``return_matrix=True``, the per-(Gaussian, point) log
    terms (N, P) (the reference's second output)."""
    lib = N.load()
    n = _check_inputs(means, prec, logw)
    if n < 1:
        raise ValueError("need at least one Gaussian")
    if points.dtype != torch.float32 or points.dim() != 2 or points.shape[1] != 3:
        raise ValueError("points must be float32 of shape (P, 3)")
    points = points.contiguous()
    P = points.shape[0]
    dev = means.device
    point_ll = torch.empty(P, device=dev)
    total = torch.empty(1, dtype=torch.float64, device=dev)
    res = torch.empty((n, P), device=dev) if return_matrix else None
    N.check(lib.fe_gmm_log_likelihood(_ptr(means), _ptr(prec), _ptr(logw), n, _ptr(points), P,
                                      _ptr(point_ll), _ptr(res), _ptr(total), _stream()))
    nll = -total[0] / max(P, 1)
    return (nll, point_ll, res) if return_matrix else (nll, point_ll)


def bench_peak(kind):
    """Measured pipe throughput (operations/s): 'fma' (FP32 FMA), 'ex2' (MUFU ex2) or 'fma2'
    (packed f32x2 FMA, two FMAs per instruction)."""
    lib = N.load()
    out = ctypes.c_double(0.0)
    N.check(lib.fe_bench_peak({"fma": 0, "ex2": 1, "fma2": 2}[kind], 4096, ctypes.byref(out), _stream()))
    return float(out.value)


def device_status():
    """Synchronise the current stream and return (and clear) its device error word."""
    lib = N.load()
    err = ctypes.c_uint32(0)
    N.check(lib.fe_check_device_status(_stream(), ctypes.byref(err)))
    return int(err.value)


# ---------------------------------------------------------------------------------------------
# Legacy interface (fuzzy_ellipses/__init__.py:36-76,189-239 of the reference)
# ---------------------------------------------------------------------------------------------

def projection_matrix(width, height, fx, fy, cx, cy, znear, zfar):
    """``getProjectionMatrixJax`` (reference ``fuzzy_ellipses/__init__.py:36-76``): the transposed
    OpenGL-style projection; cx, cy are ignored as in the reference. float64 math, float32 result."""
    fov_x = math.atan(width / 2 / fx) * 2.0
    fov_y = math.atan(height / 2 / fy) * 2.0
    top = math.tan(fov_y / 2) * znear
    bottom = -top
    right = math.tan(fov_x / 2) * znear
    left = -right
    m = np.array([
        [2.0 * znear / (right - left), 0.0, (right + left) / (right - left), 0.0],
        [0.0, 2.0 * znear / (top - bottom), (top + bottom) / (top - bottom), 0.0],
        [0.0, 0.0, zfar / (zfar - znear), -(zfar * znear) / (zfar - znear)],
        [0.0, 0.0, 1.0, 0.0],
    ])
    return m.T.astype(np.float32)


def reference_num_stds(n):
    """``getNumStds`` (reference ``cuda_rasterizer/rasterizer_impl.cu:154-172``)."""
    if n <= 1000:
        return 3.0
    if n <= 5000:
        return 0.75
    if n <= 100000:
        return 0.5
    return 0.1


def _legacy_scalars(image_height, image_width, fx, fy, cx, cy, near, far):
    # fuzzy_ellipses/__init__.py:206-216: tan of the *full* field-of-view angle, identity view.
    tan_fovx = math.tan(math.atan(image_width / 2 / fx) * 2.0)
    tan_fovy = math.tan(math.atan(image_height / 2 / fy) * 2.0)
    view = np.eye(4, dtype=np.float32)
    proj = (view.astype(np.float64) @ projection_matrix(image_width, image_height, fx, fy, cx, cy,
                                                        near, far).astype(np.float64)).astype(np.float32)
    return np.float32(tan_fovx), np.float32(tan_fovy), view, proj


def rasterize(means3D, scales, rotations, weights, camera_rays, camera_rot, camera_trans,
              image_height, image_width, fx, fy, cx, cy, near, far):
    """Reference-signature forward render returning ``(z, alpha)`` of shape (H, W).

    Binning follows the reference exactly (tile keys bit-exact with its CUDA rasterizer); depth
    and alpha come from this library's blend over those tiles, with the precision implied by
    (scales, rotations) and the pinhole rays in ``camera_rays`` rotated by ``camera_rot`` from
    origin ``camera_trans``.
    """
    lib = N.load()
    dev = means3D.device if torch.is_tensor(means3D) and means3D.is_cuda else torch.device("cuda")
    means = _as_dev(means3D, dev)
    P = means.shape[0]
    H, W = int(image_height), int(image_width)
    tfx, tfy, view, proj = _legacy_scalars(H, W, fx, fy, cx, cy, near, far)
    d = N.LegacyDesc(H, W, P, float(tfx), float(tfy))
    bufs = [means, _as_dev(weights, dev), _as_dev(scales, dev), _as_dev(rotations, dev),
            _as_dev(camera_rays, dev), _as_dev(camera_rot, dev), _as_dev(camera_trans, dev),
            _as_dev(view, dev), _as_dev(proj, dev)]
    z = torch.empty((H, W), device=dev)
    alpha = torch.empty((H, W), device=dev)
    N.check(lib.fe_rasterize_legacy(ctypes.byref(d), *[_ptr(b) for b in bufs], _ptr(z), _ptr(alpha),
                                    _stream()))
    z = torch.nan_to_num(z, posinf=10.0, neginf=0.0)        # __init__.py:233
    alpha = torch.nan_to_num(alpha, posinf=1.0, neginf=0.0)  # __init__.py:234
    return z, alpha


def reference_binning(means, scales, rotations, viewmatrix, projmatrix, height, width, tan_fovx,
                      tan_fovy, n_std=None, key_capacity=None):
    """Reference-compatible binning on the GPU. Returns a dict of CUDA tensors:
    radii (P,) int32, means2d (P,2), tiles_touched (P,) uint32-as-int64 inclusive prefix sum,
    keys (K,) uint64-as-int64 sorted, ranges (T,2) int64."""
    lib = N.load()
    dev = means.device if torch.is_tensor(means) and means.is_cuda else torch.device("cuda")
    m = _as_dev(means, dev)
    P = m.shape[0]
    if n_std is None:
        n_std = reference_num_stds(P)
    gx, gy = (width + 7) // 8, (height + 7) // 8
    T = gx * gy
    cap = int(key_capacity) if key_capacity is not None else max(1, P * T)
    radii = torch.zeros(P, dtype=torch.int32, device=dev)
    means2d = torch.zeros((P, 2), dtype=torch.float32, device=dev)
    touched = torch.zeros(P, dtype=torch.int32, device=dev)
    keys = torch.zeros(max(cap, 1), dtype=torch.int64, device=dev)
    ranges = torch.zeros((T, 2), dtype=torch.int32, device=dev)
    nk = ctypes.c_int64(0)
    # Keep every uploaded input referenced until the call has been enqueued: a temporary dropped
    # earlier could hand its memory to the next upload before the kernels read it.
    s_d, r_d = _as_dev(scales, dev), _as_dev(rotations, dev)
    v_d, p_d = _as_dev(viewmatrix, dev), _as_dev(projmatrix, dev)
    N.check(lib.fe_reference_binning(P, int(height), int(width), float(n_std), _ptr(m),
                                     _ptr(s_d), _ptr(r_d), _ptr(v_d), _ptr(p_d),
                                     float(tan_fovx), float(tan_fovy), _ptr(radii), _ptr(means2d),
                                     _ptr(touched), _ptr(keys), cap, _ptr(ranges), ctypes.byref(nk),
                                     _stream()))
    k = int(nk.value)
    return {"radii": radii, "means2d": means2d,
            "tiles_touched": touched.to(torch.int64) & 0xFFFFFFFF,
            "keys": keys[:k], "ranges": ranges.to(torch.int64) & 0xFFFFFFFF, "num_keys": k}


# ---------------------------------------------------------------------------------------------
# Batches
# ---------------------------------------------------------------------------------------------

class Batch:
    """Many renders (scenes x cameras) planned once and launched together.

    ``scenes``: list of (gauss_offset, n) into concatenated Gaussian arrays.
    ``views``: list of dicts with keys scene, height, width, fx, fy, cx, cy, quat, trans and
    optionally pixel_offset (default: packed in order) and no_grad (skip in the backward); or a
    structured array of ``_native.VIEW_DTYPE`` (the C ``fe_view`` layout, flags included), whose
    renders are always packed in order (its pixel_offset field is overwritten).
    By default the plan reserves scratch for the worst-case key count, so ``forward`` performs no
    host synchronisation and can be captured in a CUDA graph; ``exact_keys=True`` sizes the key
    scratch from the device-side count instead (one 8-byte readback per run).
    ``tile``, ``px`` (pixels per thread) and ``chunk`` (record pairs per shared-memory stage)
    select the blend configuration; ``heavy_first=True`` makes the blend take the tiles with the
    most keys first (tile-major binning only; see FE_FLAG_HEAVY_TILES_FIRST).
    ``keep_binning=True`` lets ``backward`` reuse the binning of the preceding ``forward`` on the
    same Gaussian tensors (their contents must not change in between) instead of recomputing it.
    ``footprint="rect"`` bins every tile of each footprint's bounding rectangle
    (FE_FLAG_RECT_BINNING) instead of the tiles its footprint ellipse reaches in each tile row.
    """

    def __init__(self, scenes, views, beta2=21.4, beta3=2.66, *, cull="eps", cull_param=None,
                 tile=(16, 16), px=0, chunk=0, exact_keys=False, keep_binning=False,
                 binning="tiles", heavy_first=False, footprint="ellipse"):
        lib = N.load()
        flags = (N.flag_chunk(chunk) | (N.FE_FLAG_EXACT_KEYS if exact_keys else 0)
                 | (N.FE_FLAG_KEEP_BINNING if keep_binning else 0)
                 | _binning_flag(binning, footprint)
                 | (N.FE_FLAG_HEAVY_TILES_FIRST if heavy_first else 0))
        desc = N.make_desc(0, 1, 1, 1.0, 1.0, 0.0, 0.0, beta2, beta3, cull, cull_param, tile,
                           flags=flags, px=px)
        sc, nsc, vs, nvs = self._tables(scenes, views)
        h = ctypes.c_void_p()
        N.check(lib.fe_batch_create(ctypes.byref(desc), sc, nsc, vs, nvs, ctypes.byref(h)))
        self._h = h
        self.tile = tuple(tile)
        self._sizes()

    def _tables(self, scenes, views):
        sc = (N.SceneEntry * max(1, len(scenes)))()
        for i, (off, n) in enumerate(scenes):
            sc[i].gauss_offset = int(off)
            sc[i].n = int(n)
        if isinstance(views, np.ndarray):
            return (sc, len(scenes)) + self._array_tables(views)
        vs = (N.View * max(1, len(views)))()
        off = 0
        self.pixel_offsets = []
        self.shapes = []
        for i, v in enumerate(views):
            vs[i].scene = int(v["scene"])
            vs[i].height = int(v["height"])
            vs[i].width = int(v["width"])
            vs[i].fx, vs[i].fy, vs[i].cx, vs[i].cy = (float(v["fx"]), float(v["fy"]),
                                                      float(v["cx"]), float(v["cy"]))
            for k in range(4):
                vs[i].quat[k] = float(v["quat"][k])
            for k in range(3):
                vs[i].trans[k] = float(v["trans"][k])
            vs[i].flags = N.FE_VIEW_NO_GRAD if v.get("no_grad") else 0
            po = int(v.get("pixel_offset", off))
            vs[i].pixel_offset = po
            self.pixel_offsets.append(po)
            self.shapes.append((int(v["height"]), int(v["width"])))
            off = max(off, po + int(v["height"]) * int(v["width"]))
        return sc, len(scenes), vs, len(views)

    def _array_tables(self, views):
        arr = np.require(views, dtype=N.VIEW_DTYPE, requirements=["C", "W"])
        h = arr["height"].astype(np.int64)
        w = arr["width"].astype(np.int64)
        ends = np.cumsum(h * w)
        arr["pixel_offset"] = ends - h * w
        self.pixel_offsets = arr["pixel_offset"].tolist()
        self.shapes = list(zip(h.tolist(), w.tolist()))
        if len(arr) == 0:
            return (N.View * 1)(), 0
        return (N.View * len(arr)).from_buffer(arr), len(arr)

    def _sizes(self):
        lib = N.load()
        self.n_pixels = int(lib.fe_batch_pixels(self._h))
        self.scratch_bytes = int(lib.fe_batch_scratch_bytes(self._h))

    def reset(self, scenes, views):
        """Re-plan for new scenes/views, reusing the device buffers (they only grow)."""
        sc, nsc, vs, nvs = self._tables(scenes, views)
        N.check(N.load().fe_batch_reset(self._h, sc, nsc, vs, nvs, _stream()))
        self._sizes()

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            N.load().fe_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def forward(self, means, prec, logw, depth=None, alpha=None, stats=None):
        lib = N.load()
        dev = means.device
        if depth is None:
            depth = torch.empty(self.n_pixels, device=dev)
        if alpha is None:
            alpha = torch.empty(self.n_pixels, device=dev)
        N.check(lib.fe_batch_fwd(self._h, _ptr(means), _ptr(prec), _ptr(logw), _ptr(depth),
                                 _ptr(alpha), _ptr(stats), _stream()))
        return depth, alpha

    def forward_host(self, means, prec, logw, depth=None, alpha=None):
        """forward() from host tensors to host tensors (fe_batch_fwd_host): the Gaussians are
        copied in; into pinned outputs the blend stores depth and alpha directly as it renders,
        into pageable ones it runs in bands whose outputs are copied back while the next bands
        render. Outputs default to new pinned tensors; returns once the outputs have landed."""
        lib = N.load()
        host = []  # keeps converted copies alive until the call returns
        for t in (means, prec, logw):
            if t.is_cuda:
                raise ValueError("forward_host takes host (CPU) tensors")
            if t.dtype is not torch.float32 or not t.is_contiguous():
                t = t.detach().contiguous().float()
            host.append(t)
        if depth is None:
            depth = torch.empty(self.n_pixels, dtype=torch.float32).pin_memory()
        if alpha is None:
            alpha = torch.empty(self.n_pixels, dtype=torch.float32).pin_memory()
        for t in (depth, alpha):
            if t.is_cuda or t.dtype is not torch.float32 or not t.is_contiguous() or \
                    t.numel() < self.n_pixels:
                raise ValueError("outputs must be contiguous float32 host tensors of n_pixels")
        st = torch.cuda.current_stream()
        N.check(lib.fe_batch_fwd_host(self._h, host[0].data_ptr(), host[1].data_ptr(),
                                      host[2].data_ptr(), depth.data_ptr(), alpha.data_ptr(),
                                      st.cuda_stream))
        st.synchronize()
        return depth, alpha

    def backward(self, means, prec, logw, depth, alpha, stats, gdepth, galpha):
        lib = N.load()
        gm, gp, gw = torch.empty_like(means), torch.empty_like(prec), torch.empty_like(logw)
        N.check(lib.fe_batch_bwd(self._h, _ptr(means), _ptr(prec), _ptr(logw), _ptr(depth),
                                 _ptr(alpha), _ptr(stats), _ptr(gdepth), _ptr(galpha), _ptr(gm),
                                 _ptr(gp), _ptr(gw), _stream()))
        return gm, gp, gw

    STAGES = ("preprocess", "scan", "emit", "sort", "ranges", "blend")

    def forward_timed(self, means, prec, logw, depth=None, alpha=None, stats=None):
        """forward() with per-stage CUDA-event timings (ms); synchronises."""
        lib = N.load()
        dev = means.device
        if depth is None:
            depth = torch.empty(self.n_pixels, device=dev)
        if alpha is None:
            alpha = torch.empty(self.n_pixels, device=dev)
        ms = (ctypes.c_float * 6)()
        N.check(lib.fe_batch_fwd_timed(self._h, _ptr(means), _ptr(prec), _ptr(logw), _ptr(depth),
                                       _ptr(alpha), _ptr(stats), ms, _stream()))
        return depth, alpha, dict(zip(self.STAGES, [float(x) for x in ms]))

    @property
    def launches_per_forward(self):
        return int(N.load().fe_batch_launch_count(self._h))

    def status(self):
        lib = N.load()
        nk, wk, err = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_uint32()
        N.check(lib.fe_batch_status(self._h, _stream(), ctypes.byref(nk), ctypes.byref(wk),
                                    ctypes.byref(err)))
        return {"num_keys": nk.value, "want_keys": wk.value, "device_error": err.value}

    def view_image(self, flat, i):
        h, w = self.shapes[i]
        o = self.pixel_offsets[i]
        return flat[o:o + h * w].view(h, w)
