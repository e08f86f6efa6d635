"""Seeded synthetic fuzzy-metaball scenes and cameras.

The reference builds its scenes from the YCB-V dataset (``baseline/ycb_fmb_rotscale.py:1-306``),
which is not available here; these generators stand in for it with the distributions below.

* Gaussians: means ~ U[-a, a]^3; covariance ``R diag(s^2) R^T`` with ``R`` a Haar-random
  rotation and ``s`` log-uniform in [0.005, 0.03] m per axis; the precision factor is passed in
  the reference renderer's convention (``baseline/fm_render.py:14,26``): ``prec_full = L^T``
  with ``L = inv(chol(Sigma))`` lower-triangular, so ``triu(prec_full) triu(prec_full)^T`` is the
  precision. Log-weights ~ N(0, 0.5^2).
* Cameras: pinhole, centre ``r * d`` with ``d`` on the unit sphere, looking at the origin. The
  pose follows ``render_func_quat`` (``baseline/fm_render.py:113-126``): world rays are
  ``rays_cam @ quat_to_rot(quat)`` and the ray origin is ``t`` (the camera centre).

Every array is returned as float32 (the renderer's input type); the oracle evaluates on the
same float32 values promoted to float64.
"""

from __future__ import annotations

import dataclasses
import math

import numpy as np

__all__ = ["Scene", "Camera", "quat_to_rot", "rot_to_quat", "random_gaussians", "look_at",
           "fibonacci_sphere", "random_unit_vectors", "config0", "config1", "config2",
           "config3", "config4_request_stream"]


@dataclasses.dataclass
class Scene:
    means: np.ndarray       # (N, 3) float32
    prec: np.ndarray        # (N, 3, 3) float32, upper-triangular factor (fm_render prec_full)
    logw: np.ndarray        # (N,) float32

    @property
    def n(self) -> int:
        return int(self.means.shape[0])


@dataclasses.dataclass
class Camera:
    height: int
    width: int
    fx: float
    fy: float
    cx: float
    cy: float
    quat: np.ndarray        # (4,) float32, scalar first
    trans: np.ndarray       # (3,) float32, camera centre in world coordinates


def quat_to_rot(q):
    """Scalar-first quaternion to rotation matrix; same formula as ``util_render.py:51-76``."""
    w, x, y, z = (float(v) for v in q)
    n = w * w + x * x + y * y + z * z
    if not n > 1e-12:
        return np.eye(3)
    s = 2.0 / n
    X, Y, Z = x * s, y * s, z * s
    return np.array([
        [1.0 - (y * Y + z * Z), x * Y - w * Z, x * Z + w * Y],
        [x * Y + w * Z, 1.0 - (x * X + z * Z), y * Z - w * X],
        [x * Z - w * Y, y * Z + w * X, 1.0 - (x * X + y * Y)],
    ])


def rot_to_quat(r):
    """Rotation matrix to a unit scalar-first quaternion (Shepperd's method)."""
    r = np.asarray(r, dtype=np.float64)
    tr = r[0, 0] + r[1, 1] + r[2, 2]
    if tr > 0:
        s = math.sqrt(tr + 1.0) * 2.0
        q = [0.25 * s, (r[2, 1] - r[1, 2]) / s, (r[0, 2] - r[2, 0]) / s, (r[1, 0] - r[0, 1]) / s]
    elif r[0, 0] > r[1, 1] and r[0, 0] > r[2, 2]:
        s = math.sqrt(1.0 + r[0, 0] - r[1, 1] - r[2, 2]) * 2.0
        q = [(r[2, 1] - r[1, 2]) / s, 0.25 * s, (r[0, 1] + r[1, 0]) / s, (r[0, 2] + r[2, 0]) / s]
    elif r[1, 1] > r[2, 2]:
        s = math.sqrt(1.0 + r[1, 1] - r[0, 0] - r[2, 2]) * 2.0
        q = [(r[0, 2] - r[2, 0]) / s, (r[0, 1] + r[1, 0]) / s, 0.25 * s, (r[1, 2] + r[2, 1]) / s]
    else:
        s = math.sqrt(1.0 + r[2, 2] - r[0, 0] - r[1, 1]) * 2.0
        q = [(r[1, 0] - r[0, 1]) / s, (r[0, 2] + r[2, 0]) / s, (r[1, 2] + r[2, 1]) / s, 0.25 * s]
    q = np.array(q)
    return q / np.linalg.norm(q)


def _haar_rotations(n, rng):
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    return np.stack([quat_to_rot(qi) for qi in q]) if n else np.zeros((0, 3, 3))


def random_gaussians(n, half_extent, rng, scale_lo=0.005, scale_hi=0.03, logw_sigma=0.5):
    """``n`` Gaussians with the distributions described in the module docstring."""
    means = rng.uniform(-half_extent, half_extent, size=(n, 3))
    rots = _haar_rotations(n, rng)
    s = np.exp(rng.uniform(math.log(scale_lo), math.log(scale_hi), size=(n, 3)))
    cov = np.einsum("nij,nj,nkj->nik", rots, s ** 2, rots)
    chol = np.linalg.cholesky(cov)
    lower = np.linalg.inv(chol)                    # L = inv(chol(Sigma)), Sigma^-1 = L^T L
    prec_full = np.transpose(lower, (0, 2, 1))     # upper factor U = L^T, Sigma^-1 = U U^T
    prec_full = np.triu(prec_full)
    logw = rng.normal(0.0, logw_sigma, size=n)
    return Scene(means.astype(np.float32), prec_full.astype(np.float32), logw.astype(np.float32))


def look_at(center, target=(0.0, 0.0, 0.0)):
    """Pose (quat, trans) of a camera at ``center`` looking at ``target``.

    Camera axes are x = image right, y = image down, z = forward, stored as the rows of
    ``quat_to_rot(quat)`` so that ``rays_cam @ R`` gives world directions.
    """
    c = np.asarray(center, dtype=np.float64)
    f = np.asarray(target, dtype=np.float64) - c
    f /= np.linalg.norm(f)
    up = np.array([0.0, 0.0, 1.0])
    if abs(f @ up) > 0.99:
        up = np.array([0.0, 1.0, 0.0])
    right = np.cross(f, up)
    right /= np.linalg.norm(right)
    down = np.cross(f, right)
    rot = np.stack([right, down, f])
    return rot_to_quat(rot).astype(np.float32), c.astype(np.float32)


def fibonacci_sphere(n, radius):
    """``n`` points spread uniformly on a sphere of ``radius`` (golden-angle spiral)."""
    i = np.arange(n) + 0.5
    z = 1.0 - 2.0 * i / n
    rr = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    phi = i * math.pi * (3.0 - math.sqrt(5.0))
    return radius * np.stack([rr * np.cos(phi), rr * np.sin(phi), z], 1)


def random_unit_vectors(n, rng):
    d = rng.standard_normal((n, 3))
    return d / np.linalg.norm(d, axis=1, keepdims=True)


def _camera(center, size_hw, f, c):
    q, t = look_at(center)
    return Camera(int(size_hw[0]), int(size_hw[1]), float(f[0]), float(f[1]),
                  float(c[0]), float(c[1]), q, t)


def config0(seed=0):
    """Plain forward render: N=40, means U[-0.1,0.1]^3, one 200x200 camera (f=200) at 0.5 m."""
    rng = np.random.default_rng(seed)
    scene = random_gaussians(40, 0.1, rng)
    cam = _camera(0.5 * random_unit_vectors(1, rng)[0], (200, 200), (200.0, 200.0), (100.0, 100.0))
    return scene, [cam]


def config1(seed=0, n_cameras=16):
    """Larger forward: N=1000, means U[-0.3,0.3]^3, 16 cameras 640x480 (f=600) on a 1.0 m sphere."""
    rng = np.random.default_rng(seed)
    scene = random_gaussians(1000, 0.3, rng)
    cams = [_camera(p, (480, 640), (600.0, 600.0), (320.0, 240.0))
            for p in fibonacci_sphere(n_cameras, 1.0)]
    return scene, cams


def config2(seed=0):
    """Differentiable step: N=200 ground truth + jittered model, 20 views 128x128 (f=128) at 0.6 m.

    Returns ``(gt_scene, model_scene, cameras)``; the model has means jittered by N(0, 0.01^2) m
    and per-axis scales multiplied by U[0.8, 1.2] (applied to the precision factor as 1/k).
    """
    rng = np.random.default_rng(seed)
    n = 200
    means = rng.uniform(-0.1, 0.1, size=(n, 3))
    rots = _haar_rotations(n, rng)
    s = np.exp(rng.uniform(math.log(0.005), math.log(0.03), size=(n, 3)))
    logw = rng.normal(0.0, 0.5, size=n)

    def build(means_, s_):
        cov = np.einsum("nij,nj,nkj->nik", rots, s_ ** 2, rots)
        lower = np.linalg.inv(np.linalg.cholesky(cov))
        return Scene(means_.astype(np.float32),
                     np.triu(np.transpose(lower, (0, 2, 1))).astype(np.float32),
                     logw.astype(np.float32))

    gt = build(means, s)
    model = build(means + rng.normal(0.0, 0.01, size=(n, 3)), s * rng.uniform(0.8, 1.2, size=(n, 3)))
    cams = [_camera(p, (128, 128), (128.0, 128.0), (64.0, 64.0)) for p in fibonacci_sphere(20, 0.6)]
    return gt, model, cams


def config3(seed=0, n_scenes=256):
    """Batched uneven renders: 256 scenes, N log-uniform in [8, 512], 1-8 poses each at 0.5 m,
    image side drawn from {64, 128, 256} (f = side, c = side/2). Returns ``[(scene, [cams])]``."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_scenes):
        n = int(round(math.exp(rng.uniform(math.log(8), math.log(512)))))
        scene = random_gaussians(n, 0.1, rng)
        n_pose = int(rng.integers(1, 9))
        side = int(rng.choice([64, 128, 256]))
        cams = [_camera(0.5 * d, (side, side), (float(side), float(side)), (side / 2, side / 2))
                for d in random_unit_vectors(n_pose, rng)]
        out.append((scene, cams))
    return out


def config4_request_stream(n_requests, rate_hz, seed=0):
    """Served mixed requests: Poisson arrivals at ``rate_hz``; each request has a scene with N
    log-uniform in [20, 2000], 1-32 poses at 0.5 m, image side uniform in 96..480, and is
    forward-only with probability 0.7, else forward+backward with the silhouette BCE loss.

    Returns a list of dicts ``{arrival_s, scene, cameras, backward}``.
    """
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for _ in range(n_requests):
        t += rng.exponential(1.0 / rate_hz)
        n = int(round(math.exp(rng.uniform(math.log(20), math.log(2000)))))
        scene = random_gaussians(n, 0.1, rng)
        n_pose = int(rng.integers(1, 33))
        side = int(rng.integers(96, 481))
        cams = [_camera(0.5 * d, (side, side), (float(side), float(side)), (side / 2, side / 2))
                for d in random_unit_vectors(n_pose, rng)]
        out.append({"arrival_s": t, "scene": scene, "cameras": cams,
                    "backward": bool(rng.uniform() >= 0.7)})
    return out
