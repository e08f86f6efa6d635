"""Seeded input cases for the reference-binning parity fixtures (shared by the fixture generator
and the tests). Inputs follow the reference's legacy interface (fuzzy_ellipses/__init__.py:189-231):
camera-frame means with an identity view matrix, scales and scalar-first quaternions, the
OpenGL-style projection of getProjectionMatrixJax, and tan of the *full* field-of-view angle."""

from __future__ import annotations

import math

import numpy as np


def projection(width, height, fx, fy, znear=0.01, zfar=4.5):
    fov_x = math.atan(width / 2 / fx) * 2.0
    fov_y = math.atan(height / 2 / fy) * 2.0
    top = math.tan(fov_y / 2) * znear
    right = math.tan(fov_x / 2) * znear
    m = np.array([[znear / right, 0, 0, 0], [0, znear / top, 0, 0],
                  [0, 0, zfar / (zfar - znear), -(zfar * znear) / (zfar - znear)], [0, 0, 1, 0]])
    return m.T.astype(np.float32)


def tan_full_fov(size, f):
    return np.float32(math.tan(math.atan(size / 2 / f) * 2.0))


def num_stds(n):
    return 3.0 if n <= 1000 else (0.75 if n <= 5000 else (0.5 if n <= 100000 else 0.1))


def _quats(rng, n):
    q = rng.standard_normal((n, 4))
    return (q / np.linalg.norm(q, axis=1, keepdims=True)).astype(np.float32)


def _case(name, rng, n, H, W, f, depth_lo, depth_hi, spread, s_lo=0.005, s_hi=0.03):
    z = rng.uniform(depth_lo, depth_hi, n)
    x = rng.uniform(-spread, spread, n) * z
    y = rng.uniform(-spread, spread, n) * z * H / W
    means = np.stack([x, y, z], 1).astype(np.float32)
    scales = np.exp(rng.uniform(math.log(s_lo), math.log(s_hi), (n, 3))).astype(np.float32)
    return {"name": name, "means": means, "scales": scales, "rots": _quats(rng, n),
            "view": np.eye(4, dtype=np.float32), "proj": projection(W, H, f, f), "H": H, "W": W,
            "n_std": num_stds(n), "tan_fovx": tan_full_fov(W, f), "tan_fovy": tan_full_fov(H, f)}


def binning_cases():
    rng = np.random.default_rng(20240611)
    cases = [
        _case("cfg0_like", rng, 40, 200, 200, 200.0, 0.4, 0.6, 0.4),
        _case("cfg1_like", rng, 1000, 480, 640, 600.0, 0.7, 1.3, 0.6),
        _case("odd_size", rng, 300, 250, 333, 300.0, 0.3, 1.0, 0.7),
        _case("many_n3000", rng, 3000, 480, 640, 600.0, 0.5, 1.5, 0.6),
        _case("single", rng, 1, 64, 64, 64.0, 0.5, 0.5, 0.0),
    ]
    # Edge cases: behind / at the near plane, far off-screen, huge and tiny Gaussians.
    e = _case("edges", rng, 64, 72, 96, 90.0, 0.05, 2.0, 1.5, 0.0005, 0.5)
    e["means"][0, 2] = 0.2      # exactly at the near-plane test (culled: z <= 0.2)
    e["means"][1, 2] = np.nextafter(np.float32(0.2), np.float32(1.0))
    e["means"][2, 2] = -0.5     # behind the camera
    e["means"][3] = [50.0, 0.0, 1.0]   # far off-screen
    e["scales"][4] = [2.0, 2.0, 2.0]   # covers every tile
    cases.append(e)
    return cases
