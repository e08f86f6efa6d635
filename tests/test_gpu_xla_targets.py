"""The XLA custom-call targets called the way XLA calls them (stream, buffer-pointer array,
opaque descriptor bytes, status) give the same results as the named-pointer entry points."""

import ctypes

import numpy as np
import pytest
import torch

import fuzzy_ellipses as fe
from fuzzy_ellipses import _native as N
from fuzzy_ellipses import synthetic as S
from tests.helpers import scene_to_dev, to_dev

pytestmark = pytest.mark.gpu


def _buffers(*tensors):
    return (ctypes.c_void_p * len(tensors))(*[t.data_ptr() for t in tensors])


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def test_render_targets_match_the_plain_entries(cuda_device):
    lib = N.load()
    scene, cams = S.config0(seed=11)
    c = cams[0]
    H, W = 72, 96
    m, p, w = scene_to_dev(scene, cuda_device)
    q = to_dev(np.asarray(c.quat, np.float32), cuda_device)
    t = to_dev(np.asarray(c.trans, np.float32), cuda_device)
    desc = N.make_desc(scene.n, H, W, 90.0, 90.0, W / 2, H / 2)
    opaque = bytes(desc)
    d, a, st = (torch.empty(H, W, device=cuda_device), torch.empty(H, W, device=cuda_device),
                torch.empty(3, H, W, device=cuda_device))
    lib.fe_render_fwd_xla(_stream(), _buffers(m, p, w, q, t, d, a, st), opaque, len(opaque), None)
    d0, a0 = fe.render_forward(m, p, w, 90.0, 90.0, W / 2, H / 2, c.quat, c.trans, H, W)
    torch.cuda.synchronize()
    assert torch.equal(d, d0) and torch.equal(a, a0)

    gen = torch.Generator(device=cuda_device).manual_seed(0)
    gd = torch.randn(H, W, device=cuda_device, generator=gen) * (a0 > 1e-2)
    ga = torch.randn(H, W, device=cuda_device, generator=gen)
    gm, gp, gw = torch.empty_like(m), torch.empty_like(p), torch.empty_like(w)
    lib.fe_render_bwd_xla(_stream(), _buffers(m, p, w, q, t, d, a, st, gd, ga, gm, gp, gw), opaque,
                          len(opaque), None)
    mr, pr, wr = [x.clone().requires_grad_() for x in (m, p, w)]
    dr, ar = fe.render(mr, pr, wr, 90.0, 90.0, W / 2, H / 2, c.quat, c.trans, H, W)
    (dr * gd + ar * ga).sum().backward()
    for x, y in ((gm, mr.grad), (gp, pr.grad), (gw, wr.grad)):
        assert float((x - y).norm()) <= 1e-5 * float(y.norm()) + 1e-12  # atomics: order only


def test_legacy_target_matches_rasterize(cuda_device):
    lib = N.load()
    rng = np.random.default_rng(4)
    n, H, W = 60, 80, 100
    fx = fy = 100.0
    cx, cy = W / 2, H / 2
    means = rng.uniform(-0.1, 0.1, size=(n, 3)).astype(np.float32)
    scales = rng.uniform(0.01, 0.03, size=(n, 3)).astype(np.float32)
    rots = rng.normal(size=(n, 4)).astype(np.float32)
    rots /= np.linalg.norm(rots, axis=1, keepdims=True)
    weights = rng.normal(0, 0.5, size=n).astype(np.float32)
    v, u = np.mgrid[0:H, 0:W]
    rays = np.stack([(u.ravel() - cx) / fx, (v.ravel() - cy) / fy, np.ones(H * W)], 1).astype(np.float32)
    quat, trans = S.look_at([0.45, 0.1, 0.2])
    rot = S.quat_to_rot(quat).astype(np.float32)
    near, far = 0.01, 10.0
    z0, a0 = fe.rasterize(to_dev(means, cuda_device), to_dev(scales, cuda_device),
                          to_dev(rots, cuda_device), to_dev(weights, cuda_device),
                          to_dev(rays, cuda_device), to_dev(rot, cuda_device),
                          to_dev(np.asarray(trans, np.float32), cuda_device), H, W, fx, fy, cx, cy,
                          near, far)
    tfx, tfy, view, proj = fe.api._legacy_scalars(H, W, fx, fy, cx, cy, near, far)
    opaque = bytes(N.LegacyDesc(H, W, n, float(tfx), float(tfy)))
    ins = [to_dev(x, cuda_device) for x in (means, weights, scales, rots, rays, rot,
                                            np.asarray(trans, np.float32), view, proj)]
    z, a = torch.empty(H, W, device=cuda_device), torch.empty(H, W, device=cuda_device)
    lib.fe_rasterize_legacy_xla(_stream(), _buffers(*ins, z, a), opaque, len(opaque), None)
    torch.cuda.synchronize()
    # the reference applies nan_to_num after its custom call (fuzzy_ellipses/__init__.py:233-234)
    z = torch.nan_to_num(z, posinf=10.0, neginf=0.0)
    a = torch.nan_to_num(a, posinf=1.0, neginf=0.0)
    assert torch.equal(z, z0.reshape(H, W)) and torch.equal(a, a0.reshape(H, W))
