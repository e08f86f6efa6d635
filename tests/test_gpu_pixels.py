"""Multi-pose pixel-list renderer with optical flow (fm_render.py render_func_idx_quattrans and
_flow, argument order fixed) against the float64 oracle, and against the image renderer."""

import numpy as np
import pytest
import torch

import fuzzy_ellipses as fe
from fuzzy_ellipses import synthetic as S
from oracle import fm_render_np as O
from tests.helpers import TOL_ALPHA, TOL_DEPTH_REL, DEPTH_MASK_ALPHA, scene_to_dev

pytestmark = pytest.mark.gpu


def pose_list(cams):
    return np.stack([np.concatenate([c.quat, c.trans]) for c in cams]).astype(np.float32)


def grid_rays(H, W, k, step=1):
    v, u = np.mgrid[0:H:step, 0:W:step]
    n = u.size
    return np.stack([u.ravel() - W / 2, v.ravel() - H / 2, np.ones(n), np.full(n, k)], 1)


def test_mixed_pose_rays_match_oracle_with_flow(cuda_device):
    rng = np.random.default_rng(0)
    scene, cams = S.config0(seed=3)
    cams = [S.Camera(64, 64, 64.0, 64.0, 32.0, 32.0, *S.look_at(0.5 * d))
            for d in S.random_unit_vectors(3, rng)]
    poses = pose_list(cams)
    inv_f = 1.0 / 64.0
    rays = np.concatenate([grid_rays(64, 64, k, step=2) for k in range(3)])
    rays = rays[rng.permutation(len(rays))].astype(np.float32)  # poses interleaved
    m, p, w = scene_to_dev(scene, cuda_device)
    d, a, _, _, fp, fm = fe.render_pixels(m, p, w, torch.from_numpy(rays), inv_f,
                                          torch.from_numpy(poses), flow=True)
    d, a, fp, fm = (x.cpu().numpy().astype(np.float64) for x in (d, a, fp, fm))
    rd, ra, _, _, rfp, rfm = O.render_func_idx_quattrans_flow(scene.means, scene.prec,
                                                              scene.logw, rays, inv_f, poses,
                                                              21.4, 2.66)
    assert np.max(np.abs(a - ra)) <= TOL_ALPHA
    mask = ra > DEPTH_MASK_ALPHA
    assert np.max(np.abs(d - rd)[mask] / rd[mask]) <= TOL_DEPTH_REL
    # the flow arithmetic itself (given the depths): float32 against float64
    # (a depth-0 ray whose neighbour pose clamps to its own pose reprojects 0/0: NaN, as in the
    # reference; the NaNs must sit on the same rays)
    with np.errstate(invalid="ignore"):
        gfp, gfm = O.flow_from_depth(rays, inv_f, poses, d)
    for got, want in ((fp, gfp), (fm, gfm)):
        assert np.array_equal(np.isnan(got), np.isnan(want))
        ok = ~np.isnan(want)
        assert np.max(np.abs(got - want)[ok]) <= 1e-3
    # and end to end where depth is defined
    assert np.max(np.abs(fp - rfp)[mask]) <= 2e-2 and np.max(np.abs(fm - rfm)[mask]) <= 2e-2


def test_pixel_grid_equals_image_render(cuda_device):
    scene, cams = S.config0(seed=4)
    c = cams[0]
    H, W, f = 48, 80, 60.0
    m, p, w = scene_to_dev(scene, cuda_device)
    rays = grid_rays(H, W, 0).astype(np.float32)
    pose = pose_list([c])
    d, a, _, _ = fe.render_pixels(m, p, w, torch.from_numpy(rays), 1.0 / f, torch.from_numpy(pose))
    di, ai = fe.render_forward(m, p, w, f, f, W / 2, H / 2, c.quat, c.trans, H, W)
    assert torch.allclose(a.reshape(H, W), ai, atol=2e-6, rtol=0)
    ok = ai > DEPTH_MASK_ALPHA
    assert torch.allclose(d.reshape(H, W)[ok], di[ok], rtol=2e-5, atol=0)


def test_scaled_rays_weights_and_features(cuda_device):
    """Rays (x c, y c, c): the same line as (x, y, 1), so alpha is unchanged, while the ray
    parameter (and with it the softmax logits -beta2 z) scales by 1/c, as in fm_render; depth,
    the dense weights and the weighted features agree with the oracle's."""
    rng = np.random.default_rng(5)
    scene, cams = S.config0(seed=5)
    c = cams[0]
    pose = pose_list([c])
    inv_f = 1.0 / 40.0
    base = grid_rays(40, 40, 0, step=3)
    scaled = base.copy()
    scaled[:, :3] *= 2.0
    feats = rng.normal(size=(scene.n, 5)).astype(np.float32)
    m, p, w = scene_to_dev(scene, cuda_device)
    out1 = fe.render_pixels(m, p, w, torch.from_numpy(base.astype(np.float32)), inv_f,
                            torch.from_numpy(pose))
    out2 = fe.render_pixels(m, p, w, torch.from_numpy(scaled.astype(np.float32)), inv_f,
                            torch.from_numpy(pose), weights=True, features=torch.from_numpy(feats))
    d1, a1 = out1[0].cpu().numpy(), out1[1].cpu().numpy()
    d2, a2, wts, of = out2[0].cpu().numpy(), out2[1].cpu().numpy(), out2[3].cpu().numpy(), out2[4].cpu().numpy()
    assert np.allclose(a2, a1, atol=1e-6)
    rd, ra, _, rw = O.render_func_idx_quattrans(scene.means, scene.prec, scene.logw, scaled, inv_f,
                                                pose, 21.4, 2.66, return_weights=True)
    mask = ra > DEPTH_MASK_ALPHA
    assert np.max(np.abs(a2 - ra)) <= TOL_ALPHA
    assert np.max(np.abs(d2 - rd)[mask] / rd[mask]) <= TOL_DEPTH_REL
    assert np.max(np.abs(wts - rw)[:, mask]) <= 1e-4
    assert np.allclose(wts.sum(0)[mask], 1.0, atol=1e-5)
    assert np.max(np.abs(of - (rw.T @ feats.astype(np.float64)))[mask]) <= 1e-3
