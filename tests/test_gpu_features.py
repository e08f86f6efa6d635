"""Softmax-weighted features of an image render (fm_render's w applied to per-Gaussian features)
against the float64 oracle's w @ f, against the pixel-list path, and the weight sum."""

import numpy as np
import pytest
import torch

import fuzzy_ellipses as fe
from fuzzy_ellipses import synthetic as S
from oracle import fm_render_np as O
from tests.helpers import DEPTH_MASK_ALPHA, scene_to_dev

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("tile,H,W", [((16, 16), 64, 64), ((8, 8), 37, 53), ((32, 8), 45, 70)])
def test_features_match_oracle_weights(cuda_device, tile, H, W):
    rng = np.random.default_rng(sum(tile) + H)
    scene, cams = S.config0(seed=7)
    c = cams[0]
    f = float(max(H, W))
    feats = rng.normal(size=(scene.n, 6)).astype(np.float32)  # two chunks of four
    m, p, w = scene_to_dev(scene, cuda_device)
    d, a, out = fe.render_features(m, p, w, torch.from_numpy(feats), f, f, W / 2, H / 2, c.quat,
                                   c.trans, H, W, tile=tile)
    out = out.cpu().numpy().reshape(-1, 6)
    rays = O.pinhole_rays(H, W, f, f, W / 2, H / 2)
    _, ra, _, rw = O.render_func_quat(scene.means, scene.prec, scene.logw, rays, c.quat, c.trans,
                                      21.4, 2.66, return_weights=True)
    mask = ra > DEPTH_MASK_ALPHA
    ref = rw.T @ feats.astype(np.float64)
    assert np.max(np.abs(out - ref)[mask]) <= 1e-3
    # all-ones feature: the weights sum to one wherever a front Gaussian exists (to 5e-5: this
    # pass re-evaluates each weight in scalar arithmetic, the forward summed its normaliser with
    # packed arithmetic associated differently)
    ones = fe.render_features(m, p, w, torch.ones(scene.n, 1), f, f, W / 2, H / 2, c.quat, c.trans,
                              H, W, tile=tile)[2].cpu().numpy().ravel()
    assert np.allclose(ones[mask], 1.0, atol=5e-5)
    assert np.all((ones == 0) | (np.abs(ones - 1) < 5e-5))


def test_features_equal_the_pixel_list_path(cuda_device):
    rng = np.random.default_rng(3)
    scene, cams = S.config0(seed=8)
    c = cams[0]
    H, W, f = 48, 64, 60.0
    feats = torch.from_numpy(rng.normal(size=(scene.n, 3)).astype(np.float32))
    m, p, w = scene_to_dev(scene, cuda_device)
    _, a, out = fe.render_features(m, p, w, feats, f, f, W / 2, H / 2, c.quat, c.trans, H, W)
    v, u = np.mgrid[0:H, 0:W]
    rays = np.stack([u.ravel() - W / 2, v.ravel() - H / 2, np.ones(H * W), np.zeros(H * W)], 1)
    pose = np.concatenate([c.quat, c.trans])[None].astype(np.float32)
    res = fe.render_pixels(m, p, w, torch.from_numpy(rays.astype(np.float32)), 1.0 / f,
                           torch.from_numpy(pose), features=feats)
    ok = (a > DEPTH_MASK_ALPHA).reshape(-1)
    assert torch.allclose(out.reshape(-1, 3)[ok], res[4][ok], rtol=1e-4, atol=1e-5)
