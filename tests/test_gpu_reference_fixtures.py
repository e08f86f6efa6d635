"""The CUDA path against outputs of the reference's own baseline/fm_render.py.

tests/golden/fm_render_golden.npz was made by running the unmodified reference renderer in
float64 (tests/golden/make_fm_render_golden.py). These tests render the stored inputs on the GPU
and compare with the stored outputs at the stated tolerances (1e-5 absolute alpha, 1e-4
relative depth where the reference's alpha exceeds 1e-3). Pixels where fm_render's depth is set
by its +1e-20 weight floor (a behind-camera Gaussian's logit dominating the max) are excluded
from the depth check and covered by test_gpu_render.py.
"""

import numpy as np
import pytest
import torch

import fuzzy_ellipses as fe
from tests.helpers import (DEPTH_MASK_ALPHA, GOLDEN_VIEWS, TOL_ALPHA, TOL_DEPTH_REL,
                           floor_dominated, golden, golden_camera, golden_cameras, golden_scene,
                           parity_errors, scene_to_dev)

pytestmark = pytest.mark.gpu
TILES = [(8, 8), (16, 16), (32, 8)]


def _render(dev, scene, cam, **kw):
    m, p, w = scene_to_dev(scene, dev)
    d, a = fe.render_forward(m, p, w, cam.fx, cam.fy, cam.cx, cam.cy, cam.quat, cam.trans,
                             cam.height, cam.width, **kw)
    torch.cuda.synchronize()
    assert fe.device_status() == 0
    return d.cpu().numpy(), a.cpu().numpy()


@pytest.mark.parametrize("key", GOLDEN_VIEWS)
@pytest.mark.parametrize("tile", TILES)
def test_full_views_match_reference(cuda_device, key, tile):
    scene = golden_scene(key)
    cam, d_ref, a_ref = golden_camera(key)
    d, a = _render(cuda_device, scene, cam, tile=tile)
    ea, ed = parity_errors(d, a, d_ref, a_ref, exclude=floor_dominated(scene, cam))
    assert ea <= TOL_ALPHA and ed <= TOL_DEPTH_REL, (key, tile, ea, ed)


def test_config1_every_camera_matches_reference(cuda_device):
    """All 16 cameras of the 1000-Gaussian 640x480 configuration, 2000 fixed pixels each."""
    g = golden()
    scene = golden_scene("cfg1")
    worst = (0.0, 0.0)
    for ci, cam in enumerate(golden_cameras("cfg1")):
        d, a = _render(cuda_device, scene, cam)
        pix = g["cfg1_pix"][ci]
        ea, ed = parity_errors(d.ravel()[pix], a.ravel()[pix], g["cfg1_depth"][ci],
                               g["cfg1_alpha"][ci])
        assert ea <= TOL_ALPHA and ed <= TOL_DEPTH_REL, (ci, ea, ed)
        worst = (max(worst[0], ea), max(worst[1], ed))
    print(f"config 1, 16 cameras x 2000 pixels: alpha {worst[0]:.2e}, depth rel {worst[1]:.2e}")


def test_config1_batched_matches_reference(cuda_device):
    """The same 16 views rendered as one batch (persistent blend over all their tiles)."""
    g = golden()
    scene = golden_scene("cfg1")
    cams = golden_cameras("cfg1")
    m, p, w = scene_to_dev(scene, cuda_device)
    views = [dict(scene=0, height=c.height, width=c.width, fx=c.fx, fy=c.fy, cx=c.cx, cy=c.cy,
                  quat=c.quat, trans=c.trans) for c in cams]
    batch = fe.Batch([(0, scene.n)], views)
    depth, alpha = batch.forward(m, p, w)
    assert batch.status()["device_error"] == 0
    for ci, cam in enumerate(cams):
        pix = g["cfg1_pix"][ci]
        d = batch.view_image(depth, ci).cpu().numpy().ravel()[pix]
        a = batch.view_image(alpha, ci).cpu().numpy().ravel()[pix]
        ea, ed = parity_errors(d, a, g["cfg1_depth"][ci], g["cfg1_alpha"][ci])
        assert ea <= TOL_ALPHA and ed <= TOL_DEPTH_REL, (ci, ea, ed)


def test_config2_views_match_reference(cuda_device):
    g = golden()
    model = golden_scene("cfg2")
    cams = golden_cameras("cfg2")
    for vi in (0, 11):
        d, a = _render(cuda_device, model, cams[vi])
        ea, ed = parity_errors(d, a, g[f"cfg2_v{vi}_depth"], g[f"cfg2_v{vi}_alpha"])
        assert ea <= TOL_ALPHA and ed <= TOL_DEPTH_REL, (vi, ea, ed)


def test_pixel_lists_match_reference(cuda_device):
    """render_func_idx_quattrans[_flow] with dense weights and flows."""
    g = golden()
    scene = golden_scene("pix")
    m, p, w = scene_to_dev(scene, cuda_device)
    rays = torch.from_numpy(g["pix_rays"])
    poses = torch.from_numpy(g["pix_poses"])
    d, a, _, wts, fp, fm = fe.render_pixels(m, p, w, rays, float(g["pix_invf"]), poses, flow=True,
                                            weights=True)
    d, a, wts, fp, fm = (x.cpu().numpy().astype(np.float64) for x in (d, a, wts, fp, fm))
    ra, rd = g["pix_alpha"], g["pix_depth"]
    mask = ra > DEPTH_MASK_ALPHA
    assert np.max(np.abs(a - ra)) <= TOL_ALPHA
    assert np.max(np.abs(d - rd)[mask] / rd[mask]) <= TOL_DEPTH_REL
    assert np.max(np.abs(wts - g["pix_w"])[:, mask]) <= 1e-4
    # flows in pixels, where depth is defined: float32 reprojection of a depth good to 1e-4
    assert np.max(np.abs(fp - g["pix_flowp"])[mask]) <= 2e-2
    assert np.max(np.abs(fm - g["pix_flowm"])[mask]) <= 2e-2


def test_quat_cam_matches_reference(cuda_device):
    """render_func_quat_cam: normalised-pixel rays with an aspect ratio and the 0.5 shift."""
    g = golden()
    scene = golden_scene("cam")
    m, p, w = scene_to_dev(scene, cuda_device)
    inv_f, aspect = (float(x) for x in g["cam_invf_aspect"])
    d, a, _, _ = fe.render_pixels_cam(m, p, w, torch.from_numpy(g["cam_pixels"]), aspect, inv_f,
                                      g["cam_quat"], g["cam_trans"])
    d, a = d.cpu().numpy().astype(np.float64), a.cpu().numpy().astype(np.float64)
    ea, ed = parity_errors(d, a, g["cam_depth"], g["cam_alpha"])
    assert ea <= TOL_ALPHA and ed <= TOL_DEPTH_REL, (ea, ed)


def test_gmm_log_likelihood_matches_reference(cuda_device):
    g = golden()
    scene = golden_scene("gmm")
    m, p, w = scene_to_dev(scene, cuda_device)
    pts = torch.from_numpy(g["gmm_points"]).to(cuda_device)
    nll, point_ll, res = fe.gmm_log_likelihood(m, p, w, pts, return_matrix=True)
    res = res.cpu().numpy().astype(np.float64)
    ref = g["gmm_res"]
    assert np.max(np.abs(res - ref)) <= 2e-6 * np.abs(ref).max()
    assert abs(float(nll) - float(g["gmm_ll"])) <= 2e-6 * abs(float(g["gmm_ll"]))
