"""fe_render_fwd_noalloc (fixed device scratch, no allocation) against fe_render_fwd.

Collected last on purpose: it must pass both in a fresh process and after every other test has
used the arena-backed entries. Calls go through the C ABI with ctypes; torch only provides the
device buffers and the stream.
"""

import ctypes

import numpy as np
import pytest
import torch

from fuzzy_ellipses import _native as N
from fuzzy_ellipses import synthetic as S

from tests.helpers import TOL_ALPHA, TOL_DEPTH_REL, scene_to_dev, to_dev

pytestmark = pytest.mark.gpu

FE_ERR_SCRATCH_LIMIT = 8


def _ptr(t):
    return ctypes.c_void_p(0 if t is None else t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _outputs(h, w, dev):
    return (torch.full((h, w), float("nan"), device=dev), torch.full((h, w), float("nan"), device=dev),
            torch.full((3, h, w), float("nan"), device=dev))


def _call(entry, scene_dev, cam, desc, outs, err=None):
    lib = N.load()
    m, p, w = scene_dev
    q = to_dev(np.asarray(cam.quat, np.float32), m.device)
    t = to_dev(np.asarray(cam.trans, np.float32), m.device)
    args = [ctypes.byref(desc), _ptr(m), _ptr(p), _ptr(w), _ptr(q), _ptr(t), _ptr(outs[0]),
            _ptr(outs[1]), _ptr(outs[2])]
    if entry == "fe_render_fwd_noalloc":
        args.append(_ptr(err))
    rc = getattr(lib, entry)(*args, _stream())
    torch.cuda.synchronize()
    return rc


def _desc(scene, cam, tile=(16, 16), px=0, flags=0):
    return N.make_desc(scene.n, cam.height, cam.width, cam.fx, cam.fy, cam.cx, cam.cy,
                       tile=tile, px=px, flags=flags)


def _assert_close(ref, got):
    d0, a0, s0 = (x.cpu().numpy() for x in ref)
    d1, a1, s1 = (x.cpu().numpy() for x in got)
    assert np.all(np.isfinite(d1)) and np.all(np.isfinite(a1))
    assert np.max(np.abs(a1 - a0)) <= TOL_ALPHA
    mask = a0 > 1e-3
    assert np.max(np.abs(d1 - d0)[mask] / np.maximum(np.abs(d0[mask]), 1e-6)) <= TOL_DEPTH_REL
    assert np.allclose(s1, s0, rtol=1e-5, atol=1e-6)


def test_noalloc_matches_arena_entry_twice_in_a_row(cuda_device):
    scene, cams = S.config1(seed=5)
    cam = cams[3]  # 640x480, 1000 Gaussians: 1.2M worst-case pairs, inside the fixed scratch
    sd = scene_to_dev(scene, cuda_device)
    desc = _desc(scene, cam)
    ref = _outputs(cam.height, cam.width, cuda_device)
    assert _call("fe_render_fwd", sd, cam, desc, ref) == 0
    err = torch.full((1,), 7, dtype=torch.int32, device=cuda_device)
    for _ in range(2):
        got = _outputs(cam.height, cam.width, cuda_device)
        assert _call("fe_render_fwd_noalloc", sd, cam, desc, got, err) == 0, \
            N.load().fe_last_error_message()
        assert int(err.item()) == 0
        _assert_close(ref, got)


def test_noalloc_smaller_request_then_larger_again(cuda_device):
    # A different layout of the same scratch in between (8x8 tiles, 2 pixels per thread, a
    # ragged image): stale ranges or keys of one call must not leak into the next.
    rng = np.random.default_rng(11)
    small = S.random_gaussians(300, 0.1, rng)
    cam_s = S.Camera(77, 101, 90.0, 90.0, 50.5, 38.0, *S.look_at([0.4, 0.2, 0.25]))
    scene, cams = S.config1(seed=6)
    big_d = scene_to_dev(scene, cuda_device)
    small_d = scene_to_dev(small, cuda_device)
    for sc, sd, cam, tile, px in ((scene, big_d, cams[0], (16, 16), 0),
                                  (small, small_d, cam_s, (8, 8), 2),
                                  (scene, big_d, cams[9], (16, 16), 0)):
        desc = _desc(sc, cam, tile, px)
        ref = _outputs(cam.height, cam.width, cuda_device)
        got = _outputs(cam.height, cam.width, cuda_device)
        assert _call("fe_render_fwd", sd, cam, desc, ref) == 0
        assert _call("fe_render_fwd_noalloc", sd, cam, desc, got) == 0
        _assert_close(ref, got)


@pytest.mark.parametrize("n,flags", [(1000, N.FE_FLAG_RADIX_BINNING), (5000, 0)])
def test_noalloc_emit_and_radix_sort_branch(cuda_device, n, flags):
    """The binning branch that carves the scan space, the second key buffer and the sort
    histograms out of the fixed array: forced by FE_FLAG_RADIX_BINNING, and chosen by the size
    rule for 5000 Gaussians on one 640x480 view (above the tile-major limit, 6 M worst-case
    pairs, inside the fixed scratch). Two calls in a row against the arena entry."""
    rng = np.random.default_rng(13)
    scene = S.random_gaussians(n, 0.3, rng)
    cam = S.config1(seed=0)[1][5]
    sd = scene_to_dev(scene, cuda_device)
    desc = _desc(scene, cam, flags=flags)
    ref = _outputs(cam.height, cam.width, cuda_device)
    assert _call("fe_render_fwd", sd, cam, desc, ref) == 0
    for _ in range(2):
        got = _outputs(cam.height, cam.width, cuda_device)
        assert _call("fe_render_fwd_noalloc", sd, cam, desc, got) == 0, \
            N.load().fe_last_error_message()
        _assert_close(ref, got)


def test_noalloc_rejects_requests_beyond_the_fixed_scratch(cuda_device):
    rng = np.random.default_rng(12)
    scene = S.random_gaussians(7000, 0.1, rng)  # 7000 x 1200 tiles: over the fixed scratch
    cam = S.config1(seed=0)[1][0]
    sd = scene_to_dev(scene, cuda_device)
    outs = _outputs(cam.height, cam.width, cuda_device)
    rc = _call("fe_render_fwd_noalloc", sd, cam, _desc(scene, cam), outs)
    assert rc == FE_ERR_SCRATCH_LIMIT
    msg = N.load().fe_last_error_message().decode()
    assert "7000 Gaussians" in msg and str(128 << 20) in msg
    assert torch.isnan(outs[1]).all()  # nothing was launched
    # The same request through the arena entry still works.
    assert _call("fe_render_fwd", sd, cam, _desc(scene, cam), outs) == 0
