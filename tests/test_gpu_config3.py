"""The batched-uneven-renders configuration at its stated size: 256 scenes (N log-uniform in
[8, 512]), 1-8 poses each, image sides from {64, 128, 256}, all rendered in one persistent,
CUDA-graph-captured batch with the autotuned blend configuration.

The reference renders one camera per call (fuzzy_ellipses/__init__.py:189-239). Here every view
of the batch is compared with its own plain single-view render (to rounding: the blend pairs
records differently inside a batch), a sample of views with the float64 fm_render oracle at the
stated tolerance, and the graph replay with the eager launch (bit for bit).
"""

import numpy as np
import pytest
import torch

import fuzzy_ellipses as fe
from fuzzy_ellipses import autotune
from fuzzy_ellipses import synthetic as S
from tests.helpers import TOL_ALPHA, TOL_DEPTH_REL, oracle_pixels, parity_errors, scene_to_dev

pytestmark = pytest.mark.gpu


def _config3(dev):
    items = S.config3(seed=0)
    assert len(items) == 256
    means, prec, logw, scenes, views, owner = [], [], [], [], [], []
    off = 0
    for si, (sc, cams) in enumerate(items):
        means.append(sc.means); prec.append(sc.prec); logw.append(sc.logw)
        scenes.append((off, sc.n))
        off += sc.n
        for c in cams:
            views.append(dict(scene=si, height=c.height, width=c.width, fx=c.fx, fy=c.fy,
                              cx=c.cx, cy=c.cy, quat=c.quat, trans=c.trans))
            owner.append((si, c))
    tens = [torch.from_numpy(np.concatenate(x)).to(dev) for x in (means, prec, logw)]
    return items, scenes, views, owner, tens


@pytest.fixture(scope="module")
def cfg3(cuda_device):
    return _config3(cuda_device)


def test_config3_full_batch_graph_replay(cuda_device, cfg3, tmp_path):
    items, scenes, views, owner, (m, p, w) = cfg3
    tuner = autotune.Autotuner(path=str(tmp_path / "tune.json"))
    best = tuner.tune(scenes, views, m, p, w, reps=2)
    b = fe.Batch(scenes, views, tile=best["tile"], px=best["px"], chunk=best["chunk"],
                 heavy_first=best["heavy_first"])
    depth = torch.empty(b.n_pixels, device=cuda_device)
    alpha = torch.empty(b.n_pixels, device=cuda_device)
    b.forward(m, p, w, depth, alpha)
    st = b.status()
    assert st["device_error"] == 0 and st["num_keys"] == st["want_keys"], st
    d_eager, a_eager = depth.clone(), alpha.clone()

    # One persistent launch sequence captured as a CUDA graph, replayed.
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        b.forward(m, p, w, depth, alpha)
    depth.zero_()
    alpha.zero_()
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(depth, d_eager) and torch.equal(alpha, a_eager)
    assert b.status()["device_error"] == 0

    # Every view against its plain single-view render.
    scene_dev = {}
    for vi, (si, c) in enumerate(owner):
        if si not in scene_dev:
            scene_dev[si] = scene_to_dev(items[si][0], cuda_device)
        ms, ps, ws = scene_dev[si]
        d1, a1 = fe.render_forward(ms, ps, ws, c.fx, c.fy, c.cx, c.cy, c.quat, c.trans, c.height,
                                   c.width, tile=best["tile"])
        torch.testing.assert_close(b.view_image(depth, vi), d1, rtol=1e-6, atol=1e-7)
        torch.testing.assert_close(b.view_image(alpha, vi), a1, rtol=0, atol=1e-6)

    # A sample of views (each image size) against the float64 oracle.
    rng = np.random.default_rng(0)
    sample = rng.choice(len(owner), 24, replace=False)
    sizes = set()
    for vi in sample:
        si, c = owner[vi]
        sizes.add(c.height)
        pix = rng.choice(c.height * c.width, min(1500, c.height * c.width), replace=False)
        d_ref, a_ref = oracle_pixels(items[si][0], c, pix)
        d = b.view_image(depth, vi).cpu().numpy().ravel()[pix]
        a = b.view_image(alpha, vi).cpu().numpy().ravel()[pix]
        ea, ed = parity_errors(d, a, d_ref, a_ref)
        assert ea <= TOL_ALPHA and ed <= TOL_DEPTH_REL, (vi, ea, ed)
    assert sizes == {64, 128, 256}
    b.close()
