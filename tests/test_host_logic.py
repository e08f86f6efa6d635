"""Host-side logic of the autotuner and the server (no GPU)."""

import numpy as np

from fuzzy_ellipses import autotune, serve
from fuzzy_ellipses import synthetic as S


def test_bucket_is_stable_and_discriminates():
    sc = [(0, 100), (100, 2000)]
    v_small = [dict(scene=0, height=64, width=64)] * 4
    v_big = [dict(scene=1, height=480, width=640)] * 16
    assert autotune.bucket(sc, v_small) == autotune.bucket(sc, list(v_small))
    assert autotune.bucket(sc, v_small) != autotune.bucket(sc, v_big)


def test_autotuner_default_and_cache_roundtrip(tmp_path):
    t = autotune.Autotuner(path=str(tmp_path / "x.json"))
    sc, views = [(0, 10)], [dict(scene=0, height=32, width=32)]
    assert t.lookup(sc, views) == autotune.DEFAULT


def test_footprint_estimate_monotone():
    rng = np.random.default_rng(0)
    sc = S.random_gaussians(100, 0.1, rng)
    cam = S.Camera(64, 64, 64.0, 64.0, 32.0, 32.0, *S.look_at([0.5, 0, 0]))
    r1 = serve.RenderRequest(sc.means, sc.prec, sc.logw, [cam])
    r2 = serve.RenderRequest(sc.means, sc.prec, sc.logw, [cam, cam])
    r3 = serve.RenderRequest(sc.means, sc.prec, sc.logw, [cam], [np.zeros((64, 64), np.float32)])
    assert serve.estimate_footprint(r1) < serve.estimate_footprint(r2)
    assert serve.estimate_footprint(r1) < serve.estimate_footprint(r3)


def test_bce_gradient_matches_autograd():
    import torch
    a = torch.tensor([1e-9, 0.2, 0.5, 0.9, 1 - 1e-9], dtype=torch.float64, requires_grad=True)
    t = torch.tensor([1.0, 0.0, 1.0, 0.0, 1.0], dtype=torch.float64)
    loss, g = serve.bce_alpha_grad(a.detach(), t, a.numel())
    ac = a.clamp(3e-8, 1 - 3e-8)
    ref = -(t * torch.log(ac) + (1 - t) * torch.log(1 - ac)).mean()
    ref.backward()
    assert torch.allclose(loss / a.numel(), ref.detach())
    assert g.dtype == torch.float32
    assert torch.allclose(g.double(), a.grad, rtol=1e-6)
    # float32 alpha at 1.0 stays finite: the clamp bound 1-3e-8 is applied in float64
    loss1, g1 = serve.bce_alpha_grad(torch.ones(3), torch.zeros(3), 3)
    assert torch.isfinite(loss1) and abs(float(loss1) / 3 + np.log(3e-8)) < 1e-6
    assert float(g1.abs().max()) == 0.0
