"""Host-side logic of the autotuner and the server (no GPU)."""

import ctypes

import numpy as np
import pytest

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


def test_autotuner_keeps_device_and_host_picks_apart(tmp_path):
    """The host-to-host target is cached under its own key: a device pick does not answer a
    host lookup and the other way round; both survive a reload from the cache file."""
    import json

    path = tmp_path / "tune.json"
    sc, views = [(0, 1000)], [dict(scene=0, height=480, width=640)] * 16
    key = autotune.bucket(sc, views)
    path.write_text(json.dumps({
        key: {"tile": [16, 16], "px": 4, "chunk": 32, "heavy_first": True, "ms": 0.2},
        key + "_host": {"tile": [32, 8], "px": 2, "chunk": 16, "heavy_first": False, "ms": 0.27}}))
    t = autotune.Autotuner(path=str(path))
    dev, host = t.lookup(sc, views), t.lookup(sc, views, target="host")
    assert (dev["tile"], dev["px"], dev["chunk"], dev["heavy_first"]) == ((16, 16), 4, 32, True)
    assert (host["tile"], host["px"], host["chunk"]) == ((32, 8), 2, 16)
    only_dev = autotune.Autotuner(path=str(tmp_path / "missing.json"))
    only_dev.table[key] = {"tile": [8, 8], "px": 2, "chunk": 8}
    assert only_dev.lookup(sc, views, target="host") == autotune.DEFAULT


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


def test_malformed_requests_are_rejected_on_the_host():
    rng = np.random.default_rng(3)
    sc = S.random_gaussians(10, 0.1, rng)
    cam = S.Camera(32, 40, 40.0, 40.0, 20.0, 16.0, *S.look_at([0.5, 0, 0]))
    serve._validate(serve.RenderRequest(sc.means, sc.prec, sc.logw, [cam]))
    bad_cam = S.Camera(32, 40, 0.0, 40.0, 20.0, 16.0, *S.look_at([0.5, 0, 0]))
    cases = [serve.RenderRequest(sc.means, sc.prec, sc.logw, []),
             serve.RenderRequest(sc.means, sc.prec, sc.logw, [bad_cam]),
             serve.RenderRequest(sc.means[:5], sc.prec, sc.logw, [cam]),
             serve.RenderRequest(sc.means, sc.prec, sc.logw, [cam], [np.zeros((40, 32))])]
    for r in cases:
        with pytest.raises(ValueError):
            serve._validate(r)


def test_view_table_matches_the_c_layout():
    from fuzzy_ellipses import _native as N
    rng = np.random.default_rng(4)
    sc = S.random_gaussians(10, 0.1, rng)
    cams = [S.Camera(30 + i, 50, 60.0, 61.0, 25.0, 15.0, *S.look_at([0.5, 0.1 * i, 0]))
            for i in range(3)]
    v = serve._view_table(serve.RenderRequest(sc.means, sc.prec, sc.logw, cams))
    assert v.dtype.itemsize == ctypes.sizeof(N.View)
    c = (N.View * 3).from_buffer(v)
    assert [c[i].height for i in range(3)] == [30, 31, 32]
    assert abs(c[2].fy - 61.0) < 1e-6 and c[1].flags == N.FE_VIEW_NO_GRAD
    assert np.allclose(list(c[2].quat), cams[2].quat) and np.allclose(list(c[2].trans), cams[2].trans)


def test_footprint_matches_the_library_admission_unit():
    from fuzzy_ellipses import _native as N
    lib = N.load()
    rng = np.random.default_rng(5)
    for bwd in (False, True):
        for n, nv, side in ((20, 1, 96), (700, 5, 211), (2000, 32, 480)):
            sc = S.random_gaussians(n, 0.1, rng)
            cams = [S.Camera(side, side + 7, float(side), float(side), side / 2, side / 2,
                             *S.look_at([0.5, 0.0, 0.1 * i])) for i in range(nv)]
            tg = [np.zeros((side, side + 7), np.float32) for _ in cams] if bwd else None
            req = serve.RenderRequest(sc.means, sc.prec, sc.logw, cams, tg)
            views = serve._view_table(req)
            r = N.Request()
            r.n_gaussians, r.n_views = n, nv
            r.views = views.ctypes.data
            tptr = (ctypes.c_void_p * nv)(*([1] * nv))
            r.targets = ctypes.cast(tptr, ctypes.c_void_p) if bwd else None
            for tile in (8, 16):
                assert lib.fe_request_footprint(ctypes.byref(r), tile, tile) == \
                    serve.estimate_footprint(req, tile)


def test_jax_binding_reports_missing_jax():
    import importlib
    try:
        import jax  # noqa: F401
        pytest.skip("jax is installed: the binding is importable")
    except ImportError:
        pass
    with pytest.raises(ImportError, match="JAX"):
        importlib.import_module("fuzzy_ellipses.jax_ops")


@pytest.mark.parametrize("n", [1, 2, 7, 8, 9, 16])
def test_running_sums_give_the_column_moments(n):
    """The backward pixel loop (blend_bwd.cu) keeps, per lane of a pixel pair, the running sums
    S0 = sum h, C1 = sum of S0, C2 = sum of C1 over the row's n pair steps, and forms
    sum h du = D0 S0 + 2 (n S0 - C1) and
    sum h du^2 = D0^2 S0 + 4 D0 (n S0 - C1) + 4 (n^2 S0 - (2n+1) C1 + 2 C2)
    with du = D0 + 2 i at step i. Checked here in float64 against the direct sums."""
    rng = np.random.default_rng(n)
    h = rng.normal(size=n)
    d0 = -7.5 + rng.integers(0, 2)
    s0 = c1 = c2 = 0.0
    for i in range(n):
        s0 += h[i]
        c1 += s0
        c2 += c1
    du = d0 + 2.0 * np.arange(n)
    i1 = n * s0 - c1
    i2 = n * n * s0 - (2 * n + 1) * c1 + 2 * c2
    assert np.isclose(d0 * s0 + 2 * i1, (h * du).sum(), rtol=1e-12, atol=1e-12)
    assert np.isclose(d0 * d0 * s0 + 4 * d0 * i1 + 4 * i2, (h * du * du).sum(), rtol=1e-12,
                      atol=1e-10)
