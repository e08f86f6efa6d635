"""Tile keys, sort order and tile ranges of the reference-compatible binning are bit-exact with
the reference CUDA rasterizer (golden fixtures from its own kernels) and with the C oracle."""

import os

import numpy as np
import pytest
import torch

import fuzzy_ellipses as fe
from fuzzy_ellipses import synthetic as S
from oracle import fm_render_np as O
from oracle.ref_binning import ref_binning
from tests.golden.binning_cases import binning_cases, num_stds, projection, tan_full_fov
from tests.helpers import TOL_ALPHA, TOL_DEPTH_REL, parity_errors, tile_lists_from_keys

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ref_binning_golden.npz")
CASES = {c["name"]: c for c in binning_cases()}


def gpu_binning(case):
    return fe.reference_binning(case["means"], case["scales"], case["rots"], case["view"],
                                case["proj"], case["H"], case["W"], case["tan_fovx"],
                                case["tan_fovy"], case["n_std"])


@pytest.mark.parametrize("name", sorted(CASES))
def test_reference_binning_bit_exact(cuda_device, name):
    golden = np.load(GOLDEN)
    g = gpu_binning(CASES[name])
    torch.cuda.synchronize()
    pre = f"{name}/nofma_"
    assert np.array_equal(g["radii"].cpu().numpy(), golden[pre + "radii"])
    assert np.array_equal(g["means2d"].cpu().numpy().view(np.uint32),
                          golden[pre + "means2d"].view(np.uint32))
    assert np.array_equal(g["tiles_touched"].cpu().numpy().astype(np.uint32),
                          golden[pre + "tiles_touched"])
    assert np.array_equal(g["keys"].cpu().numpy().view(np.uint64), golden[pre + "keys"])
    assert np.array_equal(g["ranges"].cpu().numpy().astype(np.uint32), golden[pre + "ranges"])


@pytest.mark.parametrize("seed", range(4))
def test_reference_binning_matches_c_oracle_random(cuda_device, seed):
    rng = np.random.default_rng(100 + seed)
    n = int(rng.integers(1, 3000))
    H, W = int(rng.integers(8, 500)), int(rng.integers(8, 700))
    f = float(rng.uniform(0.5, 1.5) * W)
    z = rng.uniform(0.1, 3.0, n)
    means = np.stack([rng.uniform(-0.8, 0.8, n) * z, rng.uniform(-0.8, 0.8, n) * z, z], 1).astype(np.float32)
    scales = np.exp(rng.uniform(np.log(1e-3), np.log(0.2), (n, 3))).astype(np.float32)
    q = rng.standard_normal((n, 4)).astype(np.float32)
    case = {"means": means, "scales": scales, "rots": q, "view": np.eye(4, dtype=np.float32),
            "proj": projection(W, H, f, f), "H": H, "W": W, "n_std": num_stds(n),
            "tan_fovx": tan_full_fov(W, f), "tan_fovy": tan_full_fov(H, f)}
    r = ref_binning(case["means"], case["scales"], case["rots"], case["view"], case["proj"], H, W,
                    case["tan_fovx"], case["tan_fovy"], case["n_std"])
    g = gpu_binning(case)
    assert g["num_keys"] == r["num_keys"]
    assert np.array_equal(g["keys"].cpu().numpy().view(np.uint64), r["keys"])
    assert np.array_equal(g["ranges"].cpu().numpy().astype(np.uint32), r["ranges"])
    assert np.array_equal(g["radii"].cpu().numpy(), r["radii"])


def test_legacy_rasterize_matches_culled_oracle(cuda_device):
    """The reference-signature entry point: reference binning, then this library's blend."""
    case = CASES["cfg0_like"]
    H, W, f = case["H"], case["W"], 200.0
    cx, cy = W / 2, H / 2
    n = case["means"].shape[0]
    logw = np.random.default_rng(7).normal(0, 0.5, n).astype(np.float32)
    rays = O.pinhole_rays(H, W, f, f, cx, cy).astype(np.float32)
    rot, trans = np.eye(3, dtype=np.float32), np.zeros(3, np.float32)
    z, a = fe.rasterize(case["means"], case["scales"], case["rots"], logw, rays, rot, trans, H, W,
                        f, f, cx, cy, 0.01, 4.5)
    torch.cuda.synchronize()
    # The binning the legacy entry used is the reference's (same floats as the wrapper builds).
    tfx, tfy, view, proj = fe.api._legacy_scalars(H, W, f, f, cx, cy, 0.01, 4.5)
    rb = ref_binning(case["means"], case["scales"], case["rots"], view, proj, H, W, tfx, tfy,
                     fe.reference_num_stds(n))
    keys = rb["keys"]
    lists = [[] for _ in range(rb["ranges"].shape[0])]
    for k in keys:
        lists[int(k >> np.uint64(32))].append(int(k & np.uint64(0xFFFFFFFF)))
    # Precision implied by (scales, rotations): Sigma = R diag(s^2) R^T, U = inv(chol(Sigma))^T.
    prec = []
    for s, qq in zip(case["scales"].astype(np.float64), case["rots"].astype(np.float64)):
        r, x, y, zq = qq
        R = np.array([[1 - 2 * (y * y + zq * zq), 2 * (x * y - r * zq), 2 * (x * zq + r * y)],
                      [2 * (x * y + r * zq), 1 - 2 * (x * x + zq * zq), 2 * (y * zq - r * x)],
                      [2 * (x * zq - r * y), 2 * (y * zq + r * x), 1 - 2 * (x * x + y * y)]])
        sig = R @ np.diag(s * s) @ R.T
        prec.append(np.linalg.inv(np.linalg.cholesky(sig)).T)
    prec = np.array(prec)
    dc, ac = O.render_culled(case["means"], prec, logw, H, W, f, f, cx, cy, [1, 0, 0, 0],
                             [0, 0, 0], [np.array(l, np.int64) for l in lists], 8, 8)
    ea, ed = parity_errors(z.cpu().numpy(), a.cpu().numpy(), dc, ac)
    assert ea <= 2 * TOL_ALPHA and ed <= TOL_DEPTH_REL, (ea, ed)


@pytest.mark.parametrize("tile", [(8, 8), (16, 16), (32, 8)])
def test_product_tile_sets_match_float64_screen_bounds(cuda_device, tile):
    """With rectangle binning, every Gaussian's tiles in the product binning (float32) form the
    rectangle of the float64 restatement of its k-sigma screen bound; boundary cases may differ by
    one tile row/column."""
    from oracle import screen_bounds as SB
    scene, cams = S.config1(seed=2)
    m, p, w = [torch.from_numpy(x).to(cuda_device) for x in (scene.means, scene.prec, scene.logw)]
    exact, total = 0, 0
    for c in cams[:6]:
        keys, _ = fe.render_binning(m, p, w, c.fx, c.fy, c.cx, c.cy, c.quat, c.trans, c.height,
                                    c.width, tile=tile, footprint="rect")
        k = keys.cpu().numpy().astype(np.uint64)
        tiles = (k >> np.uint64(32)).astype(np.int64)
        gid = (k & np.uint64(0xFFFFFFFF)).astype(np.int64)
        gx = -(-c.width // tile[0])
        rect = SB.tile_rects(scene.means, scene.prec, scene.logw, c, *tile)
        for g in range(scene.n):
            t = tiles[gid == g]
            x0, y0, x1, y1 = rect[g]
            want = {(ty * gx + tx) for ty in range(y0, y1) for tx in range(x0, x1)}
            got = set(t.tolist())
            total += 1
            if got == want:
                exact += 1
                continue
            tx, ty = t % gx, t // gx
            if len(t):
                assert tx.min() >= x0 - 1 and tx.max() <= x1 and ty.min() >= y0 - 1 and ty.max() <= y1
            assert len(got ^ want) <= max(x1 - x0, y1 - y0, 1) + 2
    assert exact >= 0.999 * total


@pytest.mark.parametrize("tile", [(8, 8), (16, 16), (32, 8)])
def test_product_row_spans_match_float64_footprint_rows(cuda_device, tile):
    """By default every Gaussian is binned, in each tile row, to the tiles its footprint ellipse
    reaches there: the product's float32 spans equal the float64 restatement's
    (screen_bounds.tile_row_spans) for at least 99.5% of the Gaussians, the others differ by
    boundary tiles only; and the spans hold about a quarter fewer keys than the rectangles."""
    from oracle import screen_bounds as SB
    scene, cams = S.config1(seed=2)
    m, p, w = [torch.from_numpy(x).to(cuda_device) for x in (scene.means, scene.prec, scene.logw)]
    exact, total, n_ell, n_rect = 0, 0, 0, 0
    for c in cams[:6]:
        args = (m, p, w, c.fx, c.fy, c.cx, c.cy, c.quat, c.trans, c.height, c.width)
        keys, _ = fe.render_binning(*args, tile=tile)
        krect, _ = fe.render_binning(*args, tile=tile, footprint="rect")
        n_ell += keys.numel()
        n_rect += krect.numel()
        k = keys.cpu().numpy().astype(np.uint64)
        tiles = (k >> np.uint64(32)).astype(np.int64)
        gid = (k & np.uint64(0xFFFFFFFF)).astype(np.int64)
        gx = -(-c.width // tile[0])
        spans = SB.tile_row_spans(scene.means, scene.prec, scene.logw, c, *tile)
        order = np.argsort(gid, kind="stable")
        starts = np.searchsorted(gid[order], np.arange(scene.n + 1))
        for g in range(scene.n):
            got = set(tiles[order[starts[g]:starts[g + 1]]].tolist())
            want = {ty * gx + tx for ty in range(spans.shape[1])
                    for tx in range(spans[g, ty, 0], spans[g, ty, 1])}
            total += 1
            if got == want:
                exact += 1
                continue
            # boundary differences only: at most two tiles per row the footprint spans
            rows = max(1, int((spans[g, :, 1] > spans[g, :, 0]).sum()))
            assert len(got ^ want) <= 2 * rows + 2, (g, len(got ^ want), rows)
    assert exact >= 0.995 * total, (exact, total)
    assert n_ell < 0.85 * n_rect, (n_ell, n_rect)


def test_eval_counts_match_float64_screen_bounds(cuda_device):
    """The benchmark's unit (evaluations of a render binned to footprint rectangles of 8x8 tiles,
    the reference rasterizer's rule) from the GPU binning equals the float64 restatement's count
    on the 16-camera workload."""
    from oracle import screen_bounds as SB
    scene, cams = S.config1(seed=0)
    m, p, w = [torch.from_numpy(x).to(cuda_device) for x in (scene.means, scene.prec, scene.logw)]
    for c in cams:
        _, ranges = fe.render_binning(m, p, w, c.fx, c.fy, c.cx, c.cy, c.quat, c.trans,
                                      c.height, c.width, tile=(8, 8), footprint="rect")
        r = ranges.cpu().numpy()
        gx = (c.width + 7) // 8
        t = np.arange(r.shape[0])
        pix = np.minimum(8, c.width - 8 * (t % gx)) * np.minimum(8, c.height - 8 * (t // gx))
        gpu = int(((r[:, 1] - r[:, 0]) * pix).sum())
        cpu = SB.evals_per_render(scene.means, scene.prec, scene.logw, c)
        assert abs(gpu - cpu) <= 1e-4 * cpu


@pytest.mark.parametrize("footprint", ["ellipse", "rect"])
@pytest.mark.parametrize("tile", [(8, 8), (16, 16), (32, 8)])
def test_tile_major_binning_equals_radix_sort(cuda_device, tile, footprint):
    """The tile-major binning (per tile row: spans filtered in id order, a ballot per tile) and
    key emission + stable radix sort give the same keys and ranges bit for bit, with footprint
    rows and with whole rectangles; the keys are ascending and every non-empty tile's range is
    exactly its run of keys."""
    scene, cams = S.config1(seed=4)
    m, p, w = [torch.from_numpy(x).to(cuda_device) for x in (scene.means, scene.prec, scene.logw)]
    for c in cams[:4]:
        args = (m, p, w, c.fx, c.fy, c.cx, c.cy, c.quat, c.trans, c.height, c.width)
        k1, r1 = fe.render_binning(*args, tile=tile, binning="tiles", footprint=footprint)
        k2, r2 = fe.render_binning(*args, tile=tile, binning="radix", footprint=footprint)
        assert torch.equal(k1, k2) and torch.equal(r1, r2)
        k = k1.cpu().numpy().astype(np.uint64)
        assert np.all(k[1:] > k[:-1])
        r = r1.cpu().numpy()
        tiles = (k >> np.uint64(32)).astype(np.int64)
        first = np.searchsorted(tiles, np.arange(r.shape[0]), side="left")
        last = np.searchsorted(tiles, np.arange(r.shape[0]), side="right")
        nonempty = last > first
        assert np.array_equal(r[nonempty, 0], first[nonempty])
        assert np.array_equal(r[nonempty, 1], last[nonempty])
        assert not r[~nonempty].any()


@pytest.mark.parametrize("tile,n_views,n_gauss", [((16, 16), 6, 1000), ((16, 16), 16, 1000),
                                                  ((8, 8), 16, 1000), ((16, 16), 4, 3000)])
def test_tile_major_batch_equals_radix_batch(cuda_device, tile, n_views, n_gauss):
    """A batch binned tile-major renders bit-identically to the same batch binned by radix sort
    (same keys, so the same tile records and the same evaluation order). The cases cover rows
    split over several emission blocks, whole 40- and 80-tile rows, and rows filtered in
    several segments of records (3000 Gaussians)."""
    scene, cams = S.config1(seed=5)
    if n_gauss != scene.n:
        scene = S.random_gaussians(n_gauss, 0.3, np.random.default_rng(5))
    m, p, w = [torch.from_numpy(x).to(cuda_device) for x in (scene.means, scene.prec, scene.logw)]
    views = [dict(scene=0, height=c.height, width=c.width, fx=c.fx, fy=c.fy, cx=c.cx, cy=c.cy,
                  quat=c.quat, trans=c.trans) for c in cams[:n_views]]
    out = []
    for binning in ("tiles", "radix"):
        b = fe.Batch([(0, scene.n)], views, tile=tile, binning=binning)
        d, a = b.forward(m, p, w)
        st = b.status()
        assert st["device_error"] == 0
        out.append((d, a, st["num_keys"]))
    assert out[0][2] == out[1][2]
    assert torch.equal(out[0][0], out[1][0]) and torch.equal(out[0][1], out[1][1])


@pytest.mark.parametrize("tile", [(16, 16), (8, 8)])
def test_many_view_batch_row_bases_equal_radix_batch(cuda_device, tile):
    """Past the view count where the tile-major binning first forms every row's key base
    (row_offsets_kernel, view_bases_kernel), a batch of 60 uneven views of 12 scenes renders
    bit-identically to the radix-sorted batch, in index order and heaviest tiles first. These
    views are at most 32 tiles wide (256 pixels in 8x8 tiles is exactly 32), so the emission is
    the warp-per-row kernel."""
    items = S.config3(seed=7, n_scenes=12)
    means, prec, logw, scenes, views = [], [], [], [], []
    off = 0
    for si, (sc, cams) in enumerate(items):
        means.append(sc.means); prec.append(sc.prec); logw.append(sc.logw)
        scenes.append((off, sc.n))
        off += sc.n
        for c in cams:
            views.append(dict(scene=si, height=c.height, width=c.width, fx=c.fx, fy=c.fy,
                              cx=c.cx, cy=c.cy, quat=c.quat, trans=c.trans))
    while len(views) < 60:  # repeat poses until past the threshold
        views.append(dict(views[len(views) % 20]))
    m, p, w = [torch.from_numpy(np.concatenate(x)).to(cuda_device) for x in (means, prec, logw)]
    out = []
    for binning, heavy in (("radix", False), ("tiles", False), ("tiles", True)):
        b = fe.Batch(scenes, views, tile=tile, binning=binning, heavy_first=heavy)
        assert binning != "tiles" or b.launches_per_forward == 5
        d, a = b.forward(m, p, w)
        st = b.status()
        assert st["device_error"] == 0 and st["num_keys"] == st["want_keys"]
        out.append((d, a, st["num_keys"]))
    for o in out[1:]:
        assert o[2] == out[0][2]
        assert torch.equal(o[0], out[0][0]) and torch.equal(o[1], out[0][1])


def _footprint_scenes():
    rng = np.random.default_rng(21)
    out = {}
    scene, cams = S.config0(seed=3)
    out["config0"] = (scene, cams[0])
    sub = S.random_gaussians(60, 0.1, rng, scale_lo=0.002, scale_hi=0.006)
    q, t = S.look_at(0.5 * S.random_unit_vectors(1, rng)[0])
    out["subpixel"] = (sub, S.Camera(64, 80, 64.0, 64.0, 40.0, 32.0, q, t))
    thin = S.random_gaussians(60, 0.1, rng, scale_lo=0.001, scale_hi=0.05)
    q, t = S.look_at(0.45 * S.random_unit_vectors(1, rng)[0])
    out["elongated"] = (thin, S.Camera(96, 120, 110.0, 110.0, 60.0, 48.0, q, t))
    # the camera inside one Gaussian's k-sigma region and beside others: unbounded footprints
    means = np.array([[0.3, 0.0, 0.02], [0.0, 0.0, 0.6], [0.05, -0.04, 0.3]], np.float32)
    prec = np.stack([np.triu(np.eye(3) / 0.1), np.triu(np.eye(3) / 0.05),
                     np.triu(np.eye(3) / 0.02)]).astype(np.float32)
    logw = np.array([0.0, 0.5, -0.3], np.float32)
    out["straddling"] = (S.Scene(means, prec, logw),
                         S.Camera(40, 48, 40.0, 40.0, 24.0, 20.0, np.array([1, 0, 0, 0], np.float32),
                                  np.zeros(3, np.float32)))
    return out


@pytest.mark.parametrize("cull", ["eps", "nstd"])
@pytest.mark.parametrize("tile", [(8, 8), (16, 16), (32, 8)])
@pytest.mark.parametrize("name", ["config0", "subpixel", "elongated", "straddling"])
def test_footprint_rows_list_every_pixel_above_the_cut_off(cuda_device, name, tile, cull):
    """Footprint-row binning is conservative: wherever a Gaussian's peak density along a pixel's
    ray clears the cut-off (its Mahalanobis distance below k, by 1e-5 in k^2), the Gaussian is
    listed for that pixel's tile; on config-0, sub-pixel, strongly elongated and
    camera-straddling Gaussians, every tile shape and both cut-off modes (dense float64 oracle
    over every pixel)."""
    scene, cam = _footprint_scenes()[name]
    m, p, w = [torch.from_numpy(x).to(cuda_device) for x in (scene.means, scene.prec, scene.logw)]
    param = 1e-7 if cull == "eps" else 3.0
    keys, ranges = fe.render_binning(m, p, w, cam.fx, cam.fy, cam.cx, cam.cy, cam.quat, cam.trans,
                                     cam.height, cam.width, cull=cull, cull_param=param,
                                     tile=tile)
    lists = tile_lists_from_keys(keys, ranges.shape[0])
    rays = O.pinhole_rays(cam.height, cam.width, cam.fx, cam.fy, cam.cx, cam.cy) @ \
        O.quat_to_rot(cam.quat)
    _, stds = O.ray_gaussian_terms(rays, np.tile(cam.trans.astype(np.float64), (rays.shape[0], 1)),
                                   scene.means, scene.prec, scene.logw)
    logw = scene.logw.astype(np.float64)[:, None]
    d0 = 2.0 * (logw - stds)  # Mahalanobis distance of each ray's peak, squared
    k2 = 2.0 * (logw - np.log(param)) if cull == "eps" else np.full_like(logw, param * param)
    need = d0 < k2 - 1e-5
    gx = -(-cam.width // tile[0])
    v, u = np.divmod(np.arange(cam.height * cam.width), cam.width)
    tid = (v // tile[1]) * gx + u // tile[0]
    listed = [set(l.tolist()) for l in lists]
    for g in range(scene.n):
        for t in np.unique(tid[need[g]]):
            assert g in listed[t], (name, tile, cull, g, int(t))


def test_footprint_rows_and_rectangles_render_alike(cuda_device):
    """A batch binned to footprint rows and the same batch binned to whole rectangles
    (FE_FLAG_RECT_BINNING) render alike: the tiles the rows leave out hold only pixels where the
    dropped Gaussian's density is below the cut-off, so alpha moves by far less than its 1e-5
    tolerance and depth by far less than its 1e-4 (where alpha > 1e-3); the forward statistics
    and the backward's gradients agree as well."""
    scene, cams = S.config1(seed=6)
    m, p, w = [torch.from_numpy(x).to(cuda_device) for x in (scene.means, scene.prec, scene.logw)]
    views = [dict(scene=0, height=c.height, width=c.width, fx=c.fx, fy=c.fy, cx=c.cx, cy=c.cy,
                  quat=c.quat, trans=c.trans) for c in cams[:4]]
    out = {}
    for fp in ("ellipse", "rect"):
        b = fe.Batch([(0, scene.n)], views, footprint=fp, keep_binning=True)
        stats = torch.empty(3 * b.n_pixels, device=cuda_device)
        d, a = b.forward(m, p, w, stats=stats)
        gen = torch.Generator(device=cuda_device).manual_seed(3)
        gd = torch.randn(b.n_pixels, device=cuda_device, generator=gen) * (a > 1e-3)
        ga = torch.randn(b.n_pixels, device=cuda_device, generator=gen)
        grads = b.backward(m, p, w, d, a, stats, gd, ga)
        st = b.status()
        assert st["device_error"] == 0
        out[fp] = (d, a, grads, st["num_keys"])
        b.close()
    (d0, a0, g0, k0), (d1, a1, g1, k1) = out["ellipse"], out["rect"]
    assert k0 < 0.85 * k1
    assert float((a0 - a1).abs().max()) <= 1e-6
    mask = a1 > 1e-3
    assert float(((d0 - d1).abs()[mask] / d1[mask]).max()) <= 1e-5
    for x, y in zip(g0, g1):
        assert float((x - y).norm() / y.norm()) <= 1e-4
