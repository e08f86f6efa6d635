"""Batched renders of uneven scenes and cameras equal the plain per-call renders; the batch runs
without host synchronisation and replays from a CUDA graph.

The blend evaluates records in pairs taken from the global key list, so a view's records pair
up differently inside a batch than alone and its float32 sums are associated differently: the
two agree to rounding (checked at 1e-6), and each is bit-for-bit repeatable."""

import numpy as np
import pytest
import torch

import fuzzy_ellipses as fe
from fuzzy_ellipses import synthetic as S
from tests.helpers import scene_to_dev

pytestmark = pytest.mark.gpu


def make_batch(dev, n_scenes=6, seed=0, tile=(16, 16), **kw):
    items = S.config3(seed=seed, n_scenes=n_scenes)
    means, prec, logw, scenes, views = [], [], [], [], []
    off = 0
    for si, (sc, cams) in enumerate(items):
        means.append(sc.means); prec.append(sc.prec); logw.append(sc.logw)
        scenes.append((off, sc.n))
        off += sc.n
        for c in cams:
            views.append(dict(scene=si, height=c.height, width=c.width, fx=c.fx, fy=c.fy, cx=c.cx,
                              cy=c.cy, quat=c.quat, trans=c.trans))
    b = fe.Batch(scenes, views, tile=tile, **kw)
    tens = [torch.from_numpy(np.concatenate(x)).to(dev) for x in (means, prec, logw)]
    return b, items, views, tens


@pytest.mark.parametrize("tile", [(8, 8), (16, 16), (32, 8)])
def test_batch_equals_single_renders(cuda_device, tile):
    dev = cuda_device
    b, items, views, (m, p, w) = make_batch(dev, tile=tile)
    depth, alpha = b.forward(m, p, w)
    st = b.status()
    assert st["device_error"] == 0 and st["num_keys"] == st["want_keys"]
    vi = 0
    for si, (sc, cams) in enumerate(items):
        ms, ps, ws = scene_to_dev(sc, dev)
        for c in cams:
            d1, a1 = fe.render_forward(ms, ps, ws, c.fx, c.fy, c.cx, c.cy, c.quat, c.trans,
                                       c.height, c.width, tile=tile)
            torch.testing.assert_close(b.view_image(depth, vi), d1, rtol=1e-6, atol=1e-7)
            torch.testing.assert_close(b.view_image(alpha, vi), a1, rtol=0, atol=1e-6)
            vi += 1
    depth2, alpha2 = b.forward(m, p, w)
    assert torch.equal(depth2, depth) and torch.equal(alpha2, alpha)


def test_batch_backward_equals_sum_of_single(cuda_device):
    dev = cuda_device
    b, items, views, (m, p, w) = make_batch(dev, n_scenes=4, seed=1)
    stats = torch.empty(3 * b.n_pixels, device=dev)
    depth, alpha = b.forward(m, p, w, stats=stats)
    gen = torch.Generator(device=dev).manual_seed(0)
    ga = torch.randn(b.n_pixels, device=dev, generator=gen)
    gd = torch.zeros(b.n_pixels, device=dev)
    gm, gp, gw = b.backward(m, p, w, depth, alpha, stats, gd, ga)
    rm, rp, rw = torch.zeros_like(m), torch.zeros_like(p), torch.zeros_like(w)
    off, vi = 0, 0
    for sc, cams in items:
        sl = slice(off, off + sc.n)
        for c in cams:
            mm, pp, ww = [t[sl].clone().requires_grad_() for t in (m, p, w)]
            _, a = fe.render(mm, pp, ww, c.fx, c.fy, c.cx, c.cy, c.quat, c.trans, c.height, c.width)
            (a * b.view_image(ga, vi)).sum().backward()
            rm[sl] += mm.grad; rp[sl] += pp.grad; rw[sl] += ww.grad
            vi += 1
        off += sc.n
    for x, y in ((gm, rm), (gp, rp), (gw, rw)):
        assert float((x - y).norm() / y.norm()) < 1e-4


def test_batch_replays_from_cuda_graph(cuda_device):
    dev = cuda_device
    b, items, views, (m, p, w) = make_batch(dev, n_scenes=5, seed=2)
    depth = torch.empty(b.n_pixels, device=dev)
    alpha = torch.empty(b.n_pixels, device=dev)
    ref_d, ref_a = b.forward(m, p, w)
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        b.forward(m, p, w, depth, alpha)  # warm-up on the capture stream
    torch.cuda.current_stream().wait_stream(s)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        b.forward(m, p, w, depth, alpha)
    depth.zero_(); alpha.zero_()
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(depth, ref_d) and torch.equal(alpha, ref_a)


def test_backward_reusing_the_forward_binning_equals_recomputing(cuda_device):
    """FE_FLAG_KEEP_BINNING: the backward right after a forward on the same tensors reuses its
    binning and gives the same gradients; a backward on other tensors recomputes."""
    dev = cuda_device
    ref, _, _, (m, p, w) = make_batch(dev, n_scenes=4, seed=2)
    keep, _, _, _ = make_batch(dev, n_scenes=4, seed=2, keep_binning=True)
    gen = torch.Generator(device=dev).manual_seed(3)
    outs = []
    for b in (ref, keep):
        stats = torch.empty(3 * b.n_pixels, device=dev)
        depth, alpha = b.forward(m, p, w, stats=stats)
        gd = torch.randn(b.n_pixels, device=dev, generator=gen) * 1e-2
        ga = torch.randn(b.n_pixels, device=dev, generator=gen)
        gen.manual_seed(3)
        outs.append(b.backward(m, p, w, depth, alpha, stats, gd, ga))
    # (the record gradients are accumulated with atomics: equal up to summation order)
    for x, y in zip(*outs):
        assert float((x - y).norm()) <= 1e-5 * float(y.norm()) + 1e-12
    # Other tensors (same values, new storage): the kept binning is not used for them.
    m2, p2, w2 = m.clone() * 1.0001, p.clone(), w.clone()
    stats = torch.empty(3 * keep.n_pixels, device=dev)
    depth, alpha = ref.forward(m2, p2, w2, stats=stats)
    gd = torch.randn(keep.n_pixels, device=dev, generator=gen) * 1e-2
    ga = torch.randn(keep.n_pixels, device=dev, generator=gen)
    g_ref = ref.backward(m2, p2, w2, depth, alpha, stats, gd, ga)
    g_keep = keep.backward(m2, p2, w2, depth, alpha, stats, gd, ga)  # last forward was on m, p, w
    for x, y in zip(g_ref, g_keep):
        assert float((x - y).norm()) <= 1e-5 * float(y.norm()) + 1e-12


def _host_forward_matches(b, m, p, w, pinned=True):
    depth, alpha = b.forward(m, p, w)
    torch.cuda.synchronize()
    if pinned:
        # pinned inputs too: the preprocess reads them through their device mapping
        hd, ha = b.forward_host(m.cpu().pin_memory(), p.cpu().pin_memory(), w.cpu().pin_memory())
        assert hd.is_pinned() and ha.is_pinned()
    else:
        hd = torch.full((b.n_pixels,), -7.0)
        ha = torch.full((b.n_pixels,), -7.0)
        b.forward_host(m.cpu(), p.cpu(), w.cpu(), hd, ha)
    # The banded blend evaluates every tile exactly as the one-launch blend does.
    assert torch.equal(hd, depth.cpu()) and torch.equal(ha, alpha.cpu())
    st = b.status()
    assert st["device_error"] == 0


@pytest.mark.parametrize("layout", ["depth_first", "alpha_first", "gapped"])
def test_forward_host_images_in_one_buffer(cuda_device, layout):
    """Depth and alpha as two views of one pinned host buffer, in either order and with a gap
    between them: the blend stores into both through the buffer's device mapping and writes
    nothing between them."""
    b, items, views, (m, p, w) = make_batch(cuda_device, n_scenes=4, seed=4)
    depth, alpha = b.forward(m, p, w)
    torch.cuda.synchronize()
    n = b.n_pixels
    gap = 1000 if layout == "gapped" else 0
    buf = torch.full((2 * n + gap,), -7.0).pin_memory()
    lo, hi = buf[:n], buf[n + gap:]
    hd, ha = (hi, lo) if layout == "alpha_first" else (lo, hi)
    b.forward_host(m.cpu(), p.cpu(), w.cpu(), hd, ha)
    assert torch.equal(hd, depth.cpu()) and torch.equal(ha, alpha.cpu())
    if gap:
        assert torch.all(buf[n:n + gap] == -7.0)  # nothing written between the two images
    assert b.status()["device_error"] == 0


@pytest.mark.parametrize("pinned", [True, False])
def test_forward_host_equals_device_forward(cuda_device, pinned):
    b, items, views, (m, p, w) = make_batch(cuda_device, n_scenes=6, seed=3)
    _host_forward_matches(b, m, p, w, pinned)
    _host_forward_matches(b, m, p, w, pinned)  # repeat: counters, streams and events reused


def test_forward_host_bands_within_and_across_views(cuda_device):
    dev = cuda_device
    scene, cams = S.config1(seed=0)
    m, p, w = [torch.from_numpy(x).to(dev) for x in (scene.means, scene.prec, scene.logw)]
    # 16 views of 640x480: several bands, each ending at a view or tile-row boundary.
    views = [dict(scene=0, height=c.height, width=c.width, fx=c.fx, fy=c.fy, cx=c.cx, cy=c.cy,
                  quat=c.quat, trans=c.trans) for c in cams]
    # Pageable outputs take the banded copies; pinned ones the direct stores.
    b = fe.Batch([(0, scene.n)], views, tile=(16, 16))
    _host_forward_matches(b, m, p, w, pinned=False)
    _host_forward_matches(b, m, p, w, pinned=True)
    # One large view (1280x968: the last tile row is partial): bands of tile rows inside it.
    c = cams[0]
    big = [dict(scene=0, height=968, width=1280, fx=2 * c.fx, fy=2 * c.fy, cx=640.0, cy=484.0,
                quat=c.quat, trans=c.trans)]
    b.reset([(0, scene.n)], big)
    _host_forward_matches(b, m, p, w, pinned=False)
    _host_forward_matches(b, m, p, w, pinned=True)
    # Views laid out in reverse order in the output: no band spans two views.
    n_px = [v["height"] * v["width"] for v in views[:5]]
    offs = np.cumsum([0] + n_px[::-1][:-1])[::-1]
    rev = [dict(v, pixel_offset=int(o)) for v, o in zip(views[:5], offs)]
    b2 = fe.Batch([(0, scene.n)], rev, tile=(32, 8))
    _host_forward_matches(b2, m, p, w, pinned=False)
    _host_forward_matches(b2, m, p, w, pinned=True)


def test_forward_host_mixed_and_ragged_outputs(cuda_device):
    """One pinned and one pageable output take the banded copies; ragged widths (not a multiple
    of the thread's pixel vector) and an output base off the vector alignment take the per-pixel
    stores at row ends and the direct path's unaligned rows."""
    dev = cuda_device
    scene, cams = S.config1(seed=1)
    m, p, w = [torch.from_numpy(x).to(dev) for x in (scene.means, scene.prec, scene.logw)]
    c = cams[2]
    views = [dict(scene=0, height=h, width=wd, fx=c.fx * wd / 640, fy=c.fy * h / 480,
                  cx=wd / 2, cy=h / 2, quat=c.quat, trans=c.trans)
             for h, wd in ((131, 197), (64, 61), (250, 333))]
    b = fe.Batch([(0, scene.n)], views, tile=(16, 16), px=4)
    depth, alpha = b.forward(m, p, w)
    torch.cuda.synchronize()
    n = b.n_pixels
    hd = torch.full((n,), -7.0).pin_memory()
    ha = torch.full((n,), -7.0)
    b.forward_host(m.cpu(), p.cpu(), w.cpu(), hd, ha)
    assert torch.equal(hd, depth.cpu()) and torch.equal(ha, alpha.cpu())
    # Outputs starting one float past a 16-byte boundary of a pinned buffer.
    buf = torch.full((2 * n + 2,), -7.0).pin_memory()
    hd, ha = buf[1:n + 1], buf[n + 2:]
    b.forward_host(m.cpu(), p.cpu(), w.cpu(), hd, ha)
    assert torch.equal(hd, depth.cpu()) and torch.equal(ha, alpha.cpu())
    assert buf[0] == -7.0 and buf[n + 1] == -7.0
    assert b.status()["device_error"] == 0


_OVERFLOW_CHILD = r"""
import sys, json
sys.path[:0] = sys.argv[1:3]
import numpy as np, torch
import fuzzy_ellipses as fe
from fuzzy_ellipses import synthetic as S
scene, cams = S.config1(seed=0)
dev = torch.device("cuda")
m, p, w = [torch.from_numpy(x).to(dev) for x in (scene.means, scene.prec, scene.logw)]
views = [dict(scene=0, height=c.height, width=c.width, fx=c.fx, fy=c.fy, cx=c.cx, cy=c.cy,
              quat=c.quat, trans=c.trans) for c in cams[:4]]
out = {}
for binning in ("tiles", "radix"):
    b = fe.Batch([(0, scene.n)], views, binning=binning)
    d, a = b.forward(m, p, w)
    torch.cuda.synchronize()
    st = b.status()
    out[binning] = dict(st, finite=bool(torch.isfinite(d).all() and torch.isfinite(a).all()))
print(json.dumps(out))
"""


def test_key_overflow_is_flagged_on_both_binning_paths(cuda_device):
    """With a key budget far below the keys a batch needs (FE_KEY_BUDGET_BYTES, read once per
    process, so in a child process), both binnings keep the first keys that fit, set the
    capacity error bit, report the needed count, and render without faulting."""
    import json
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, FE_KEY_BUDGET_BYTES=str(1 << 20))  # 65,536 keys of 16 B
    r = subprocess.run([sys.executable, "-c", _OVERFLOW_CHILD, root,
                        os.path.join(root, "fuzzy-ellipses_gb300")],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    for binning, st in out.items():
        assert st["num_keys"] == 1 << 16, (binning, st)
        assert st["want_keys"] > st["num_keys"], (binning, st)
        assert st["device_error"] & 1, (binning, st)  # FE_DEVERR_CAPACITY
        assert st["finite"], (binning, st)
    assert out["tiles"]["want_keys"] == out["radix"]["want_keys"]


@pytest.mark.parametrize("tile", [(8, 8), (16, 16), (32, 8)])
def test_heavy_tiles_first_renders_identically(cuda_device, tile):
    """Taking the tiles with the most keys first changes only which CTA renders a tile, not how:
    the images are bit-identical to index order, on the batch and the single-view path."""
    dev = cuda_device
    b0, items, views, (m, p, w) = make_batch(dev, n_scenes=6, seed=4, tile=tile)
    b1, _, _, _ = make_batch(dev, n_scenes=6, seed=4, tile=tile, heavy_first=True)
    d0, a0 = b0.forward(m, p, w)
    d1, a1 = b1.forward(m, p, w)
    assert b1.status()["device_error"] == 0
    assert torch.equal(d0, d1) and torch.equal(a0, a1)
    scene, cams = S.config1(seed=3)
    ms, ps, ws = scene_to_dev(scene, dev)
    c = cams[2]
    views1 = [dict(scene=0, height=c.height, width=c.width, fx=c.fx, fy=c.fy, cx=c.cx, cy=c.cy,
                   quat=c.quat, trans=c.trans)]
    out = []
    for hf in (False, True):
        b = fe.Batch([(0, scene.n)], views1, tile=tile, heavy_first=hf)
        out.append(b.forward(ms, ps, ws))
        assert b.status()["device_error"] == 0
    assert torch.equal(out[0][0], out[1][0]) and torch.equal(out[0][1], out[1][1])
