"""The hand-written backward against torch float64 autograd of the fm_render restatement (the
stand-in for jax.grad of fm_render, itself checked against central differences of the reference's
own fm_render in tests/test_oracle.py), against those reference central differences directly, and
against central differences of the CUDA forward."""

import numpy as np
import pytest
import torch

import fuzzy_ellipses as fe
from fuzzy_ellipses import synthetic as S
from oracle import fm_render_torch as OT
from oracle import fm_render_np as O
from tests.helpers import golden, golden_cameras, golden_scene, scene_to_dev

pytestmark = pytest.mark.gpu
GRAD_TOL = 2e-3  # relative L2 error per parameter group


def rel(a, b):
    return float((a - b).norm() / b.norm().clamp_min(1e-30))


@pytest.fixture(scope="module")
def cfg2():
    """The differentiable-step configuration at its stated size: the 200-Gaussian model, all 20
    views at 128x128, silhouettes (alpha > 0.5 of the ground-truth scene) as the reference's own
    fm_render rendered them."""
    g = golden()
    model = golden_scene("cfg2")
    cams = golden_cameras("cfg2")
    targets = [g["cfg2_targets"][i].astype(np.float64) for i in range(len(cams))]
    assert len(cams) == 20
    return model, cams, targets


def gpu_loss_and_grads(dev, model, cams, targets):
    m, p, w = [t.clone().requires_grad_() for t in scene_to_dev(model, dev)]
    loss = 0.0
    for c, tgt in zip(cams, targets):
        _, a = fe.render(m, p, w, c.fx, c.fy, c.cx, c.cy, c.quat, c.trans, c.height, c.width)
        loss = loss + OT.bce_silhouette_loss(a.double(), torch.from_numpy(tgt).to(dev))
    loss = loss / len(cams)
    loss.backward()
    return loss.item(), m.grad.double().cpu(), p.grad.double().cpu(), w.grad.double().cpu()


def oracle_loss_and_grads(model, cams, targets, dev="cpu"):
    """float64 autograd of the torch restatement, one view at a time (gradients accumulate), on
    ``dev`` (the GPU evaluates the float64 checker quickly for all 20 views)."""
    m = torch.from_numpy(model.means).double().to(dev).requires_grad_()
    p = torch.from_numpy(model.prec).double().to(dev).requires_grad_()
    w = torch.from_numpy(model.logw).double().to(dev).requires_grad_()
    total = 0.0
    for c, tgt in zip(cams, targets):
        _, a = OT.render_pinhole(m, p, w, c.height, c.width, c.fx, c.fy, c.cx, c.cy,
                                 torch.from_numpy(c.quat).double().to(dev),
                                 torch.from_numpy(c.trans).double().to(dev))
        loss = OT.bce_silhouette_loss(a.reshape(c.height, c.width),
                                      torch.from_numpy(tgt).to(dev)) / len(cams)
        loss.backward()
        total += loss.item()
    return total, m.grad.cpu(), p.grad.cpu(), w.grad.cpu()


def test_silhouette_bce_gradients_match_float64_autograd(cuda_device, cfg2):
    """All 20 views of the differentiable-step configuration."""
    model, cams, targets = cfg2
    l_gpu, gm, gp, gw = gpu_loss_and_grads(cuda_device, model, cams, targets)
    l_ref, rm, rp, rw = oracle_loss_and_grads(model, cams, targets, dev=cuda_device)
    assert abs(l_gpu - l_ref) <= 1e-5 * abs(l_ref)
    assert rel(gm, rm) < GRAD_TOL, rel(gm, rm)
    assert rel(gp, rp) < GRAD_TOL, rel(gp, rp)
    assert rel(gw, rw) < GRAD_TOL, rel(gw, rw)
    assert torch.all(torch.tril(gp, -1) == 0)  # like jax.grad through triu


@pytest.mark.parametrize("H,W,tile", [(64, 64, (16, 16)), (37, 53, (16, 16)), (29, 45, (8, 8)),
                                      (41, 77, (32, 8))])
def test_depth_gradients_match_float64_autograd(cuda_device, H, W, tile):
    """Ragged sizes (odd widths, partial edge tiles) on every tile shape."""
    scene, cams = S.config0(seed=1)
    c = cams[0]
    f = float(max(H, W))
    cx, cy = W / 2, H / 2
    dev = cuda_device
    _, a_ref = O.render_pinhole(scene.means, scene.prec, scene.logw, H, W, f, f, cx, cy, c.quat, c.trans)
    gen = torch.Generator().manual_seed(0)
    # Depth cotangents only where depth is meaningful (alpha > 1e-2), alpha cotangents everywhere.
    gd = torch.randn(H, W, generator=gen, dtype=torch.float64) * torch.from_numpy(a_ref > 1e-2)
    ga = torch.randn(H, W, generator=gen, dtype=torch.float64)
    m, p, w = [t.clone().requires_grad_() for t in scene_to_dev(scene, dev)]
    d, a = fe.render(m, p, w, f, f, cx, cy, c.quat, c.trans, H, W, tile=tile)
    (d.double() * gd.to(dev) + a.double() * ga.to(dev)).sum().backward()
    m64, p64, w64 = [torch.from_numpy(x).double().requires_grad_() for x in (scene.means, scene.prec, scene.logw)]
    d64, a64 = OT.render_pinhole(m64, p64, w64, H, W, f, f, cx, cy,
                                 torch.from_numpy(c.quat).double(), torch.from_numpy(c.trans).double())
    (d64 * gd + a64 * ga).sum().backward()
    assert rel(m.grad.double().cpu(), m64.grad) < GRAD_TOL
    assert rel(p.grad.double().cpu(), p64.grad) < GRAD_TOL
    assert rel(w.grad.double().cpu(), w64.grad) < GRAD_TOL


def test_gradients_match_reference_central_differences(cuda_device, cfg2):
    """The CUDA backward against float64 central differences (h = 1e-6) of the reference's own
    fm_render on 48 parameters (means, upper and strictly-lower precision entries, log-weights),
    silhouette BCE over views 0, 5, 10 and 15."""
    model, cams, targets = cfg2
    g = golden()
    views = [int(v) for v in g["cfg2_fd_views"]]
    _, gm, gp, gw = gpu_loss_and_grads(cuda_device, model, [cams[v] for v in views],
                                       [targets[v] for v in views])
    ana = []
    for kind, gi, i, j in g["cfg2_fd_params"]:
        ana.append(float(gm[gi, i] if kind == 0 else gp[gi, i, j] if kind == 1 else gw[gi]))
    ana = np.array(ana)
    fd = g["cfg2_fd_grad"]
    scale = np.abs(fd).max()
    err = np.abs(ana - fd)
    assert np.all(err <= 2e-2 * np.abs(fd) + 2e-3 * scale), (err / scale).max()
    lower = [k for k, (kind, _, i, j) in enumerate(g["cfg2_fd_params"]) if kind == 1 and i > j]
    assert np.all(ana[lower] == 0)


def test_gradients_match_central_differences(cuda_device, cfg2):
    """64 random parameters, central differences with eps = 1e-4 of the CUDA forward's loss
    (views 0 and 5 of the 20: two forwards per parameter)."""
    model, cams, targets = cfg2
    dev = cuda_device
    cams, targets = [cams[0], cams[5]], [targets[0], targets[5]]
    _, gm, gp, gw = gpu_loss_and_grads(dev, model, cams, targets)
    base = scene_to_dev(model, dev)
    tg = [torch.from_numpy(t).to(dev) for t in targets]

    def loss_at(m, p, w):
        tot = 0.0
        for c, t in zip(cams, tg):
            _, a = fe.render_forward(m, p, w, c.fx, c.fy, c.cx, c.cy, c.quat, c.trans, c.height, c.width)
            tot += OT.bce_silhouette_loss(a.double(), t).item()
        return tot / len(cams)

    rng = np.random.default_rng(3)
    n = model.n
    upper = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
    errs = []
    for _ in range(64):
        kind = rng.integers(3)
        g = int(rng.integers(n))
        m, p, w = [t.clone() for t in base]
        if kind == 0:
            k = int(rng.integers(3))
            h = 1e-4
            m[g, k] += h; lp = loss_at(m, p, w); m[g, k] -= 2 * h; lm = loss_at(m, p, w)
            ana = gm[g, k].item()
        elif kind == 1:
            i, j = upper[int(rng.integers(6))]
            h = 1e-4 * max(1.0, abs(float(p[g, i, j])))
            p[g, i, j] += h; lp = loss_at(m, p, w); p[g, i, j] -= 2 * h; lm = loss_at(m, p, w)
            ana = gp[g, i, j].item()
        else:
            h = 1e-4
            w[g] += h; lp = loss_at(m, p, w); w[g] -= 2 * h; lm = loss_at(m, p, w)
            ana = gw[g].item()
        fd = (lp - lm) / (2 * h)
        errs.append((fd, ana))
    fd, ana = np.array(errs).T
    scale = np.abs(ana).max()
    # float32 forward: the difference quotient carries ~1e-7 relative loss noise / 2e-4.
    assert np.all(np.abs(fd - ana) <= 2e-2 * np.abs(ana) + 2e-3 * scale), np.abs(fd - ana).max() / scale
