"""The hand-written backward against torch float64 autograd of the fm_render restatement (the
stand-in for jax.grad of fm_render) and against central differences of the CUDA forward."""

import numpy as np
import pytest
import torch

import fuzzy_ellipses as fe
from fuzzy_ellipses import synthetic as S
from oracle import fm_render_torch as OT
from oracle import fm_render_np as O
from tests.helpers import scene_to_dev

pytestmark = pytest.mark.gpu
GRAD_TOL = 2e-3  # relative L2 error per parameter group


def rel(a, b):
    return float((a - b).norm() / b.norm().clamp_min(1e-30))


@pytest.fixture(scope="module")
def cfg2():
    gt, model, cams = S.config2(seed=0)
    cams = cams[::5]  # 4 of the 20 views keep the float64 autograd reference fast
    targets = []
    for c in cams:
        _, a = O.render_pinhole(gt.means, gt.prec, gt.logw, c.height, c.width, c.fx, c.fy, c.cx,
                                c.cy, c.quat, c.trans)
        targets.append((a > 0.5).astype(np.float64))
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


def oracle_loss_and_grads(model, cams, targets):
    m = torch.from_numpy(model.means).double().requires_grad_()
    p = torch.from_numpy(model.prec).double().requires_grad_()
    w = torch.from_numpy(model.logw).double().requires_grad_()
    loss = 0.0
    for c, tgt in zip(cams, targets):
        _, a = OT.render_pinhole(m, p, w, c.height, c.width, c.fx, c.fy, c.cx, c.cy,
                                 torch.from_numpy(c.quat).double(), torch.from_numpy(c.trans).double())
        loss = loss + OT.bce_silhouette_loss(a.reshape(c.height, c.width), torch.from_numpy(tgt))
    loss = loss / len(cams)
    loss.backward()
    return loss.item(), m.grad, p.grad, w.grad


def test_silhouette_bce_gradients_match_float64_autograd(cuda_device, cfg2):
    model, cams, targets = cfg2
    l_gpu, gm, gp, gw = gpu_loss_and_grads(cuda_device, model, cams, targets)
    l_ref, rm, rp, rw = oracle_loss_and_grads(model, cams, targets)
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


def test_gradients_match_central_differences(cuda_device, cfg2):
    """64 random parameters, central differences with eps = 1e-4 of the CUDA forward's loss."""
    model, cams, targets = cfg2
    dev = cuda_device
    cams, targets = cams[:2], targets[:2]
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
