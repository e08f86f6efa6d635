"""Scene-parameter adapters (precision factor from scales + rotations, pose transforms of
points): forward and backward kernels against float64 torch autograd of the oracle
restatements, and the reference's optimisation chain end to end (object pose -> means,
scales + rotations -> precision, render, silhouette BCE, gradients to every parameter)."""

import numpy as np
import pytest
import torch

import fuzzy_ellipses as fe
from fuzzy_ellipses import adapters as A
from fuzzy_ellipses import synthetic as S
from oracle import adapters_torch as AT
from oracle import fm_render_torch as OT

pytestmark = pytest.mark.gpu
GRAD_TOL = 2e-3


def rel(a, b):
    return float((a - b).norm() / b.norm().clamp_min(1e-30))


def random_params(n, seed):
    g = torch.Generator().manual_seed(seed)
    s = torch.exp(torch.empty(n, 3, dtype=torch.float64).uniform_(np.log(0.005), np.log(0.03), generator=g))
    q = torch.randn(n, 4, generator=g, dtype=torch.float64)
    return s, q


def test_prec_from_scale_rot_matches_oracle(cuda_device):
    s, q = random_params(2000, 0)
    U = A.prec_from_scale_rot(s.float().to(cuda_device), q.float().to(cuda_device)).cpu().double()
    ref = AT.prec_from_scale_rot(s.float().double(), q.float().double())
    assert torch.all(torch.tril(U, -1) == 0)
    assert rel(U, ref) < 1e-6
    assert float(((U - ref).abs() / ref.abs().clamp_min(1e-3 * ref.abs().max())).max()) < 1e-5


def test_prec_from_scale_rot_backward_matches_autograd(cuda_device):
    s, q = random_params(500, 1)
    s32, q32 = s.float(), q.float()
    G = torch.randn(500, 3, 3, dtype=torch.float64, generator=torch.Generator().manual_seed(2))
    sd = s32.to(cuda_device).requires_grad_()
    qd = q32.to(cuda_device).requires_grad_()
    (A.prec_from_scale_rot(sd, qd).double() * G.to(cuda_device)).sum().backward()
    s64 = s32.double().requires_grad_()
    q64 = q32.double().requires_grad_()
    (AT.prec_from_scale_rot(s64, q64) * G).sum().backward()
    assert rel(sd.grad.cpu().double(), s64.grad) < 1e-5
    assert rel(qd.grad.cpu().double(), q64.grad) < 1e-5


@pytest.mark.parametrize("inverse", [False, True])
def test_transform_points_forward_and_backward(cuda_device, inverse):
    g = torch.Generator().manual_seed(3)
    pts = torch.randn(10003, 3, generator=g, dtype=torch.float64).float()  # a ragged tail
    pose = torch.cat([torch.randn(3, generator=g, dtype=torch.float64),
                      torch.randn(4, generator=g, dtype=torch.float64)]).float()
    G = torch.randn(10003, 3, generator=g, dtype=torch.float64)
    f = A.transform_points_by_inv if inverse else A.transform_points
    fr = AT.transform_points_by_inv if inverse else AT.transform_points
    pd = pts.to(cuda_device).requires_grad_()
    posed = pose.to(cuda_device).requires_grad_()
    out = f(posed, pd)
    (out.double() * G.to(cuda_device)).sum().backward()
    p64 = pts.double().requires_grad_()
    pose64 = pose.double().requires_grad_()
    ref = fr(pose64, p64)
    (ref * G).sum().backward()
    assert rel(out.detach().cpu().double(), ref.detach()) < 1e-6
    assert rel(pd.grad.cpu().double(), p64.grad) < 1e-6
    assert rel(posed.grad.cpu().double(), pose64.grad) < 1e-6


def test_reference_optimisation_chain_gradients(cuda_device):
    """jax_objective of the reference notebook (cell 12), restated: means in object frame moved
    by the object pose, precision from scales + rotations, one camera, mean silhouette BCE."""
    dev = cuda_device
    rng = np.random.default_rng(5)
    n = 60
    means = rng.uniform(-0.08, 0.08, size=(n, 3)).astype(np.float32)
    s, q = random_params(n, 6)
    s, q = s.float(), q.float()
    logw = rng.normal(0, 0.5, size=n).astype(np.float32)
    obj_pose = np.concatenate([[0.01, -0.02, 0.015], S.rot_to_quat(S.quat_to_rot([0.9, 0.1, 0.2, 0.3]))]).astype(np.float32)
    cam = S.Camera(96, 96, 96.0, 96.0, 48.0, 48.0, *S.look_at([0.45, 0.1, 0.2]))
    # Target: the silhouette of slightly different ground-truth parameters, as in the reference
    # loop. (A random target would put target-1 pixels in the far field, where the BCE gradient
    # per pixel is O(1) for alphas between the 3e-8 clip and the renderer's 1e-7 density cut-off,
    # so a dense and a culled render differ there by construction.)
    with torch.no_grad():
        gt_means = torch.from_numpy(means).double() + 0.004
        gt_U = AT.prec_from_scale_rot(s.double(), q.double())
        gt_mw = AT.transform_points(torch.from_numpy(obj_pose).double(), gt_means)
        _, a_gt = OT.render_pinhole(gt_mw, gt_U, torch.from_numpy(logw).double(), 96, 96, cam.fx,
                                    cam.fy, cam.cx, cam.cy, torch.from_numpy(cam.quat).double(),
                                    torch.from_numpy(cam.trans).double())
    target = (a_gt.reshape(96, 96) > 0.5).double()

    def chain(m, sc, qu, w, pose, render):
        mw = (AT if render is None else A).transform_points(pose, m)
        U = (AT if render is None else A).prec_from_scale_rot(sc, qu)
        if render is None:
            _, a = OT.render_pinhole(mw, U, w, 96, 96, cam.fx, cam.fy, cam.cx, cam.cy,
                                     torch.from_numpy(cam.quat).double(),
                                     torch.from_numpy(cam.trans).double())
            a = a.reshape(96, 96)
            return OT.bce_silhouette_loss(a, target)
        _, a = fe.render(mw, U, w, cam.fx, cam.fy, cam.cx, cam.cy, cam.quat, cam.trans, 96, 96)
        a = a.double().clamp(3e-8, 1 - 3e-8)
        t = target.to(dev)
        return -(t * torch.log(a) + (1 - t) * torch.log(1 - a)).mean()

    gpu = [torch.from_numpy(np.asarray(x)).to(dev).float().requires_grad_()
           for x in (means, s, q, logw, obj_pose)]
    chain(*gpu, render=True).backward()
    cpu = [torch.from_numpy(np.asarray(x)).double().requires_grad_() for x in (means, s, q, logw, obj_pose)]
    chain(*cpu, render=None).backward()
    for name, a, b in zip(("means", "scales", "quats", "logw", "pose"), gpu, cpu):
        assert rel(a.grad.cpu().double(), b.grad) < GRAD_TOL, name
