"""GMM log-likelihood kernel (the reference's log_likelihood, baseline/fm_render.py:231-259)
against the float64 restatement (itself pinned to scikit-learn's score_samples).

Tolerance: the float32 kernel evaluates |U^T (mu - x)|^2 and the constants with relative error
~1e-7 each, so errors scale with the magnitude of the log terms: |ll_gpu - ll_ref| <=
2e-6 (1 + |max_i r_ij| + |ll_ref|) per point, and the same per matrix entry."""

import numpy as np
import pytest
import torch

import fuzzy_ellipses as fe
from fuzzy_ellipses import synthetic as S
from oracle import gmm_np

pytestmark = pytest.mark.gpu


def run(dev, sc, pts, matrix=False):
    m, p, w = [torch.from_numpy(np.ascontiguousarray(x)).to(dev) for x in (sc.means, sc.prec, sc.logw)]
    x = torch.from_numpy(np.ascontiguousarray(pts, np.float32)).to(dev)
    out = fe.gmm_log_likelihood(m, p, w, x, return_matrix=matrix)
    return [o.cpu().numpy() if o is not None else None for o in out]


@pytest.mark.parametrize("n,P", [(1, 1), (7, 513), (40, 4096), (1300, 3001)])
def test_point_log_likelihoods_match_oracle(cuda_device, n, P):
    rng = np.random.default_rng(n + P)
    sc = S.random_gaussians(n, 0.2, rng)
    pts = rng.uniform(-0.35, 0.35, size=(P, 3)).astype(np.float32)
    nll, ll, res = run(cuda_device, sc, pts, matrix=True)
    ref_nll, ref_res, ref_ll = gmm_np.log_likelihood(sc.means, sc.prec, sc.logw, pts)
    scale = 1 + np.abs(ref_res).max(0) + np.abs(ref_ll)
    assert np.all(np.abs(ll - ref_ll) <= 2e-6 * scale)
    assert np.all(np.abs(res - ref_res) <= 2e-6 * (1 + np.abs(ref_res)))
    assert abs(float(nll) - ref_nll) <= 2e-6 * float(scale.mean())


def test_far_points_and_a_dominant_component(cuda_device):
    """Points far from every Gaussian (log terms near -1e5) and one component that dominates by
    orders of magnitude: the online logsumexp neither underflows nor overflows."""
    rng = np.random.default_rng(9)
    sc = S.random_gaussians(30, 0.1, rng)
    sc.logw[3] = 40.0
    pts = np.concatenate([rng.uniform(-0.1, 0.1, size=(200, 3)),
                          rng.uniform(2.0, 3.0, size=(200, 3))]).astype(np.float32)
    nll, ll = run(cuda_device, sc, pts)
    _, ref_res, ref_ll = gmm_np.log_likelihood(sc.means, sc.prec, sc.logw, pts)
    assert np.all(np.isfinite(ll))
    scale = 1 + np.abs(ref_res).max(0) + np.abs(ref_ll)
    assert np.all(np.abs(ll - ref_ll) <= 2e-6 * scale)


def test_no_points(cuda_device):
    rng = np.random.default_rng(1)
    sc = S.random_gaussians(5, 0.1, rng)
    nll, ll = run(cuda_device, sc, np.zeros((0, 3), np.float32))
    assert ll.shape == (0,) and float(nll) == 0.0
