"""Float64 restatement of the reference's GMM log-likelihood (test infrastructure only).

``log_likelihood`` follows baseline/fm_render.py:231-259 operation for operation: triu of
prec_full, weights = softmax(logw), per (Gaussian, point) ``-0.5 (|prc p|^2 + 3 log 2 pi) +
log w + log prod |diag prc|`` with prc = triu(prec_full)^T and p = mean - point, and the result
``(-mean_j logsumexp_i res[i, j], res)``.
"""

from __future__ import annotations

import numpy as np


def log_likelihood(means, prec_full, weights_log, points):
    means = np.asarray(means, np.float64)
    prec = np.triu(np.asarray(prec_full, np.float64))
    wl = np.asarray(weights_log, np.float64)
    points = np.asarray(points, np.float64)
    w = np.exp(wl - wl.max())
    w = w / w.sum()
    res = np.empty((means.shape[0], points.shape[0]))
    for i in range(means.shape[0]):
        prc = prec[i].T
        div = np.prod(np.abs(np.diag(prc)))
        p = means[i][None, :] - points
        pteval = ((p @ prc.T) ** 2).sum(1)
        res[i] = -0.5 * (pteval + 3 * np.log(np.pi * 2)) + np.log(w[i]) + np.log(div)
    m = res.max(0)
    lse = m + np.log(np.exp(res - m).sum(0))
    return -lse.mean(), res, lse
