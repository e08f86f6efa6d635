"""Float64 restatement of the renderer's screen bounds (test infrastructure, not product code).

The product's preprocess (fuzzy-ellipses_gb300/csrc/preprocess.cu, ``footprint_and_record``)
bins a Gaussian to the tiles covered by the exact screen projection of its k-sigma ellipsoid,
k^2 = 2 (logw - ln eps) for the density cut-off eps (default 1e-7), or a fixed k. This module
restates that bound in float64 NumPy so that tests can check the GPU's tile rectangles and
``bench.py``'s reference arm can count the evaluations a render performs without a GPU.

Derivation. With the precision factor U (fm_render's prec_full, Sigma^-1 = U U^T, fm_render.py)
and the world-to-camera rotation R (camera point pc = R (mean - t)), the camera-frame precision
is M^T M with M = U^T R^T, so Sigma_c = Yh^T Yh with Yh = cof(M) / det(M). A pixel ray
r = (x, y, 1) touches the k-sigma ellipsoid iff r^T (k^2 Sigma_c - pc pc^T) r >= 0 (the dual
conic). For each image axis the bound is the pair of tangent lines of that conic:
    x = (c02 +- sqrt(c02^2 - c00 c22)) / c22,  c_ij = k^2 Sigma_c[i,j] - pc_i pc_j,
with the discriminant written as k^2 (|pz y0 - px y2|^2 - k^2 |y0 x y2|^2) (y_i: columns of Yh),
which has no cancellation. c22 >= 0 (the camera inside the ellipsoid, or the ellipsoid reaching
the camera plane) means an unbounded projection: every tile. Pixel u = fx x + cx; tiles are
widened by a 0.02 px margin, as in the product.
"""

from __future__ import annotations

import numpy as np

from .fm_render_np import quat_to_rot

DEFAULT_CULL_EPS = 1e-7
MARGIN_PX = 0.02


def _cofactor(M):
    """Cofactor matrices of a stack (..., 3, 3)."""
    C = np.empty_like(M)
    for i in range(3):
        for j in range(3):
            r = [k for k in range(3) if k != i]
            c = [k for k in range(3) if k != j]
            minor = M[..., r[0], c[0]] * M[..., r[1], c[1]] - M[..., r[0], c[1]] * M[..., r[1], c[0]]
            C[..., i, j] = (-1) ** (i + j) * minor
    return C


def tile_rects(means, prec, logw, cam, tile_w, tile_h, cull="eps", cull_param=None):
    """(N, 4) int64 tile rectangles [tx0, ty0, tx1, ty1) of every Gaussian for one camera
    (empty rectangles are all zeros)."""
    means = np.asarray(means, np.float64)
    U = np.triu(np.asarray(prec, np.float64))
    logw = np.asarray(logw, np.float64)
    gx = -(-cam.width // tile_w)
    gy = -(-cam.height // tile_h)
    R = quat_to_rot(np.asarray(cam.quat, np.float64))
    pc = (means - np.asarray(cam.trans, np.float64)) @ R.T
    M = np.swapaxes(U, -1, -2) @ R.T
    det = U[:, 0, 0] * U[:, 1, 1] * U[:, 2, 2]
    if cull == "eps":
        eps = DEFAULT_CULL_EPS if not cull_param else float(cull_param)
        k2 = 2.0 * (logw - np.log(eps))
    else:
        k = 3.0 if not cull_param else float(cull_param)
        k2 = np.full(len(logw), k * k)
    with np.errstate(all="ignore"):
        Yh = _cofactor(M) / det[:, None, None]
        y0, y1, y2 = Yh[:, :, 0], Yh[:, :, 1], Yh[:, :, 2]
        s02 = (y0 * y2).sum(1)
        s12 = (y1 * y2).sum(1)
        s22 = (y2 * y2).sum(1)
        px, py, pz = pc[:, 0], pc[:, 1], pc[:, 2]
        c22 = k2 * s22 - pz * pz
        ex = pz[:, None] * y0 - px[:, None] * y2
        ey = pz[:, None] * y1 - py[:, None] * y2
        xx = np.cross(y0, y2)
        xy = np.cross(y1, y2)
        dx = np.maximum(k2 * ((ex * ex).sum(1) - k2 * (xx * xx).sum(1)), 0.0)
        dy = np.maximum(k2 * ((ey * ey).sum(1) - k2 * (xy * xy).sum(1)), 0.0)
        c02 = k2 * s02 - px * pz
        c12 = k2 * s12 - py * pz
        xa, xb = (c02 + np.sqrt(dx)) / c22, (c02 - np.sqrt(dx)) / c22
        ya, yb = (c12 + np.sqrt(dy)) / c22, (c12 - np.sqrt(dy)) / c22
        ulo = cam.fx * np.minimum(xa, xb) + cam.cx
        uhi = cam.fx * np.maximum(xa, xb) + cam.cx
        vlo = cam.fy * np.minimum(ya, yb) + cam.cy
        vhi = cam.fy * np.maximum(ya, yb) + cam.cy
        bounded = np.isfinite(det) & (det != 0) & (c22 < 0) & np.isfinite(ulo) & \
            np.isfinite(uhi) & np.isfinite(vlo) & np.isfinite(vhi)
        tx0 = np.clip(np.floor((ulo - MARGIN_PX) / tile_w), 0, gx)
        tx1 = np.clip(np.floor((uhi + MARGIN_PX) / tile_w) + 1, 0, gx)
        ty0 = np.clip(np.floor((vlo - MARGIN_PX) / tile_h), 0, gy)
        ty1 = np.clip(np.floor((vhi + MARGIN_PX) / tile_h) + 1, 0, gy)
    rect = np.stack([np.where(bounded, tx0, 0), np.where(bounded, ty0, 0),
                     np.where(bounded, tx1, gx), np.where(bounded, ty1, gy)], 1)
    rect = np.nan_to_num(rect).astype(np.int64)
    empty = (k2 <= 0) | (rect[:, 2] <= rect[:, 0]) | (rect[:, 3] <= rect[:, 1])
    rect[empty] = 0
    return rect


def evals_per_render(means, prec, logw, cam, tile_w=8, tile_h=8, **kw):
    """Ray-Gaussian evaluations of one tile-binned render: for every Gaussian, the pixels of the
    tiles it is binned to (the metric unit of the benchmark)."""
    rect = tile_rects(means, prec, logw, cam, tile_w, tile_h, **kw)
    gx = -(-cam.width // tile_w)
    gy = -(-cam.height // tile_h)
    wcum = np.concatenate([[0], np.cumsum(np.minimum(tile_w, cam.width - tile_w * np.arange(gx)))])
    hcum = np.concatenate([[0], np.cumsum(np.minimum(tile_h, cam.height - tile_h * np.arange(gy)))])
    cols = wcum[rect[:, 2]] - wcum[rect[:, 0]]
    rows = hcum[rect[:, 3]] - hcum[rect[:, 1]]
    return int((cols * rows).sum())


def footprint_rows(means, prec, logw, cam, cull="eps", cull_param=None):
    """Row form of every Gaussian's footprint ellipse in float64, in pixel coordinates: the
    pixels (u, v) whose rays pass within Mahalanobis distance k of the mean,
    Q(u, v) = |Y (r x pc)|^2 - k^2 |M r|^2 <= 0 with r = ((u - cx)/fx, (v - cy)/fy, 1), M = U^T R^T,
    Y = cof(M) (|M r x M pc| = |Y (r x pc)|, so Q <= 0 is d0 = |y|^2 / |a|^2 <= k^2).
    Returns (ok, uc, vc, c1, hc, h2, vl, vr): at row v the ellipse spans
    uc + c1 (v - vc) -+ sqrt(hc + h2 (v - vc)^2); vl, vr are the rows of its leftmost and rightmost
    points; ok is False where the footprint is unbounded or degenerate. This restates the
    product's footprint rows (preprocess.cu, foot_rows) from the Gaussian parameters directly."""
    means = np.asarray(means, np.float64)
    U = np.triu(np.asarray(prec, np.float64))
    logw = np.asarray(logw, np.float64)
    R = quat_to_rot(np.asarray(cam.quat, np.float64))
    pc = (means - np.asarray(cam.trans, np.float64)) @ R.T
    M = np.swapaxes(U, -1, -2) @ R.T
    Y = _cofactor(M)
    if cull == "eps":
        eps = DEFAULT_CULL_EPS if not cull_param else float(cull_param)
        k2 = 2.0 * (logw - np.log(eps))
    else:
        k = 3.0 if not cull_param else float(cull_param)
        k2 = np.full(len(logw), k * k)
    r0 = np.array([-cam.cx / cam.fx, -cam.cy / cam.fy, 1.0])
    eu = np.array([1.0 / cam.fx, 0.0, 0.0])
    ev = np.array([0.0, 1.0 / cam.fy, 0.0])
    a = [M @ r for r in (r0, eu, ev)]
    y = [np.einsum("nij,nj->ni", Y, np.cross(np.broadcast_to(r, pc.shape), pc)) for r in (r0, eu, ev)]

    def q(i, j):
        return (y[i] * y[j]).sum(1) - k2 * (a[i] * a[j]).sum(1)

    with np.errstate(all="ignore"):
        Quu, Quv, Qvv, Qu, Qv, Q0 = q(1, 1), q(1, 2), q(2, 2), q(0, 1), q(0, 2), q(0, 0)
        det = Quu * Qvv - Quv * Quv
        uc = (Qv * Quv - Qu * Qvv) / det
        vc = (Qu * Quv - Qv * Quu) / det
        qc = Q0 + Qu * uc + Qv * vc
        lam = np.sqrt(-qc / (Qvv * det))
        ok = (k2 > 0) & (Quu > 0) & (Qvv > 0) & (det > 0) & (qc < 0) & np.isfinite(lam)
        # the camera outside the ellipsoid and the ellipsoid in front of it (bounded projection)
        ok &= pc[:, 2] > 0
        return (ok, uc, vc, -Quv / Quu, -qc / Quu, -det / (Quu * Quu), vc + lam * Quv,
                vc - lam * Quv)


def tile_row_spans(means, prec, logw, cam, tile_w, tile_h, margin=0.1, cull="eps",
                   cull_param=None):
    """(N, gy, 2) int64 tile spans [x0, x1) of every Gaussian in every tile row: the tiles its
    footprint ellipse reaches in the row (pixel rows [row th, row th + th - 1], widened by
    `margin` pixels), within its rectangle (tile_rects); rows outside the rectangle are empty.
    Unbounded footprints span their whole rectangle."""
    rect = tile_rects(means, prec, logw, cam, tile_w, tile_h, cull=cull, cull_param=cull_param)
    ok, uc, vc, c1, hc, h2, vl, vr = footprint_rows(means, prec, logw, cam, cull, cull_param)
    gy = -(-cam.height // tile_h)
    out = np.zeros((len(rect), gy, 2), np.int64)
    for row in range(gy):
        va, vb = float(row * tile_h), float(row * tile_h + tile_h - 1)
        inrow = (rect[:, 1] <= row) & (row < rect[:, 3]) & (rect[:, 0] < rect[:, 2])
        x0 = rect[:, 0].astype(np.float64)
        x1 = rect[:, 2].astype(np.float64)
        with np.errstate(all="ignore"):
            for edge, side in ((vl, -1.0), (vr, 1.0)):
                inside = (edge >= va) & (edge <= vb)
                dv = np.where(edge < va, va, vb) - vc
                h = np.sqrt(np.maximum(hc + h2 * dv * dv, 0.0))
                u = uc + c1 * dv + side * (h + margin)
                if side < 0:
                    t = np.floor(u / tile_w)
                    x0 = np.where(ok & ~inside & (t > x0), np.minimum(t, x1), x0)
                else:
                    t = np.floor(u / tile_w) + 1
                    x1 = np.where(ok & ~inside & (t < x1), np.maximum(t, x0), x1)
        out[:, row, 0] = np.where(inrow, x0, 0)
        out[:, row, 1] = np.where(inrow, x1, 0)
    empty = out[:, :, 1] <= out[:, :, 0]
    out[empty] = 0
    return out
