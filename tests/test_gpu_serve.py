"""Continuous-batching server: results equal the plain per-call path, are the same alone and
in a mix of concurrent requests, admission respects the HBM budget; the autotuner picks a valid
configuration."""

import numpy as np
import pytest
import torch

import fuzzy_ellipses as fe
from fuzzy_ellipses import autotune, serve
from fuzzy_ellipses import synthetic as S

pytestmark = pytest.mark.gpu


def small_stream(n, seed, backward_every=3):
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n):
        sc = S.random_gaussians(int(rng.integers(20, 300)), 0.1, rng)
        side = int(rng.integers(40, 130))
        cams = [S.Camera(side, side, float(side), float(side), side / 2, side / 2,
                         *S.look_at(0.5 * d)) for d in S.random_unit_vectors(int(rng.integers(1, 5)), rng)]
        targets = None
        if i % backward_every == 0:
            targets = [(rng.uniform(size=(c.height, c.width)) > 0.7).astype(np.float32) for c in cams]
        reqs.append(serve.RenderRequest(sc.means, sc.prec, sc.logw, cams, targets))
    return reqs


def plain(req, dev):
    m, p, w = [torch.from_numpy(x).to(dev) for x in (req.means, req.prec, req.logw)]
    if req.targets is None:
        outs = [fe.render_forward(m, p, w, c.fx, c.fy, c.cx, c.cy, c.quat, c.trans, c.height, c.width)
                for c in req.cameras]
        return [o[0].cpu().numpy() for o in outs], [o[1].cpu().numpy() for o in outs], None
    m.requires_grad_(); p.requires_grad_(); w.requires_grad_()
    loss, count, ds, als = 0.0, 0, [], []
    for c, t in zip(req.cameras, req.targets):
        d, a = fe.render(m, p, w, c.fx, c.fy, c.cx, c.cy, c.quat, c.trans, c.height, c.width)
        a64 = a.double()
        tt = torch.from_numpy(t).to(dev).double()
        ac = a64.clamp(3e-8, 1 - 3e-8)
        loss = loss - (tt * torch.log(ac) + (1 - tt) * torch.log(1 - ac)).sum()
        count += a.numel()
        ds.append(d.detach().cpu().numpy()); als.append(a.detach().cpu().numpy())
    (loss / count).backward()
    return ds, als, (float(loss.detach() / count), m.grad.cpu().numpy(), p.grad.cpu().numpy(), w.grad.cpu().numpy())


def close(a, b, rtol=1e-5, atol=1e-6):
    return np.allclose(a, b, rtol=rtol, atol=atol)


def loss_tol(alphas_1, alphas_2, targets, loss):
    """First-order bound on the BCE loss difference caused by the observed alpha differences,
    sum |dBCE/da| |a1 - a2| / count (doubled), plus 4e-6 relative for the float32 reduction.
    BCE is ill-conditioned where alpha saturates: d/da log(1 - a) = -1/(1 - a)."""
    num, count = 0.0, 0
    for a1, a2, t in zip(alphas_1, alphas_2, targets):
        a = np.clip(np.minimum(a1, a2).astype(np.float64), 3e-8, 1 - 3e-8)
        b = np.clip(np.maximum(a1, a2).astype(np.float64), 3e-8, 1 - 3e-8)
        sens = t / a + (1 - t) / (1 - b)
        num += float((sens * (b - a)).sum())
        count += t.size
    return 2.0 * num / count + 4e-6 * abs(loss)


def test_server_matches_plain_calls(cuda_device):
    reqs = small_stream(7, seed=0)
    with serve.RenderServer(device=cuda_device, lanes=2) as srv:
        futs = [srv.submit(r) for r in reqs]
        results = [f.result(timeout=120) for f in futs]
    for req, res in zip(reqs, results):
        ds, als, g = plain(req, cuda_device)
        for d1, d2 in zip(res.depth, ds):
            assert close(d1, d2)
        for a1, a2 in zip(res.alpha, als):
            assert close(a1, a2, atol=1e-6)
        if g is not None:
            assert abs(res.loss - g[0]) <= loss_tol(res.alpha, als, req.targets, g[0])
            for x, y in zip((res.grad_means, res.grad_prec, res.grad_logw), g[1:]):
                assert np.linalg.norm(x - y) <= 1e-4 * np.linalg.norm(y) + 1e-12


def test_same_result_alone_and_in_mix(cuda_device):
    reqs = small_stream(16, seed=1)
    probe = reqs[6]  # a backward request (6 % 3 == 0)
    assert probe.backward
    with serve.RenderServer(device=cuda_device, lanes=1) as srv:
        alone = srv.submit(probe).result(timeout=120)
    with serve.RenderServer(device=cuda_device, lanes=3, max_batch_views=24) as srv:
        futs = [srv.submit(r) for r in reqs]
        mixed = futs[6].result(timeout=120)
        [f.result(timeout=120) for f in futs]
        assert srv.stats()["batches"] >= 2
    for a, b in zip(alone.alpha, mixed.alpha):
        assert close(a, b, rtol=0, atol=1e-6)
    for a, b in zip(alone.depth, mixed.depth):
        assert close(a, b, rtol=1e-6, atol=1e-7)
    assert abs(alone.loss - mixed.loss) <= loss_tol(alone.alpha, mixed.alpha, probe.targets,
                                                    alone.loss)
    for x, y in ((alone.grad_means, mixed.grad_means), (alone.grad_prec, mixed.grad_prec),
                 (alone.grad_logw, mixed.grad_logw)):
        assert np.linalg.norm(x - y) <= 1e-5 * np.linalg.norm(y) + 1e-12


def test_budget_admission_serialises_and_rejects(cuda_device):
    reqs = small_stream(6, seed=2, backward_every=100)
    need = max(serve.estimate_footprint(r) for r in reqs)
    with serve.RenderServer(device=cuda_device, lanes=2, hbm_budget_bytes=need) as srv:
        futs = [srv.submit(r) for r in reqs]
        res = [f.result(timeout=120) for f in futs]
        assert all(len(r.alpha) == len(q.cameras) for r, q in zip(res, reqs))
        big = serve.RenderRequest(np.zeros((200000, 3), np.float32),
                                  np.tile(np.eye(3, dtype=np.float32), (200000, 1, 1)),
                                  np.zeros(200000, np.float32), reqs[0].cameras * 8)
        with pytest.raises(MemoryError):
            srv.submit(big).result(timeout=60)


def test_autotuner_picks_a_candidate(cuda_device, tmp_path):
    items = S.config3(seed=3, n_scenes=6)
    means, prec, logw, scenes, views, off = [], [], [], [], [], 0
    for si, (sc, cams) in enumerate(items):
        means.append(sc.means); prec.append(sc.prec); logw.append(sc.logw)
        scenes.append((off, sc.n)); off += sc.n
        views += [dict(scene=si, height=c.height, width=c.width, fx=c.fx, fy=c.fy, cx=c.cx, cy=c.cy,
                       quat=c.quat, trans=c.trans) for c in cams]
    m, p, w = [torch.from_numpy(np.concatenate(x)).to(cuda_device) for x in (means, prec, logw)]
    tuner = autotune.Autotuner(path=str(tmp_path / "tune.json"))
    best = tuner.tune(scenes, views, m, p, w, reps=2)
    assert (tuple(best["tile"]), best["px"], best["chunk"]) in [(t, x, c) for t, x, c in autotune.CANDIDATES]
    assert tuner.lookup(scenes, views)["tile"] == tuple(best["tile"])
    assert autotune.Autotuner(path=str(tmp_path / "tune.json")).lookup(scenes, views)["px"] == best["px"]
    # every candidate renders the same images (to rounding)
    ref = None
    for tile, px, chunk in autotune.CANDIDATES:
        b = fe.Batch(scenes, views, tile=tile, px=px, chunk=chunk)
        d, a = b.forward(m, p, w)
        if ref is None:
            ref = a.clone()
        assert torch.allclose(a, ref, atol=2e-6, rtol=0)
        b.close()
    # Tuned for host outputs: its own cache entry, no heavy-first trial (the direct stores take
    # tiles in index order), and the picked batch's host call equals its device forward.
    host = tuner.tune(scenes, views, m, p, w, reps=2, target="host")
    assert (tuple(host["tile"]), host["px"], host["chunk"]) in \
        [(t, x, c) for t, x, c in autotune.CANDIDATES]
    assert len(host["candidates"]) == len(autotune.CANDIDATES)
    assert host["bucket"].endswith("_host")
    assert tuner.lookup(scenes, views, target="host")["tile"] == tuple(host["tile"])
    assert tuner.lookup(scenes, views)["tile"] == tuple(best["tile"])
    b = fe.Batch(scenes, views, tile=host["tile"], px=host["px"], chunk=host["chunk"])
    d, a = b.forward(m, p, w)
    hd, ha = b.forward_host(m.cpu(), p.cpu(), w.cpu())
    assert torch.equal(hd, d.cpu()) and torch.equal(ha, a.cpu())
    b.close()


def test_device_without_index_and_malformed_request(cuda_device):
    req = small_stream(1, seed=4)[0]
    with serve.RenderServer(device="cuda", lanes=1) as srv:
        assert srv.device.index is not None
        res = srv.submit(req).result(timeout=120)
        assert len(res.alpha) == len(req.cameras)
    # A malformed request is rejected at submission and does not disturb the next one.
    bad = serve.RenderRequest(req.means, req.prec, req.logw,
                              [S.Camera(32, 32, 0.0, 0.0, 16.0, 16.0, *S.look_at([0.5, 0, 0]))])
    with serve.RenderServer(device=cuda_device, lanes=1) as srv:
        with pytest.raises(ValueError):
            srv.submit(bad)
        ok = srv.submit(req).result(timeout=120)
        assert len(ok.alpha) == len(req.cameras)


def test_fused_silhouette_bce_matches_float64(cuda_device):
    # Renders of ragged sizes back to back (boundaries inside warps), alphas at and around the
    # clamp bounds, soft and binary targets.
    rng = np.random.default_rng(7)
    sizes = [1, 37, 128, 1000, 4099, 3]
    n = sum(sizes)
    a = rng.uniform(size=n).astype(np.float32)
    special = np.array([0.0, 1.0, 1e-9, 3e-8, 1 - 1e-8, 0.99999994, 1e-30, 0.5], np.float32)
    a[rng.choice(n, 400, replace=False)] = rng.choice(special, 400)
    t = (rng.uniform(size=n) > 0.6).astype(np.float32)
    t[::7] = rng.uniform(size=t[::7].size)
    alpha, target = torch.from_numpy(a).to(cuda_device), torch.from_numpy(t).to(cuda_device)
    ends = torch.tensor(np.cumsum(sizes), dtype=torch.int64, device=cuda_device)
    loss, galpha = fe.api.silhouette_bce(alpha, target, ends)
    terms, d = serve.bce_terms(alpha, target)
    lo = 0
    for s, hi in enumerate(np.cumsum(sizes)):
        ref = float(terms[lo:hi].mean())
        assert abs(float(loss[s]) - ref) <= 1e-6 * abs(ref) + 1e-9
        # float32 evaluation of -t/a + (1-t)/(1-a): error relative to the terms' magnitudes
        # (the two terms cancel for soft targets)
        a64 = alpha[lo:hi].double().clamp(3e-8, 1 - 3e-8)
        t64 = target[lo:hi].double()
        scale = (t64 / a64 + (1 - t64) / (1 - a64)) / (hi - lo)
        err = (galpha[lo:hi].double() - d[lo:hi] / (hi - lo)).abs()
        assert bool((err <= 1e-6 * scale + 1e-30).all())
        lo = hi
