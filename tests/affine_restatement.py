"""Test-side FP64 restatement of the landmark affine start: the GPU kernel's definition
(landmark_affine_projection_kernel, src/embedding_cuda_kernels.cpp:552-733) and the reference's
CPU statement of it (project_embedding_affine_cpp, src/embedding_utils.cpp:2120-2335): excess-
distance weights with the median excess as scale, a weighted local affine fit by ridge-regularised
Cholesky, its displacement capped at max_extrapolation times the neighbourhood radius, the
weighted neighbour mean where the fit fails. Test infrastructure only."""
import numpy as np

EPS = 1.4901161193847656e-8


def _weighted_mean(L, refs, d, valid, rho, sigma):
    w = np.where(valid, np.exp(-np.maximum(0.0, d - rho) / max(sigma, EPS)), 0.0)
    s = w.sum()
    if not np.isfinite(s) or s <= 0:
        s = 1.0
    return (w[:, None] * L[np.where(valid, refs, 0)]).sum(0) / s


def affine_start(X, Q, L, idx, dist, off, m_req, ridge, max_ext):
    """Test-side restatement of the landmark affine start in float64."""
    nq, k = idx.shape
    n_ref = L.shape[0]
    m = max(3, min(m_req, min(k, 12)))
    out = np.zeros((nq, 2))
    for i in range(nq):
        refs = idx[i].astype(np.int64) - off
        d = dist[i].astype(np.float64)
        inr = (refs >= 0) & (refs < n_ref)
        valid = inr & np.isfinite(d) & (d >= 0)
        rho = d[valid].min() if valid.any() else 0.0
        zero = np.where(valid & (d <= EPS))[0]
        if len(zero):
            out[i] = L[refs[zero[0]]]
            continue
        exc = np.where(valid, np.maximum(0.0, d - rho), np.inf)
        pos = np.sort(exc[np.isfinite(exc) & (exc > EPS)])
        sigma = np.median(pos) if len(pos) else max(rho, EPS)
        if not np.isfinite(sigma) or sigma < EPS:
            sigma = EPS
        r, vm, im = refs[:m], valid[:m], inr[:m]
        ex = np.where(vm, np.maximum(0.0, d[:m] - rho), np.inf)
        w = np.where(im & np.isfinite(ex), np.exp(-ex / sigma), 0.0)
        if not np.isfinite(w.sum()) or w.sum() <= 0:
            out[i] = _weighted_mean(L, refs, d, valid, rho, sigma)
            continue
        w = w / w.sum()
        sw = np.sqrt(w)
        rc = np.where(im, r, 0)
        Lr = np.where(im[:, None], L[rc], 0.0)
        cy = (w[:, None] * Lr).sum(0)
        U = np.where(im[:, None], Lr - cy, 0.0)
        rhs = sw[:, None] * U
        radius2 = (U ** 2).sum(1).max()
        Xr = np.where(im[:, None], X[rc].astype(np.float64), 0.0)
        xc = (w[:, None] * Xr).sum(0)
        C = np.where(im[:, None], Xr - xc, 0.0)
        qc = Q[i].astype(np.float64) - xc
        G = (C @ C.T) * np.outer(sw, sw)
        qv = (C @ qc) * sw
        trace = (w * (C ** 2).sum(1)).sum()
        G += (ridge * max(trace, EPS) + EPS) * np.eye(m)
        Lc = np.zeros_like(G)
        ok = True
        for j in range(m):
            dg = G[j, j] - (Lc[j, :j] ** 2).sum()
            if not np.isfinite(dg) or dg <= EPS:
                ok = False
                break
            Lc[j, j] = np.sqrt(dg)
            for t in range(j + 1, m):
                Lc[t, j] = (G[t, j] - (Lc[t, :j] * Lc[j, :j]).sum()) / Lc[j, j]
        if ok:
            z = np.linalg.solve(Lc.T, np.linalg.solve(Lc, rhs))
            disp = qv @ z
            cap = max_ext * np.sqrt(max(radius2, EPS))
            nd = np.sqrt((disp ** 2).sum())
            if nd * nd > cap * cap:
                disp = disp * cap / (nd + EPS)
            start = cy + disp
            ok = np.all(np.isfinite(start))
        out[i] = start if ok else _weighted_mean(L, refs, d, valid, rho, sigma)
    return out
