"""Float64 numpy restatements of the empty-space components (test
infrastructure). These components have no counterpart in the reference; the
definitions restated here are the ones the CUDA kernels implement:

- occupancy grid: cell g per axis spans voxels [(g - 1) c, g c) (one border
  cell each side); occupied iff any voxel within two voxels of the cell is
  non-zero; value = Chebyshev distance in cells to the nearest occupied
  cell, capped at max_dist (0 = occupied);
- extent: first and last sample (t = s / (S - 1)) of the box-culled march
  whose eight trilinear corners are not all zero, (1, 0) when none;
- proposal features: entry/exit points of the footprint box (-1, dim),
  normalised by dim, with sin/cos of pi 2^k v for k = 0..3, zero-padded to 64;
- proposal network 64-64-64-2 (ReLU) and its asymmetric loss
  alpha * relu(e)^2 + relu(-e)^2 with e_near = y0 - t0, e_far = t1 - y1;
  for a ray with an empty target (t0 > t1), relu(y1 - y0 + EMPTY_MARGIN)^2
  (any proposal with y0 > y1 skips it whole, so only a proposed window costs).
"""

from __future__ import annotations

import numpy as np

from .numpy_oracle import _rays, _taps

EMPTY_MARGIN = 0.05  # target gap y0 - y1 (box-span units) for rays with nothing to march


def occupancy_grid(vol, cell: int, max_dist: int) -> np.ndarray:
    vol = np.asarray(vol)
    D, H, W = vol.shape
    gz, gy, gx = (D + cell - 1) // cell + 2, (H + cell - 1) // cell + 2, (W + cell - 1) // cell + 2
    nz = vol != 0
    occ = np.zeros((gz, gy, gx), dtype=bool)
    for cz in range(gz):
        z0, z1 = max((cz - 1) * cell - 2, 0), min(cz * cell + 1, D - 1)
        if z0 > z1:
            continue
        for cy in range(gy):
            y0, y1 = max((cy - 1) * cell - 2, 0), min(cy * cell + 1, H - 1)
            if y0 > y1:
                continue
            for cx in range(gx):
                x0, x1 = max((cx - 1) * cell - 2, 0), min(cx * cell + 1, W - 1)
                if x0 > x1:
                    continue
                occ[cz, cy, cx] = nz[z0 : z1 + 1, y0 : y1 + 1, x0 : x1 + 1].any()
    dist = np.where(occ, 0, max_dist).astype(np.int64)
    for _ in range(max_dist):
        pad = np.pad(dist, 1, constant_values=10**6)
        m = dist.copy()
        for dz in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dx in (-1, 0, 1):
                    m = np.minimum(m, pad[1 + dz : 1 + dz + gz, 1 + dy : 1 + dy + gy, 1 + dx : 1 + dx + gx] + 1)
        dist = np.where(occ, 0, m)
    return dist.astype(np.uint8)


def extent(vol, M, src, tgt, n_samples) -> np.ndarray:
    """[B, N, 2] first/last non-empty sample t over all samples."""
    vol = np.asarray(vol, np.float64)
    M, src, tgt = (np.asarray(a, np.float64) for a in (M, src, tgt))
    B, N, _ = tgt.shape
    out = np.zeros((B, N, 2))
    for b in range(B):
        t, _, p = _rays(M, src, tgt, b, slice(0, N), n_samples)
        vals, *_ = _taps(vol, p[..., 0], p[..., 1], p[..., 2])
        nz = np.zeros(p.shape[:2], bool)
        for v, *_ in vals.values():
            nz |= v != 0
        for n in range(N):
            idx = np.nonzero(nz[n])[0]
            out[b, n] = (t[idx[0]], t[idx[-1]]) if idx.size else (1.0, 0.0)
    return out


def proposal_features(p0, d, dims) -> tuple[np.ndarray, np.ndarray, np.ndarray, np.ndarray]:
    """(features [R, 64], tau0 [R], tau1 [R], hit [R]) for voxel-space rays
    p0 + t d (p0, d: [R, 3] in x, y, z order) and dims = (D, H, W)."""
    p0, d = np.asarray(p0, np.float64), np.asarray(d, np.float64)
    D, H, W = dims
    hi = np.array([W, H, D], np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        a = (-1.0 - p0) / d
        b = (hi - p0) / d
    lo_t = np.where(np.abs(d) < 1e-20, np.where((p0 >= -1) & (p0 <= hi), -np.inf, np.inf), np.minimum(a, b))
    hi_t = np.where(np.abs(d) < 1e-20, np.where((p0 >= -1) & (p0 <= hi), np.inf, -np.inf), np.maximum(a, b))
    tau0, tau1 = lo_t.max(1), hi_t.min(1)
    hit = (tau0 < tau1) & np.isfinite(tau0) & np.isfinite(tau1)
    v = np.zeros((p0.shape[0], 6))
    e = p0 + np.where(hit, tau0, 0)[:, None] * d
    x = p0 + np.where(hit, tau1, 0)[:, None] * d
    v[:, :3] = np.where(hit[:, None], e / hi, 0)
    v[:, 3:] = np.where(hit[:, None], x / hi, 0)
    f = np.zeros((p0.shape[0], 64))
    f[:, :6] = v
    for k in range(4):
        f[:, 6 + 12 * k : 12 + 12 * k] = np.sin(np.pi * 2**k * v)
        f[:, 12 + 12 * k : 18 + 12 * k] = np.cos(np.pi * 2**k * v)
    return f, tau0, tau1, hit


def _unpack(P):
    P = np.asarray(P, np.float64)
    W1 = P[0:4096].reshape(64, 64)
    b1 = P[4096:4160]
    W2 = P[4160:8256].reshape(64, 64)
    b2 = P[8256:8320]
    W3 = P[8320:8448].reshape(2, 64)
    b3 = P[8448:8450]
    return W1, b1, W2, b2, W3, b3


def proposal_forward(P, X) -> np.ndarray:
    W1, b1, W2, b2, W3, b3 = _unpack(P)
    h1 = np.maximum(np.asarray(X, np.float64) @ W1.T + b1, 0)
    h2 = np.maximum(h1 @ W2.T + b2, 0)
    return h2 @ W3.T + b3


def proposal_loss_grad(P, X, T, V, alpha: float, inv_count: float) -> tuple[float, np.ndarray]:
    """(inv_count * sum of losses over valid rays, gradient [8450])."""
    W1, b1, W2, b2, W3, b3 = _unpack(P)
    X = np.asarray(X, np.float64)
    T = np.asarray(T, np.float64)
    V = np.asarray(V).astype(bool)
    h1 = np.maximum(X @ W1.T + b1, 0)
    h2 = np.maximum(h1 @ W2.T + b2, 0)
    y = h2 @ W3.T + b3
    empty = T[:, 0] > T[:, 1]
    en = y[:, 0] - T[:, 0]
    ef = T[:, 1] - y[:, 1]
    wn = np.where(en > 0, alpha, 1.0)
    wf = np.where(ef > 0, alpha, 1.0)
    ee = np.maximum(y[:, 1] - y[:, 0] + EMPTY_MARGIN, 0.0)
    per_ray = np.where(empty, ee**2, wn * en**2 + wf * ef**2)
    loss = float((per_ray * V).sum() * inv_count)
    dy = np.where(empty[:, None], np.stack([-2 * ee, 2 * ee], 1), np.stack([2 * wn * en, -2 * wf * ef], 1))
    dy = dy * (V[:, None] * inv_count)
    dh2 = (dy @ W3) * (h2 > 0)
    dh1 = (dh2 @ W2) * (h1 > 0)
    g = np.zeros(8450)
    g[0:4096] = (dh1.T @ X).ravel()
    g[4096:4160] = dh1.sum(0)
    g[4160:8256] = (dh2.T @ h1).ravel()
    g[8256:8320] = dh2.sum(0)
    g[8320:8448] = (dy.T @ h2).ravel()
    g[8448:8450] = dy.sum(0)
    return loss, g
