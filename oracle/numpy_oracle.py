"""Float64 numpy restatement of the fused kernel's per-sample arithmetic and its
analytic adjoint (test infrastructure).

Follows nanodrr src/nanodrr/drr/_fused.py: camera -> voxel line
p = M [q, 1] with q = lerp(src, tgt, t), t = s / (S - 1) (:133-142, :191-194);
trilinear tap with zero padding per corner (:195-220, helper :11-16);
nearest label with ties to even and drop of labels outside [0, C) (:28-32,
:225-228, :300); output step * Σ (:327-331). Adjoint (:230-298): g = go[cls] *
step, analytic position gradient, dL/dM = Σ g ∇v ⊗ [q, 1], camera-space
chains to src/tgt/step and the scatter of g * w into the volume gradient.
No culling: every sample is evaluated (culling is bitwise-neutral by design).
"""

from __future__ import annotations

import numpy as np


def _taps(vol, px, py, pz):
    """Corner values, fractions and indices of the trilinear cell (zeros outside)."""
    D, H, W = vol.shape
    x0 = np.floor(px)
    y0 = np.floor(py)
    z0 = np.floor(pz)
    fx, fy, fz = px - x0, py - y0, pz - z0
    ix, iy, iz = x0.astype(np.int64), y0.astype(np.int64), z0.astype(np.int64)
    vals = {}
    for cz in (0, 1):
        for cy in (0, 1):
            for cx in (0, 1):
                jx, jy, jz = ix + cx, iy + cy, iz + cz
                inb = (jx >= 0) & (jx < W) & (jy >= 0) & (jy < H) & (jz >= 0) & (jz < D)
                v = np.zeros(px.shape, dtype=np.float64)
                v[inb] = vol[jz[inb], jy[inb], jx[inb]]
                vals[(cz, cy, cx)] = (v, inb, jx, jy, jz)
    return vals, fx, fy, fz


def _value(vals, fx, fy, fz):
    v = lambda k: vals[k][0]  # noqa: E731
    c00 = v((0, 0, 0)) * (1 - fx) + v((0, 0, 1)) * fx
    c01 = v((0, 1, 0)) * (1 - fx) + v((0, 1, 1)) * fx
    c10 = v((1, 0, 0)) * (1 - fx) + v((1, 0, 1)) * fx
    c11 = v((1, 1, 0)) * (1 - fx) + v((1, 1, 1)) * fx
    c0 = c00 * (1 - fy) + c01 * fy
    c1 = c10 * (1 - fy) + c11 * fy
    return c0 * (1 - fz) + c1 * fz


def _labels(lab, px, py, pz, C):
    D, H, W = lab.shape
    rx, ry, rz = np.rint(px).astype(np.int64), np.rint(py).astype(np.int64), np.rint(pz).astype(np.int64)
    inb = (rx >= 0) & (rx < W) & (ry >= 0) & (ry < H) & (rz >= 0) & (rz < D)
    cls = np.zeros(px.shape, dtype=np.int64)
    cls[inb] = np.trunc(lab[rz[inb], ry[inb], rx[inb]].astype(np.float64)).astype(np.int64)
    return cls


def _rays(M, src, tgt, b, sl, S):
    t = np.arange(S, dtype=np.float64) / (S - 1)
    s = src[b, 0:1] if src.shape[1] == 1 else src[b, sl]
    e = tgt[b, sl] - s
    q = s[:, None, :] + t[None, :, None] * e[:, None, :]  # [n, S, 3]
    Mb = M[b]
    p = q @ Mb[:, :3].T + Mb[:, 3]
    return t, q, p


def march_numpy(vol, lab, M, src, tgt, step, n_samples, n_classes=1, chunk=1024):
    """[B, C, N] float64 forward."""
    vol = np.asarray(vol, np.float64)
    M, src, tgt, step = (np.asarray(a, np.float64) for a in (M, src, tgt, step))
    B, N, _ = tgt.shape
    out = np.zeros((B, n_classes, N))
    for b in range(B):
        for i in range(0, N, chunk):
            sl = slice(i, min(N, i + chunk))
            _, _, p = _rays(M, src, tgt, b, sl, n_samples)
            vals, fx, fy, fz = _taps(vol, p[..., 0], p[..., 1], p[..., 2])
            val = _value(vals, fx, fy, fz)
            if n_classes == 1:
                out[b, 0, sl] = val.sum(1) * step[b, sl]
            else:
                cls = _labels(np.asarray(lab), p[..., 0], p[..., 1], p[..., 2], n_classes)
                for c in range(n_classes):
                    out[b, c, sl] = np.where(cls == c, val, 0.0).sum(1) * step[b, sl]
    return out


def march_numpy_adjoint(go, vol, lab, M, src, tgt, step, n_samples, n_classes=1, chunk=1024):
    """Analytic adjoint: (gvol [D,H,W], gM [B,3,4], gsrc like src, gtgt [B,N,3], gstep [B,N])."""
    vol = np.asarray(vol, np.float64)
    go, M, src, tgt, step = (np.asarray(a, np.float64) for a in (go, M, src, tgt, step))
    B, N, _ = tgt.shape
    gvol = np.zeros(vol.shape)
    gM = np.zeros((B, 3, 4))
    gsrc = np.zeros(src.shape)
    gtgt = np.zeros((B, N, 3))
    gstep = np.zeros((B, N))
    flat = gvol.reshape(-1)
    D, H, W = vol.shape
    for b in range(B):
        Mb = M[b]
        for i in range(0, N, chunk):
            sl = slice(i, min(N, i + chunk))
            t, q, p = _rays(M, src, tgt, b, sl, n_samples)
            vals, fx, fy, fz = _taps(vol, p[..., 0], p[..., 1], p[..., 2])
            val = _value(vals, fx, fy, fz)
            if n_classes == 1:
                gg = np.broadcast_to(go[b, 0, sl][:, None], val.shape)
            else:
                cls = _labels(np.asarray(lab), p[..., 0], p[..., 1], p[..., 2], n_classes)
                ok = (cls >= 0) & (cls < n_classes)
                gg = np.where(ok, go[b, np.clip(cls, 0, n_classes - 1), np.arange(sl.start, sl.stop)[:, None]], 0.0)
            g = gg * step[b, sl][:, None]
            v = lambda k: vals[k][0]  # noqa: E731
            wx0, wy0, wz0 = 1 - fx, 1 - fy, 1 - fz
            dvx = ((v((0, 0, 1)) - v((0, 0, 0))) * wy0 + (v((0, 1, 1)) - v((0, 1, 0))) * fy) * wz0 + (
                (v((1, 0, 1)) - v((1, 0, 0))) * wy0 + (v((1, 1, 1)) - v((1, 1, 0))) * fy
            ) * fz
            dvy = ((v((0, 1, 0)) - v((0, 0, 0))) * wx0 + (v((0, 1, 1)) - v((0, 0, 1))) * fx) * wz0 + (
                (v((1, 1, 0)) - v((1, 0, 0))) * wx0 + (v((1, 1, 1)) - v((1, 0, 1))) * fx
            ) * fz
            dvz = ((v((1, 0, 0)) - v((0, 0, 0))) * wx0 + (v((1, 0, 1)) - v((0, 0, 1))) * fx) * wy0 + (
                (v((1, 1, 0)) - v((0, 1, 0))) * wx0 + (v((1, 1, 1)) - v((0, 1, 1))) * fx
            ) * fy
            gpos = np.stack([g * dvx, g * dvy, g * dvz], axis=-1)  # [n, S, 3]
            q1 = np.concatenate([q, np.ones(q.shape[:-1] + (1,))], axis=-1)
            gM[b] += np.einsum("nsi,nsj->ij", gpos, q1)
            gq = gpos @ Mb[:, :3]  # M3^T gpos
            gs = ((1 - t)[None, :, None] * gq).sum(1)
            gt = (t[None, :, None] * gq).sum(1)
            if src.shape[1] == 1:
                gsrc[b, 0] += gs.sum(0)
            else:
                gsrc[b, sl] = gs
            gtgt[b, sl] = gt
            gstep[b, sl] = (gg * val).sum(1)
            for (cz, cy, cx), (_, inb, jx, jy, jz) in vals.items():
                w = (fx if cx else wx0) * (fy if cy else wy0) * (fz if cz else wz0)
                idx = (jz * H + jy) * W + jx
                np.add.at(flat, idx[inb], (g * w)[inb])
    return gvol, gM, gsrc, gtgt, gstep
