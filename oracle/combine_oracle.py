"""CPU restatement of RFBA's CombineBlock reconstruction (test infrastructure
only): Matlab Scripts/genpsf.m, loadResult.m and CombineBlock.m:24-173 in numpy,
used to check librfba_srrf's rfba_combine_* entry points."""
from __future__ import annotations

import numpy as np


def _gaussian(rows: int, cols: int, sigma: float) -> np.ndarray:
    """fspecial('gaussian', [rows cols], sigma) (column-major accumulation)."""
    y = np.arange(rows) - (rows - 1) / 2.0
    x = np.arange(cols) - (cols - 1) / 2.0
    h = np.exp(-(x[None, :] ** 2 + y[:, None] ** 2) / (2.0 * sigma * sigma))
    h[h < np.finfo(float).eps * h.max()] = 0.0
    s = 0.0
    for v in h.T.ravel():  # MATLAB column-major order, sequential
        s += v
    return h / s if s != 0 else h


def _u16(v):
    v = np.asarray(v, np.float64)
    out = np.where(v <= 0, 0.0, np.where(v >= 65535, 65535.0, np.floor(v + 0.5)))
    return np.nan_to_num(out).astype(np.uint16)


def genpsf(sigma: float = 3.5, thr: float = 1000.0) -> np.ndarray:
    """genpsf.m: returns the cropped uint16 PSF as [z][row][col]."""
    g = 100
    xy = _gaussian(g, g, sigma)
    xy = xy * (65535.0 / xy.max())
    zl = _gaussian(1, g, sigma)[0]
    zl = zl * (65535.0 / zl.max())
    h = xy[:, :, None] * zl[None, None, :]
    mh = h.max()
    psf = _u16(h * (65535.0 / mh))  # (row, col, slice)
    half = int(round(g / 2.0))
    mid = psf[:, :, half - 1].astype(np.int64)
    x1 = 0
    for i in range(1, half + 1):
        if mid[i - 1, :].max() <= thr:
            x1 = i
    x1 += 1
    x2 = g
    for i in range(half, g + 1):
        if mid[i - 1, :].max() > thr:
            x2 = i
    x1 = min(x1, g - x2 + 1)
    x2 = g - x1 + 1
    y1 = 0
    for i in range(1, half + 1):
        if mid[:, i - 1].max() <= thr:
            y1 = i
    y1 += 1
    y2 = g
    for i in range(half, g + 1):
        if mid[:, i - 1].max() > thr:
            y2 = i
    y1 = min(y1, g - y2 + 1)
    y2 = g - y1 + 1
    out1 = psf[x1 - 1:x2, y1 - 1:y2, :]
    z1 = 0
    for i in range(1, half + 1):
        if out1[:, :, i - 1].max() <= thr:
            z1 = i
    z1 += 1
    z2 = None
    for i in range(half, g + 1):
        if out1[:, :, i - 1].max() > thr:
            z2 = i
    z1 = min(z1, g - z2 + 1)
    z2 = g - z1 + 1
    out = out1[:, :, z1 - 1:z2]
    return np.ascontiguousarray(np.transpose(out, (2, 0, 1)))


def load_result(path, border: int, start, size) -> np.ndarray:
    """loadResult.m on one file: spots (5 values) strictly inside the block minus border."""
    keep = []
    with open(path) as f:
        for line in f:
            line = line.rstrip("\r\n")
            if len(line) <= 5 or line[:4] != "PASS":
                continue
            c = line.find(":")
            vals = [float(t) for t in line[(c + 2 if c >= 0 else 6):].split()]
            for i in range(0, len(vals) - 4, 5):
                s = vals[i:i + 5]
                x, y, z = s[2] - start[0] + 1, s[3] - start[1] + 1, s[4] - start[2] + 1
                if border < x < size[0] - border and border < y < size[1] - border and border < z < size[2] - border:
                    keep.append(s)
    return np.array(keep, np.float64).reshape(-1, 5)


def _mround(v):
    return np.where(v < 0, -np.floor(-v + 0.5), np.floor(v + 0.5)).astype(np.int64)


def render(spots: np.ndarray, img_dims, zoom: int, psf: np.ndarray, r: int, rz: int, thr: int) -> np.ndarray:
    """CombineBlock.m:24-173: histogram, noise mask, convn 'same', uint16 scaling.
    Arrays [z][y][x]; psf [z][y][x]."""
    X, Y, Z = (d * zoom for d in img_dims)
    hist = np.zeros((Z, Y, X), np.int64)
    if len(spots):
        ix, iy, iz = (_mround(spots[:, k] * zoom) for k in (2, 3, 4))
        ok = (ix >= 0) & (iy >= 0) & (iz >= 0) & (ix < X) & (iy < Y) & (iz < Z)
        np.add.at(hist, (iz[ok], iy[ok], ix[ok]), 1)
    occ = (hist > 0).astype(np.int64)
    L = np.zeros_like(occ)
    S = np.zeros_like(occ)
    if Y >= 2 * r + 1:
        c = np.concatenate([np.zeros((Z, 1, X), np.int64), np.cumsum(occ, axis=1)], axis=1)
        for y in range(r, Y - r):
            L[:, y, :] = c[:, y + r + 1, :] - c[:, y - r, :]
    if X >= 2 * r + 1:
        c = np.concatenate([np.zeros((Z, Y, 1), np.int64), np.cumsum(L, axis=2)], axis=2)
        for x in range(r, X - r):
            S[:, :, x] = c[:, :, x + r + 1] - c[:, :, x - r]
    mask = np.ones_like(occ)
    if Z >= 2 * rz + 1 and Y >= 2 * r + 1 and X >= 2 * r + 1:
        c = np.concatenate([np.zeros((1, Y, X), np.int64), np.cumsum(S, axis=0)], axis=0)
        for z in range(rz, Z - rz):
            V = c[z + rz + 1] - c[z - rz]
            mask[z, r:Y - r, r:X - r] = (V[r:Y - r, r:X - r] > thr)
    temp = hist * mask
    Kz, Ky, Kx = psf.shape
    out = np.zeros((Z, Y, X), np.int64)
    p = psf.astype(np.int64)
    for (az, ay, ax) in zip(*np.nonzero(temp)):
        v = temp[az, ay, ax]
        oz0, oy0, ox0 = az - Kz // 2, ay - Ky // 2, ax - Kx // 2
        zs, ys, xs = max(0, oz0), max(0, oy0), max(0, ox0)
        ze, ye, xe = min(Z, oz0 + Kz), min(Y, oy0 + Ky), min(X, ox0 + Kx)
        out[zs:ze, ys:ye, xs:xe] += v * p[zs - oz0:ze - oz0, ys - oy0:ye - oy0, xs - ox0:xe - ox0]
    m = out.max()
    res = (out.astype(np.float64) / m) * 65535.0 if m > 0 else np.zeros(out.shape)
    return _u16(res)
