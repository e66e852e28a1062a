"""FP64 restatement of the sinogram + circus path (test infrastructure).

The same operations as the reference's float path (the C oracle in
tt_oracle.c restates that one bit for bit), evaluated in double precision with
numpy, vectorised over the columns of each rotated image.  It is the yardstick
for the per-functional error statements: the reference's float path and the
GPU engine are both compared against it.

Follows, in double:
  pad geometry        c++/src/auxiliary.cpp:257-275 (the oracle's pad())
  rotate/interpolate  c++/src/auxiliary.cpp:182-255, origin (N-1)/2,
                      c = cos(-theta), s = sin(-theta), bilinear from modf
  findWeightedMedian  c++/src/functionals.cpp:21-30 (first i with 2 prefix >= sum)
  T0 .. T7            c++/src/functionals.cpp:95-276
  P1, P2, P3          c++/src/functionals.cpp:287-360 (P3 through numpy's rfft)
"""
from __future__ import annotations

import numpy as np


def rotate(padded: np.ndarray, angle_deg: float) -> np.ndarray:
    """Rotated N x N image (float64) of a square padded image."""
    n = padded.shape[0]
    th = float(angle_deg) * np.pi / 180.0
    c, s = np.cos(-th), np.sin(-th)
    o = (n - 1) / 2.0
    g = np.arange(n, dtype=np.float64) - o
    X = g[None, :]  # column
    Y = g[:, None]  # row
    qx = X * c + Y * s + o
    qy = X * (-s) + Y * c + o
    ok = (qx >= 0) & (qx < n - 1) & (qy >= 0) & (qy < n - 1)
    xi = np.where(ok, np.floor(qx), 0).astype(np.int64)
    yi = np.where(ok, np.floor(qy), 0).astype(np.int64)
    xf = np.where(ok, qx - xi, 0.0)
    yf = np.where(ok, qy - yi, 0.0)
    p = padded.astype(np.float64)
    x1 = np.minimum(xi + 1, n - 1)
    y1 = np.minimum(yi + 1, n - 1)
    v = (p[yi, xi] * (1 - xf) * (1 - yf) + p[yi, x1] * xf * (1 - yf) +
         p[y1, xi] * (1 - xf) * yf + p[y1, x1] * xf * yf)
    return np.where(ok, v, 0.0)


def weighted_median(x: np.ndarray) -> np.ndarray:
    """Per column of x (rows = samples): first i with 2 * prefix >= total,
    else the last row."""
    cs = np.cumsum(x, axis=0)
    hit = 2 * cs >= cs[-1:, :]
    idx = np.argmax(hit, axis=0)
    return np.where(hit.any(axis=0), idx, x.shape[0] - 1)


def _tail(x: np.ndarray, m: np.ndarray):
    """r = row - m (>= 0 where it counts) and the mask row >= m."""
    r = np.arange(x.shape[0])[:, None] - m[None, :]
    return r, r >= 0


def _t345_tables(n: int):
    r = np.arange(n, dtype=np.float64)
    lr = np.log(np.maximum(r, 1))
    t = {3: r * np.exp(5j * lr), 4: np.exp(3j * lr), 5: np.sqrt(r) * np.exp(4j * lr)}
    for k in t:
        t[k][0] = 0
    return t


def _select(keys: np.ndarray, weights: np.ndarray, valid: np.ndarray) -> np.ndarray:
    """Per column: sort the valid keys, weighted median of the weights in key
    order, the key there (T6 / T7 / P2 selections)."""
    big = np.where(valid, keys, np.inf)
    order = np.argsort(big, axis=0, kind="stable")
    sk = np.take_along_axis(big, order, axis=0)
    sw = np.take_along_axis(np.where(valid, weights, 0.0), order, axis=0)
    cnt = valid.sum(axis=0)
    cs = np.cumsum(sw, axis=0)
    tot = cs[-1:, :]
    hit = (2 * cs >= tot) & (np.arange(keys.shape[0])[:, None] < cnt[None, :])
    idx = np.where(hit.any(axis=0), np.argmax(hit, axis=0), np.maximum(cnt - 1, 0))
    return np.take_along_axis(sk, idx[None, :], axis=0)[0]


def tfunctionals(img: np.ndarray, tfuncs) -> np.ndarray:
    """T-functionals of every column of a rotated image: (nT, N)."""
    x = img
    n = x.shape[0]
    out = []
    m1 = weighted_median(x)
    m2 = weighted_median(np.sqrt(np.maximum(x, 0)))
    tabs = None
    for f in tfuncs:
        if f == 0:
            out.append(x.sum(axis=0))
        elif f in (1, 2):
            r, ok = _tail(x, m1)
            out.append(np.where(ok, x * (r if f == 1 else r * r), 0).sum(axis=0))
        elif f in (3, 4, 5):
            if tabs is None:
                tabs = _t345_tables(n)
            r, ok = _tail(x, m2)
            ok &= r >= 1
            k = tabs[f][np.clip(r, 0, n - 1)]
            z = np.where(ok, k * x, 0).sum(axis=0)
            out.append(np.abs(z))
        elif f == 6:
            r, ok = _tail(x, m2)
            keys = np.where(ok, r * x, 0.0)
            out.append(_select(keys, np.sqrt(np.maximum(x, 0)), ok))
        elif f == 7:
            r, ok = _tail(x, m1)
            out.append(_select(x, np.sqrt(np.maximum(x, 0)), ok))
        else:
            raise ValueError(f)
    return np.stack(out)


def sinograms(padded: np.ndarray, angles_deg, tfuncs, with_medians: bool = False):
    """(nT, N, A) sinograms in double; with_medians also returns the
    weighted-median rows of x and of sqrt(x) per (column, angle), (N, A) each."""
    n = padded.shape[0]
    out = np.zeros((len(tfuncs), n, len(angles_deg)))
    m1 = np.zeros((n, len(angles_deg)), np.int64)
    m2 = np.zeros_like(m1)
    for a, ang in enumerate(angles_deg):
        img = rotate(padded, ang)
        out[:, :, a] = tfunctionals(img, tfuncs)
        if with_medians:
            m1[:, a] = weighted_median(img)
            m2[:, a] = weighted_median(np.sqrt(np.maximum(img, 0)))
    return (out, m1, m2) if with_medians else out


def circus(sino: np.ndarray, pfuncs) -> np.ndarray:
    """(nP, A) P-functionals of an N x A sinogram in double."""
    n = sino.shape[0]
    out = []
    for p in pfuncs:
        if p == 1:
            out.append(np.abs(np.diff(sino, axis=0)).sum(axis=0))
        elif p == 2:
            ok = np.ones_like(sino, dtype=bool)
            out.append(_select(sino, sino, ok))
        elif p == 3:
            F = np.fft.rfft(sino, axis=0)
            y_half = np.abs(F / n) ** 4
            mirror = np.array([k if k <= n // 2 else n - k for k in range(n)])
            y = y_half[mirror]
            lin = -1 + np.arange(n) * 2.0 / (n - 1)
            out.append((0.5 * np.diff(lin)[:, None] * (y[1:] + y[:-1])).sum(axis=0))
        else:
            raise ValueError(p)
    return np.stack(out)
