"""Parity helpers shared by the GPU tests.

Criterion (per sinogram / circus entry):
    |gpu - ref| <= RTOL * max(|ref|, EPS_FRAC * max|ref column|)
with RTOL = 1e-4: the engine's reductions run in warp order, the reference's
sequentially, so float sums agree to rounding; the column guard keeps entries
that cancel to ~0 (z-scores, T3-T5) from demanding more than float gives.

Weighted-median rows must equal the reference's, except where the
reference's own cumulative sum ties the half-total within the rounding that
a different summation order can produce (|2 P_k - S| <= N ulp(S)); such
columns are counted as ties and their median-dependent values are not
compared.
"""
from __future__ import annotations

import numpy as np

RTOL = 1e-4
EPS_FRAC = 1e-3


def close_mask(got, ref, rtol=RTOL, eps_frac=EPS_FRAC, axis=-1):
    """Boolean array: entries within tolerance (column = last axis)."""
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    colmax = np.max(np.abs(ref), axis=axis, keepdims=True)
    scale = np.maximum(np.abs(ref), eps_frac * colmax)
    ok = np.abs(got - ref) <= rtol * scale
    ok |= (got == ref)  # exact (covers all-zero columns and infs)
    ok |= np.isnan(got) & np.isnan(ref)
    return ok


def rel_err(got, ref, eps_frac=EPS_FRAC, axis=-1):
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    colmax = np.max(np.abs(ref), axis=axis, keepdims=True)
    scale = np.maximum(np.maximum(np.abs(ref), eps_frac * colmax), 1e-30)
    return np.where(got == ref, 0.0, np.abs(got - ref) / scale)


def selection_tie(keys: np.ndarray, weights: np.ndarray, got: float) -> bool:
    """Is `got` the key at which the reference's weighted median of `keys`
    could cross within float rounding?

    TFunctional6/7 and PFunctional2 sort the keys, sum the weights in sorted
    order in float and take the key at the first k with 2 C_k >= W
    (c++/src/functionals.cpp:226-311).  A different summation order may move
    the crossing across the boundary between two adjacent distinct keys when
    |2 C - W| there is within N ulp(W)."""
    keys = np.asarray(keys, np.float32)
    w = np.asarray(weights, np.float32)
    order = np.argsort(keys, kind="stable")
    k, w = keys[order], w[order]
    c = np.cumsum(w, dtype=np.float32)
    total = c[-1] if len(c) else np.float32(0)
    bound = len(k) * np.spacing(np.float32(abs(total))) + np.spacing(np.float32(0))
    idx = np.nonzero(2.0 * c.astype(np.float64) >= float(total))[0]
    i_ref = int(idx[0]) if len(idx) else len(k) - 1
    if k[i_ref] == np.float32(got):
        return True
    where = np.nonzero(k == np.float32(got))[0]
    if not len(where):
        return False
    lo_i, hi_i = (int(where[0]), i_ref) if where[0] < i_ref else (i_ref, int(where[-1]))
    # every cumulative sum between the two keys must sit at the threshold
    gap = np.abs(2.0 * c[lo_i:hi_i].astype(np.float64) - float(total))
    return bool(np.all(gap <= bound))


def median_tie(x: np.ndarray, m_ref: int, m_gpu: int) -> bool:
    """Is the reference's weighted-median crossing of column x ambiguous
    between rows m_ref and m_gpu at float precision?

    The reference takes the first k with 2 * P_k >= S, P and S summed
    sequentially in float (c++/src/functionals.cpp:21-30)."""
    x = np.asarray(x, np.float32)
    n = len(x)
    p = np.cumsum(x, dtype=np.float32)  # sequential float prefix, as the reference
    s = p[-1] if n else np.float32(0)
    lo, hi = min(m_ref, m_gpu), max(m_ref, m_gpu)
    bound = n * np.spacing(np.float32(abs(s))) + np.spacing(np.float32(0))
    # every prefix between the two candidate rows must sit at the threshold
    gap = np.abs(2.0 * p[lo:hi].astype(np.float64) - float(s))
    return bool(np.all(gap <= bound))
