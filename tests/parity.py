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
