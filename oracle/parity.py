"""Parity accounting between the CUDA engine and the oracle.

TEST INFRASTRUCTURE ONLY (tests/, and bench.py's CPU-baseline leg, which
reports the same figures for the images it times).  The product package never
imports this module.

Criterion per sinogram / circus entry:

    |got - ref| <= RTOL * max(|ref|, EPS_FRAC * max |ref column|)

with RTOL = 1e-4 (the engine reduces in warp order, the reference
sequentially, so float sums agree to rounding) and the column guard keeping
entries that cancel to ~0 from demanding more than float gives.  A column is
one angle's N trace lines for sinograms and one circus function (A angles)
for circus functions.

An entry outside the tolerance is accepted only when it is *proven* to come
from a tie in the reference's own arithmetic; everything else is counted as
unexplained and fails the check:

* median tie -- findWeightedMedian (c++/src/functionals.cpp:21-30) takes the
  first row k with 2 P_k >= S, P and S summed sequentially in float.  When
  every prefix between the reference's row and the engine's row sits within
  N ulp(S) of the threshold, a different (equally valid) summation order can
  pick either row.  The engine's value must then equal the functional
  evaluated, with the reference's arithmetic, at the engine's row
  (oracle.t_at), within the same tolerance.
* selection tie -- TFunctional6/7 and PFunctional2 (functionals.cpp:226-311)
  sort keys and take the key where the sorted cumulative weight crosses half
  the total; the engine's key must be one the crossing can reach within
  len * ulp(W).
* conditioning -- T0-T5, P1 and P3 are sums; where their terms cancel (the
  complex T3-T5 integrals, mostly) the reference's own float result can be
  off its exact value by more than 1e-4.  Such an entry is accepted when the
  exact (double) value of the reference's formula on the same float samples,
  at the same weighted-median row, shows the engine within 1e-4 of it or at
  least as close to it as the reference.

Every check returns a report: per functional the entries, the largest
relative error (over all entries, and over the entries not excused by a
proven tie), the tie counts and the first few unexplained entries.
"""
from __future__ import annotations

import numpy as np

from . import oracle as O

RTOL = 1e-4
EPS_FRAC = 1e-3
SQRT_MEDIAN = (3, 4, 5, 6)  # T-functionals whose median is that of sqrt(x)


def close_mask(got, ref, rtol=RTOL, eps_frac=EPS_FRAC, axis=-1):
    """Boolean array: entries within tolerance (column = `axis`)."""
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    colmax = np.max(np.abs(ref), axis=axis, keepdims=True)
    scale = np.maximum(np.abs(ref), eps_frac * colmax)
    with np.errstate(invalid="ignore"):
        ok = np.abs(got - ref) <= rtol * scale
    ok |= (got == ref)  # exact (covers all-zero columns and infinities)
    ok |= np.isnan(got) & np.isnan(ref)
    return ok


def rel_err(got, ref, eps_frac=EPS_FRAC, axis=-1):
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    colmax = np.max(np.abs(ref), axis=axis, keepdims=True)
    scale = np.maximum(np.maximum(np.abs(ref), eps_frac * colmax), 1e-30)
    with np.errstate(invalid="ignore"):
        return np.where(got == ref, 0.0, np.abs(got - ref) / scale)


def _close1(got: float, want: float, guard: float, rtol=RTOL) -> bool:
    if got == want or (np.isnan(got) and np.isnan(want)):
        return True
    return abs(float(got) - float(want)) <= rtol * max(abs(float(want)), EPS_FRAC * guard)


def selection_tie(keys: np.ndarray, weights: np.ndarray, got: float,
                  key_rtol: float = 0.0) -> bool:
    """Is `got` a key at which the reference's weighted median of `keys`
    can cross within float rounding?

    The reference sorts the keys, sums the weights in sorted order in float
    and takes the key at the first k with 2 C_k >= W.  A different summation
    order may move the crossing across the boundary between two adjacent
    distinct keys when every cumulative sum between them is within
    len * ulp(W) of the threshold.  key_rtol > 0 matches `got` to keys within
    that relative distance (for keys computed from sinograms that agree with
    the reference's only to rounding)."""
    keys = np.asarray(keys, np.float32)
    w = np.asarray(weights, np.float32)
    order = np.argsort(keys, kind="stable")
    k, w = keys[order], w[order]
    c = np.cumsum(w, dtype=np.float32)
    total = c[-1] if len(c) else np.float32(0)
    bound = len(k) * np.spacing(np.float32(abs(total))) + np.spacing(np.float32(0))
    idx = np.nonzero(2.0 * c.astype(np.float64) >= float(total))[0]
    i_ref = int(idx[0]) if len(idx) else len(k) - 1
    kd = k.astype(np.float64)
    match = np.abs(kd - float(got)) <= key_rtol * np.abs(kd) if key_rtol > 0 else \
        (k == np.float32(got))
    if len(k) and match[i_ref]:
        return True
    where = np.nonzero(match)[0]
    if not len(where):
        return False
    lo_i, hi_i = (int(where[0]), i_ref) if where[0] < i_ref else (i_ref, int(where[-1]))
    gap = np.abs(2.0 * c[lo_i:hi_i].astype(np.float64) - float(total))
    return bool(np.all(gap <= bound))


def median_tie(x: np.ndarray, m_ref: int, m_gpu: int) -> bool:
    """Is the reference's weighted-median crossing of column x ambiguous
    between rows m_ref and m_gpu at float precision?"""
    x = np.asarray(x, np.float32)
    n = len(x)
    p = np.cumsum(x, dtype=np.float32)  # sequential float prefix, as the reference
    s = p[-1] if n else np.float32(0)
    lo, hi = min(m_ref, m_gpu), max(m_ref, m_gpu)
    bound = n * np.spacing(np.float32(abs(s))) + np.spacing(np.float32(0))
    gap = np.abs(2.0 * p[lo:hi].astype(np.float64) - float(s))
    return bool(np.all(gap <= bound))


def tie_rows(x: np.ndarray, m_ref: int, reach: int = 4096) -> list:
    """Rows other than m_ref that the reference's crossing of x can reach
    within rounding (median_tie holds), nearest first."""
    x = np.asarray(x, np.float32)
    n = len(x)
    if n == 0:
        return []
    p = np.cumsum(x, dtype=np.float32)
    s = float(p[-1])
    bound = n * float(np.spacing(np.float32(abs(s)))) + float(np.spacing(np.float32(0)))
    gap = np.abs(2.0 * p.astype(np.float64) - s) <= bound
    rows = []
    k = m_ref - 1  # rows below: every prefix in [k, m_ref) at the threshold
    while k >= 0 and m_ref - k <= reach and gap[k]:
        rows.append(k)
        k -= 1
    k = m_ref  # rows above: every prefix in [m_ref, k) at the threshold
    while k < n - 1 and k + 1 - m_ref <= reach and gap[k]:
        rows.append(k + 1)
        k += 1
    return sorted(rows, key=lambda r: abs(r - m_ref))


def _median_input(f: int, x: np.ndarray) -> np.ndarray:
    return np.sqrt(x.astype(np.float32)) if f in SQRT_MEDIAN else x


def _select_tie_at(f: int, x: np.ndarray, m: int, got: float) -> bool:
    """T6 / T7 selection tie with the weighted median at row m."""
    tail = x[m:].astype(np.float32)
    if f == 7:
        return selection_tie(tail, np.sqrt(tail), got)
    if f == 6:
        keys = np.arange(len(tail), dtype=np.float32) * tail
        return selection_tie(keys, np.sqrt(tail), got)
    return False


def t_exact(f: int, x: np.ndarray, m: int) -> float:
    """T-functional f (0-5) of the float samples x with the weighted median
    at row m, evaluated exactly enough (double) to serve as the true value of
    the reference's formula (c++/src/functionals.cpp:95-213; the T3-T5
    kernels as the reference rounds them to float)."""
    x = np.asarray(x, np.float32).astype(np.float64)
    n = len(x)
    if f == 0:
        return float(np.sum(x))
    r = np.arange(n - m, dtype=np.float64)
    tail = x[m:]
    if f == 1:
        return float(np.sum(tail * r))
    if f == 2:
        return float(np.sum(tail * r * r))
    re, im = O.t345_tables(f, n)
    q = np.arange(1, n - m)
    return float(np.hypot(np.sum(re[q].astype(np.float64) * x[m + q]),
                          np.sum(im[q].astype(np.float64) * x[m + q])))


def p_exact(kind: int, col: np.ndarray) -> float:
    """P1 / P3 of a sinogram column in double (c++/src/functionals.cpp:287-360)."""
    x = np.asarray(col, np.float32).astype(np.float64)
    n = len(x)
    if kind == 1:
        return float(np.sum(np.abs(np.diff(x))))
    if kind == 3:
        F = np.fft.rfft(x) / n
        h = np.abs(F) ** 4
        y = np.array([h[p] if p <= n // 2 else h[n - p] for p in range(n)])
        lin = -1 + np.arange(n) * 2.0 / (n - 1) if n > 1 else np.zeros(1)
        return float(np.sum(np.diff(lin) * (y[1:] + y[:-1])) / 2.0)
    return float("nan")


def _conditioning(got: float, ref: float, exact: float, guard: float) -> bool:
    """The reference's own float result is ill-conditioned here: the engine
    is within the tolerance of the exact value, or at least as close to it
    as the reference is."""
    if not np.isfinite(exact):
        return False
    return abs(got - exact) <= max(RTOL * max(abs(exact), EPS_FRAC * guard), abs(ref - exact))


class _Report:
    def __init__(self, names):
        self.per = {nm: {"entries": 0, "max_rel": 0.0, "max_rel_unexcused": 0.0,
                         "median_ties": 0, "selection_ties": 0, "conditioning": 0,
                         "unexplained": 0}
                    for nm in names}
        self.details = []
        self.tie_columns = set()  # (t, angle) columns holding an excused entry

    def as_dict(self):
        out = {"per_functional": self.per,
               "unexplained": int(sum(v["unexplained"] for v in self.per.values())),
               "median_ties": int(sum(v["median_ties"] for v in self.per.values())),
               "selection_ties": int(sum(v["selection_ties"] for v in self.per.values())),
               "conditioning": int(sum(v["conditioning"] for v in self.per.values())),
               "entries": int(sum(v["entries"] for v in self.per.values()))}
        out["max_rel_unexcused"] = float(max([v["max_rel_unexcused"] for v in self.per.values()]
                                             + [0.0]))
        out["details"] = self.details[:12]
        out["tie_columns"] = sorted(self.tie_columns)
        return out


def account_sinograms(padded, angles, tfs, got, ref, got_med=None, ref_med=None,
                      rotate=None) -> dict:
    """Account for every entry of a sinogram stack.

    got, ref: (nT, N, A) -- entry (t, line, angle); got_med / ref_med: the
    weighted-median rows (same shape, -1 for T0), got_med may be None (the
    engine's rows are then searched among the rows the reference's crossing
    can reach).  rotate(angle_index) -> the rotated padded image (N x N,
    column `line` is the trace line); defaults to the oracle's rotate()."""
    got = np.asarray(got, np.float32)
    ref = np.asarray(ref, np.float32)
    nT, n, A = ref.shape
    if rotate is None:
        def rotate(a):
            return O.rotate(padded, float(angles[a]))
    names = [f"T{f}" for f in tfs]
    rep = _Report(names)
    # tolerance per angle column (the N lines of one angle)
    ok = np.swapaxes(close_mask(np.swapaxes(got, 1, 2), np.swapaxes(ref, 1, 2)), 1, 2)
    errs = np.swapaxes(rel_err(np.swapaxes(got, 1, 2), np.swapaxes(ref, 1, 2)), 1, 2)
    guard = np.max(np.abs(ref.astype(np.float64)), axis=1)  # (nT, A)
    excused = np.zeros_like(ok)
    suspects = ~ok
    if got_med is not None and ref_med is not None:
        suspects = suspects | (np.asarray(got_med) != np.asarray(ref_med))
    idx = np.argwhere(suspects)
    cur_a, rot = -1, None
    for t, line, a in idx[np.argsort(idx[:, 2], kind="stable")]:
        f = int(tfs[t])
        if a != cur_a:
            rot, cur_a = rotate(int(a)), int(a)
        x = rot[:, line].astype(np.float32)
        g = float(got[t, line, a])
        m_ref = int(ref_med[t, line, a]) if ref_med is not None else (
            -1 if f == 0 else O.weighted_median(_median_input(f, x)))
        why = None
        if f != 0:
            if got_med is not None:
                cands = [int(got_med[t, line, a])]
                if cands[0] != m_ref and not median_tie(_median_input(f, x), m_ref, cands[0]):
                    cands = []
                    why = f"median row {int(got_med[t, line, a])} vs {m_ref}: not a tie"
            else:
                cands = [m_ref] + tie_rows(_median_input(f, x), m_ref)
            for m in cands:
                if _close1(g, O.t_at(f, x, m), guard[t, a]) or _select_tie_at(f, x, m, g):
                    kind = "selection_ties" if m == m_ref else "median_ties"
                    if m == m_ref and _close1(g, O.t_at(f, x, m), guard[t, a]):
                        kind = None  # equal within tolerance at the same row
                    if kind:
                        rep.per[names[t]][kind] += 1
                        excused[t, line, a] = True
                        rep.tie_columns.add((int(t), int(a)))
                    why = "ok"
                    break
        elif ok[t, line, a]:
            why = "ok"
        if why != "ok" and f <= 5:
            # conditioning: the rows the engine may legitimately have used
            if f == 0:
                rows_ok = [m_ref]
            elif got_med is not None:
                mg = int(got_med[t, line, a])
                rows_ok = [mg] if mg == m_ref or median_tie(_median_input(f, x), m_ref, mg) else []
            else:
                rows_ok = [m_ref] + tie_rows(_median_input(f, x), m_ref)
            for m_use in rows_ok:
                ref_at = float(ref[t, line, a]) if m_use == m_ref else O.t_at(f, x, m_use)
                if _conditioning(g, ref_at, t_exact(f, x, max(m_use, 0)), guard[t, a]):
                    rep.per[names[t]]["conditioning"] += 1
                    if m_use != m_ref:
                        rep.per[names[t]]["median_ties"] += 1
                        rep.tie_columns.add((int(t), int(a)))
                    excused[t, line, a] = True
                    why = "ok"
                    break
        if why != "ok":
            ok[t, line, a] = False
            rep.per[names[t]]["unexplained"] += 1
            rep.details.append({"T": f, "line": int(line), "angle": int(a), "got": g,
                                "ref": float(ref[t, line, a]), "ref_median": m_ref,
                                "got_median": None if got_med is None else int(got_med[t, line, a]),
                                "why": why or "outside tolerance"})
        else:
            ok[t, line, a] = True
    for t, nm in enumerate(names):
        rep.per[nm]["entries"] = int(n * A)
        rep.per[nm]["max_rel"] = float(errs[t].max()) if errs[t].size else 0.0
        e = np.where(excused[t], 0.0, errs[t])
        rep.per[nm]["max_rel_unexcused"] = float(e.max()) if e.size else 0.0
    return rep.as_dict()


P_NAMES = {0: "H", 1: "P1", 2: "P2", 3: "P3"}


def account_circus(sino, pfs, got, ref=None, rtol=RTOL, tie_columns=(),
                   key_rtol=0.0) -> dict:
    """Account for every entry of a stack of circus functions.

    sino: (nT, N, A) sinograms the reference side used; pfs: (kind, order,
    center) tuples; got: (nT, nP, A); ref: the oracle's circus of `sino`
    (computed when None).  P2 entries outside the tolerance must be selection
    ties of their sinogram column (keys = weights = the column's values; with
    key_rtol > 0 when the engine's circus came from its own sinograms, which
    match `sino` to rounding).  Entries of a (t, angle) column in tie_columns
    -- sinogram columns with a proven median or selection tie -- are excused
    as propagated ties: every circus entry of an angle depends only on that
    angle's sinogram column (c++/src/circus.cpp:129-154)."""
    tie_columns = set((int(t), int(a)) for t, a in tie_columns)
    sino = np.asarray(sino, np.float32)
    got = np.asarray(got, np.float32)
    nT = sino.shape[0]
    if ref is None:
        ref = np.stack([O.circus(sino[t], list(pfs)) for t in range(nT)])
    names = [P_NAMES[int(k)] + (str(o) if int(k) == 0 else "") for k, o, _ in pfs]
    rep = _Report(names)
    ok = close_mask(got, ref, rtol=rtol)
    errs = rel_err(got, ref)
    excused = np.zeros_like(ok)
    for t, p, a in np.argwhere(~ok):
        kind = int(pfs[p][0])
        col = sino[t][:, a]
        if (int(t), int(a)) in tie_columns:
            rep.per[names[p]]["median_ties"] += 1
            excused[t, p, a] = True
            rep.tie_columns.add((int(t), int(a)))
            continue
        if kind == 2 and selection_tie(col, col, float(got[t, p, a]), key_rtol):
            rep.per[names[p]]["selection_ties"] += 1
            excused[t, p, a] = True
            rep.tie_columns.add((int(t), int(a)))
            continue
        if kind in (1, 3) and _conditioning(float(got[t, p, a]), float(ref[t, p, a]),
                                            p_exact(kind, col),
                                            float(np.abs(ref[t, p]).max())):
            rep.per[names[p]]["conditioning"] += 1
            excused[t, p, a] = True
            continue
        rep.per[names[p]]["unexplained"] += 1
        rep.details.append({"P": names[p], "sinogram": int(t), "angle": int(a),
                            "got": float(got[t, p, a]), "ref": float(ref[t, p, a]),
                            "rel": float(errs[t, p, a])})
    for p, nm in enumerate(names):
        rep.per[nm]["entries"] = int(got[:, p].size)
        rep.per[nm]["max_rel"] = float(errs[:, p].max()) if errs[:, p].size else 0.0
        e = np.where(excused[:, p], 0.0, errs[:, p])
        rep.per[nm]["max_rel_unexcused"] = float(e.max()) if e.size else 0.0
    return rep.as_dict()


def zscore_mismatches(circus, signatures) -> int:
    """Entries where the engine's signatures differ from the oracle's
    zscore (c++/src/auxiliary.cpp:305-318) of the engine's own circus
    functions: both must be bit-identical.  circus, signatures: (..., A)."""
    c = np.asarray(circus, np.float32).reshape(-1, np.shape(circus)[-1])
    s = np.asarray(signatures, np.float32).reshape(c.shape)
    bad = 0
    for i in range(c.shape[0]):
        z = O.zscore(c[i])
        bad += int(np.sum(~((z == s[i]) | (np.isnan(z) & np.isnan(s[i])))))
    return bad
