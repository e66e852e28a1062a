"""The parity accounting (oracle/parity.py) on the CPU: it must pass the
oracle against itself, catch planted mistakes, and excuse only ties it can
prove.  Mistakes are planted in copies of the oracle's outputs."""
import numpy as np

from tracetransform_gb300.synthetic import blob_image

from parity import (account_circus, account_sinograms, median_tie, selection_tie, tie_rows,
                    zscore_mismatches)


def _case(O, tfs=(0, 1, 2, 3, 4, 5, 6, 7)):
    img = blob_image(20, 23, 4, (2, 6), (40, 200), 11)
    padded = O.pad(img)
    ang = O.angles_for_step(10)
    ref, med = O.sinograms(padded, ang, list(tfs), with_medians=True)
    return padded, ang, list(tfs), ref, med


def test_oracle_against_itself(oracle_lib):
    padded, ang, tfs, ref, med = _case(oracle_lib)
    rep = account_sinograms(padded, ang, tfs, ref.copy(), ref, med.copy(), med)
    assert rep["unexplained"] == 0 and rep["median_ties"] == 0 and rep["selection_ties"] == 0
    assert rep["entries"] == ref.size


def test_planted_value_error_is_caught(oracle_lib):
    padded, ang, tfs, ref, med = _case(oracle_lib)
    got = ref.copy()
    t, line, a = 2, np.argmax(ref[2, :, 5]), 5  # T2 at a non-zero entry
    got[t, line, a] *= 1.001
    rep = account_sinograms(padded, ang, tfs, got, ref, med.copy(), med)
    assert rep["unexplained"] == 1
    assert rep["details"][0]["line"] == line and rep["details"][0]["angle"] == a


def test_planted_median_that_is_no_tie_is_caught(oracle_lib):
    padded, ang, tfs, ref, med = _case(oracle_lib)
    got_med = med.copy()
    t, line, a = 1, np.argmax(ref[0, :, 3]), 3
    got_med[t, line, a] += 2  # a different row, value unchanged
    rep = account_sinograms(padded, ang, tfs, ref.copy(), ref, got_med, med)
    assert rep["unexplained"] == 1
    assert "not a tie" in rep["details"][0]["why"]


def test_value_at_a_tied_median_is_excused(oracle_lib):
    """A column whose crossing sits exactly on the half-total: the value at
    the other reachable row is accepted, counted as a median tie."""
    O = oracle_lib
    x = np.array([1, 1, 0, 0, 1, 1], np.float32)
    m = O.weighted_median(x)
    assert m == 1 and tie_rows(x, m) == [2, 3, 4]
    assert median_tie(x, 1, 3) and not median_tie(np.array([1, 2, 0, 0, 1, 1], np.float32), 1, 3)
    assert O.t_at(1, x, 3) != O.t_at(1, x, 1)


def test_selection_tie():
    keys = np.array([3, 1, 2, 4], np.float32)
    w = np.array([1, 1, 1, 1], np.float32)  # sorted cumulative 1 2 3 4 of 4: 2 C = W at key 2
    assert selection_tie(keys, w, 2.0)       # the reference's key
    assert selection_tie(keys, w, 3.0)       # reachable: 2 C_2 == W exactly
    assert not selection_tie(keys, w, 4.0)
    assert not selection_tie(keys, w, 2.5)
    assert selection_tie(keys, w, 3.0001, key_rtol=1e-4)


def test_circus_accounting(oracle_lib):
    O = oracle_lib
    padded, ang, tfs, ref, _ = _case(O, (0, 1, 3))
    pfs = [(1, 0, 0), (2, 0, 0), (3, 0, 0)]
    circ = np.stack([O.circus(ref[t], pfs) for t in range(len(tfs))])
    assert account_circus(ref, pfs, circ.copy(), ref=circ)["unexplained"] == 0
    bad = circ.copy()
    bad[1, 2, 4] *= 1.01
    rep = account_circus(ref, pfs, bad, ref=circ)
    assert rep["unexplained"] == 1 and rep["details"][0]["P"] == "P3"
    # a propagated tie excuses every entry of its (sinogram, angle) column
    rep = account_circus(ref, pfs, bad, ref=circ, tie_columns=[(1, 4)])
    assert rep["unexplained"] == 0 and rep["median_ties"] == 1


def test_zscore_mismatches(oracle_lib):
    c = np.random.default_rng(0).random((2, 3, 36)).astype(np.float32)
    z = np.stack([[oracle_lib.zscore(v) for v in row] for row in c])
    assert zscore_mismatches(c, z) == 0
    z[1, 1, 7] = np.nextafter(z[1, 1, 7], np.float32(1e9))
    assert zscore_mismatches(c, z) == 1


def test_conditioning_needs_the_engine_at_least_as_accurate(oracle_lib):
    """A T3 entry off the reference's float value is excused only when the
    exact value shows the engine no worse than the reference."""
    from oracle.parity import t_exact
    padded, ang, tfs, ref, med = _case(oracle_lib, (3,))
    a = 4
    line = int(np.argmax(ref[0, :, a]))
    x = oracle_lib.rotate(padded, float(ang[a]))[:, line]
    exact = t_exact(3, x, int(med[0, line, a]))
    r = float(ref[0, line, a])
    assert abs(r - exact) <= 1e-4 * abs(exact)
    got = ref.copy()
    got[0, line, a] = np.float32(exact * (1 + 5e-5))  # off the reference by up to ~1e-4
    rep = account_sinograms(padded, ang, tfs, got, ref, med.copy(), med)
    assert rep["unexplained"] == 0
    got[0, line, a] = np.float32(exact * (1 + 3e-4))  # far from the exact value
    rep = account_sinograms(padded, ang, tfs, got, ref, med.copy(), med)
    assert rep["unexplained"] == 1


def test_exact_values_follow_the_formulas(oracle_lib):
    from oracle.parity import p_exact, t_exact
    x = np.random.default_rng(2).random(41).astype(np.float32)
    m = oracle_lib.weighted_median(x)
    for f in (0, 1, 2):
        want = float(oracle_lib.t_at(f, x, m))
        assert abs(t_exact(f, x, m) - want) <= 1e-5 * abs(want)
    sq = oracle_lib.weighted_median(np.sqrt(x))
    for f in (3, 4, 5):
        want = float(oracle_lib.t_at(f, x, sq))
        assert abs(t_exact(f, x, sq) - want) <= 1e-4 * abs(want)
    col = x.reshape(-1, 1)
    for k in (1, 3):
        want = float(oracle_lib.circus(col, [(k, 0, 0)])[0, 0])
        assert abs(p_exact(k, x) - want) <= 1e-5 * abs(want)
