"""The CPU oracle against golden outputs of the reference's own sources.

tests/golden/*.npz were produced by tests/golden/make_golden.py, which runs
maleadt/tracetransform's c++/ sources compiled against oracle/shim/.  The C
restatement in oracle/ must reproduce them bit for bit (the nearest
orthonormal sinogram excepted: both sides there stand in for Eigen's float
JacobiSVD with a double-precision Jacobi SVD, so it is compared at 1e-5).
"""
import glob
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(HERE, "golden", "*.npz"))
               if not p.endswith(("rotate9.npz", "image_io.npz")))


def load(name):
    return dict(np.load(os.path.join(HERE, "golden", name + ".npz")))


@pytest.mark.parametrize("name", CASES)
def test_transform_matches_reference(oracle_lib, name):
    O = oracle_lib
    g = load(name)
    pf = list(zip(g["pkinds"].tolist(), g["porders"].tolist()))
    res = O.transform(g["image"], int(g["step"]), g["tfuncs"].tolist(), pf)
    assert np.array_equal(res["padded"], g["padded"])
    assert np.array_equal(res["sino"], g["sino"], equal_nan=True)
    if "centers" in g:
        assert res["centers"] == g["centers"].tolist()
        for t in range(len(res["nos"])):
            np.testing.assert_allclose(res["nos"][t], g[f"nos{t}"], rtol=0, atol=1e-5)
        np.testing.assert_allclose(res["circus"], g["circus"], rtol=1e-4, atol=1e-5)
    else:
        assert np.array_equal(res["circus"], g["circus"], equal_nan=True)
        assert np.array_equal(res["sig"], g["sig"], equal_nan=True)


def test_rotation_matches_reference(oracle_lib):
    g = load("rotate9")
    for a, want in zip(g["angles"], g["rotated"]):
        got = oracle_lib.rotate(g["image"], float(a))
        assert np.array_equal(got, want), a


def test_pad_geometry(oracle_lib):
    # the padded sizes the benchmark workloads rely on
    assert oracle_lib.pad_geometry(256, 256) == (363, 54, 54)
    assert oracle_lib.pad_geometry(1024, 1024)[0] == 1449
    assert oracle_lib.pad_geometry(4096, 4096)[0] == 5793
    n, ro, co = oracle_lib.pad_geometry(20, 13)
    assert n % 2 == 1 and 0 <= ro and 0 <= co


def test_find_weighted_median_edges(oracle_lib):
    O = oracle_lib
    lib = O.lib()
    f = lambda x: lib.tto_find_weighted_median(O._fp(np.ascontiguousarray(x, np.float32)), len(x))
    assert f([0, 0, 0, 0]) == 0          # all-zero column: 2*0 >= 0 at i = 0
    assert f([0, 0, 1, 0]) == 2
    assert f([1, 1, 1, 1]) == 1          # 2*2 >= 4 at i = 1
    assert f([-1, -1, -1]) == 0          # negative total: 2*(-1) >= -3
    assert f([1, -5, 1]) == 0           # 2*1 >= -3 at the first element


def test_dft_direct_vs_chirp(oracle_lib):
    """The oracle's two DFT routes agree (direct below 2049 points, chirp-z above)."""
    O = oracle_lib
    rng = np.random.default_rng(0)
    for n in (2049, 2897, 5793):
        x = rng.random(n).astype(np.float32)
        re = np.zeros(n // 2 + 1, np.float32)
        im = np.zeros(n // 2 + 1, np.float32)
        O.lib().tto_dft_r2c(O._fp(x), n, O._fp(re), O._fp(im))
        ref = np.fft.rfft(x.astype(np.float64))
        np.testing.assert_allclose(re, ref.real, rtol=0, atol=1e-9 * n + 1e-4)
        np.testing.assert_allclose(im, ref.imag, rtol=0, atol=1e-9 * n + 1e-4)
