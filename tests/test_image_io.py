"""resize() and the image I/O of c++/src/auxiliary.cpp against the reference.

tests/golden/image_io.npz holds outputs of the reference's own sources
(tests/golden/make_golden.py io): resize() on seeded images,
readnetpbm / gray2mat / writepgm on hand-made ASCII PGM and PPM files
(comments, CRLF, warnings, malformed input), and mat2gray + writepgm on float
matrices.  The host-side reader and writers must reproduce them byte for
byte; the device resize (tt_resize, and the orthonormal mode's stretch inside
tt_transform) bit for bit.
"""
import os
import re

import numpy as np
import pytest

from tracetransform_gb300 import api

HERE = os.path.dirname(os.path.abspath(__file__))
G = dict(np.load(os.path.join(HERE, "golden", "image_io.npz")))
RESIZE = sorted({int(m.group(1)) for k in G for m in [re.match(r"resize(\d+)_in$", k)] if m})
PGM = sorted({int(m.group(1)) for k in G for m in [re.match(r"pgm(\d+)_in$", k)] if m})
M2G = sorted({int(m.group(1)) for k in G for m in [re.match(r"m2g(\d+)_in$", k)] if m})


def _write(tmp_path, name, data: bytes) -> str:
    path = os.path.join(str(tmp_path), name)
    with open(path, "wb") as f:
        f.write(data)
    return path


@pytest.mark.parametrize("i", RESIZE)
def test_oracle_resize_matches_reference(oracle_lib, i):
    out = G[f"resize{i}_out"]
    got = oracle_lib.resize(G[f"resize{i}_in"], *out.shape)
    assert np.array_equal(got.view(np.uint32), out.view(np.uint32))


@pytest.mark.parametrize("i", PGM)
def test_readnetpbm_matches_reference(tmp_path, i):
    path = _write(tmp_path, "in.pgm", bytes(G[f"pgm{i}_in"]))
    if f"pgm{i}_error" in G:
        want = bytes(G[f"pgm{i}_error"]).decode().replace("error: ", "")
        with pytest.raises(RuntimeError, match=re.escape(want)):
            api.readnetpbm(path)
        return
    chans = api.readnetpbm(path)
    n = len([k for k in G if k.startswith(f"pgm{i}_c") and k.endswith("_pixels")])
    assert len(chans) == n
    for c, m in enumerate(chans):
        assert m.dtype == np.int32
        assert np.array_equal(m, G[f"pgm{i}_c{c}_pixels"])
        gray = api.gray2mat(m)
        assert gray.dtype == np.float32 and gray.flags.f_contiguous
        assert np.array_equal(gray.view(np.uint32), G[f"pgm{i}_c{c}_gray"].view(np.uint32))
        out = os.path.join(str(tmp_path), f"out{c}.pgm")
        api.writepgm(out, m)
        assert open(out, "rb").read() == bytes(G[f"pgm{i}_c{c}_written"])


def test_readnetpbm_warnings(tmp_path, caplog):
    path = _write(tmp_path, "a.pgm", b"P2 2 1 65535 1 2 3")
    with caplog.at_level("WARNING", logger="tracetransform_gb300"):
        api.readnetpbm(path)
    msgs = [r.getMessage() for r in caplog.records]
    assert "Pixels not properly clipped to [0,255]" in msgs
    assert "Trailing data at end of image file" in msgs


def test_readnetpbm_missing_file(tmp_path):
    with pytest.raises(RuntimeError, match="could not open input file"):
        api.readnetpbm(os.path.join(str(tmp_path), "absent.pgm"))


@pytest.mark.parametrize("i", M2G)
def test_mat2gray_matches_reference(tmp_path, i):
    got = api.mat2gray(G[f"m2g{i}_in"])
    assert got.dtype == np.int32
    assert np.array_equal(got, G[f"m2g{i}_out"])
    out = os.path.join(str(tmp_path), "m.pgm")
    api.writepgm(out, got)
    assert open(out, "rb").read() == bytes(G[f"m2g{i}_written"])


def test_pgm_round_trip(tmp_path):
    rng = np.random.default_rng(5)
    pix = rng.integers(0, 256, size=(17, 29)).astype(np.int32)
    path = os.path.join(str(tmp_path), "r.pgm")
    api.writepgm(path, pix)
    (back,) = api.readnetpbm(path)
    assert np.array_equal(back, pix)
    # gray2mat then mat2gray gives the pixels back up to truncation
    again = api.mat2gray(api.gray2mat(back))
    assert np.abs(again.astype(np.int64) * back.max() / 255 - back).max() <= 1


def test_writepgm_line_length(tmp_path):
    path = os.path.join(str(tmp_path), "w.pgm")
    api.writepgm(path, np.full((40, 40), 255, np.int32))
    body = open(path).read().split("\n")[3:]
    # a line ends once it holds more than 66 characters: 17 values of "255 "
    assert all(len(line) <= 68 for line in body)
    assert sum(len(line.split()) for line in body) == 1600


def test_transformer_debug_output(tmp_path, monkeypatch):
    """getTransform's debug output (c++/src/transform.cpp:61-72) goes
    through the same writers: <basename>-<T name>.csv / .pgm."""
    calls = []
    monkeypatch.setattr(api, "writecsv", lambda fn, d: calls.append(("csv", fn, np.shape(d))))
    monkeypatch.setattr(api, "writepgm", lambda fn, d: calls.append(("pgm", fn, np.shape(d))))
    sinos = [np.ones((9, 30), np.float32), np.ones((9, 30), np.float32)]
    api._write_debug_sinograms("base", [api.TFunctionalWrapper.parse("0"),
                                        api.TFunctionalWrapper.parse("5")], sinos)
    assert calls == [("csv", "base-Radon.csv", (9, 30)), ("pgm", "base-Radon.pgm", (9, 30)),
                     ("csv", "base-T5.csv", (9, 30)), ("pgm", "base-T5.pgm", (9, 30))]


@pytest.mark.gpu
@pytest.mark.parametrize("i", RESIZE)
def test_device_resize_bit_exact(i):
    out = G[f"resize{i}_out"]
    got = api.resize(G[f"resize{i}_in"], *out.shape)
    assert np.array_equal(got.view(np.uint32), out.view(np.uint32))


@pytest.mark.gpu
def test_device_resize_rejects_bad_sizes():
    with pytest.raises(Exception):
        api.resize(np.ones((4, 4), np.float32), 0, 4)


def test_workload_pgm_round_trip(tmp_path):
    """The synthetic workloads are also written as ASCII PGM (the reference's
    demo input); readnetpbm + gray2mat give back the very floats the bench
    feeds both paths."""
    from tracetransform_gb300 import synthetic
    (path, step), = synthetic.write_pgm("single256", str(tmp_path))
    (pix,) = api.readnetpbm(path)
    (img, step2), = synthetic.workload("single256")
    assert step == step2
    assert np.array_equal(api.gray2mat(pix).view(np.uint32), img.view(np.uint32))
