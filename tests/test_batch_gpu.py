"""The batched engine (tt_transform_batch): uneven image sizes and angle
counts in one persistent, graph-captured pass, against the per-image path and
the CPU oracle."""
import numpy as np
import pytest

import tracetransform_gb300 as tt
from tracetransform_gb300.synthetic import blob_image

from parity import close_mask

pytestmark = pytest.mark.gpu

SHAPES = [(40, 40), (33, 57), (64, 20), (3, 3), (91, 91), (17, 130), (128, 96), (50, 51),
          (12, 12), (77, 31)]
STEPS = [1, 2, 3, 5, 2, 1, 4, 6, 7, 2]


def _images():
    imgs = [blob_image(r, c, 3, (2, 9), (40, 200), 50 + i) for i, (r, c) in enumerate(SHAPES)]
    imgs.append(np.zeros((20, 25), np.float32, order="F"))
    return imgs, STEPS + [3]


@pytest.mark.parametrize("tfs", [[0, 1, 2, 3, 4, 5], [0, 6, 7, 2]])
def test_batch_matches_per_image_transform(tfs):
    imgs, steps = _images()
    pfs = ["1", "2", "3"]
    got = tt.transform_batch(imgs, steps, [str(t) for t in tfs], pfs)
    assert len(got) == len(imgs)
    for img, st, (circ, sig) in zip(imgs, steps, got):
        tr = tt.Transformer(img, "x", st, False)
        want_sig = tr.getTransform([str(t) for t in tfs], pfs, write_data=False)
        assert circ.shape == tr.circus.shape
        ok = close_mask(circ, tr.circus)
        assert ok.mean() >= 0.99, (img.shape, st, (~ok).sum())
        ok_s = close_mask(sig.T, want_sig.T, rtol=1e-3)
        assert ok_s.mean() >= 0.99, (img.shape, st, (~ok_s).sum())


def test_batch_matches_oracle(oracle_lib):
    imgs, steps = _images()
    got = tt.transform_batch(imgs, steps, ["0", "1", "3"], ["1", "3"])
    for img, st, (circ, _) in list(zip(imgs, steps, got))[:6]:
        ref = oracle_lib.transform(img, st, [0, 1, 3], [(1, 0), (3, 0)])
        ok = close_mask(circ, ref["circus"])
        assert ok.mean() >= 0.99, (img.shape, st, (~ok).sum())


def test_batch_replay_is_deterministic_and_reshapes():
    imgs, steps = _images()
    a = tt.transform_batch(imgs, steps, ["0", "2", "5"], ["1", "2"])
    b = tt.transform_batch(imgs, steps, ["0", "2", "5"], ["1", "2"])  # graph replay
    for (ca, sa), (cb, sb) in zip(a, b):
        assert np.array_equal(ca, cb) and np.array_equal(sa, sb, equal_nan=True)
    c = tt.transform_batch(imgs[:4], steps[:4], ["0"], ["3"])  # a new shape
    assert [x[0].shape for x in c] == [(1, 1, 360 // s) for s in steps[:4]]


def test_batch_rejects_hermite():
    with pytest.raises(tt.api._native.TTError):
        tt.transform_batch([np.ones((8, 8), np.float32)], [4], ["0"], ["H2"])
