"""The batched engine (tt_transform_batch): uneven image sizes and angle
counts in one persistent, graph-captured pass, accounted entry by entry
against the CPU oracle as tests/test_parity_gpu.py does for one image:
the batch's own sinograms (tt_transform_batch_sinograms_device) against the
reference's, its circus functions against the reference's P-stage on those
sinograms, its signatures bit-identical to zscore of its circus functions,
and end to end against the reference's circus functions."""
import numpy as np
import pytest

import tracetransform_gb300 as tt
from tracetransform_gb300.synthetic import blob_image

from parity import (account_circus, account_sinograms, assert_accounted, record,
                    zscore_mismatches)

pytestmark = pytest.mark.gpu

SHAPES = [(40, 40), (33, 57), (64, 20), (3, 3), (91, 91), (17, 130), (128, 96), (50, 51),
          (12, 12), (77, 31)]
STEPS = [1, 2, 3, 5, 2, 1, 4, 6, 7, 2]


def _images():
    imgs = [blob_image(r, c, 3, (2, 9), (40, 200), 50 + i) for i, (r, c) in enumerate(SHAPES)]
    imgs.append(np.zeros((20, 25), np.float32, order="F"))
    return imgs, STEPS + [3]


def run_batch(imgs, steps, tfs, pfs, tile=None):
    """The batch through tt_transform_batch_device (tile: a pinned tile shape
    (lines per CTA, CTAs per SM, lines per warp), else the tuner's); returns
    per image (sinograms (nT, N, A), circus (nT, nP, A), signatures)."""
    import torch
    from tracetransform_gb300.device import Engine
    eng = Engine(0)
    if tile:
        eng.batch_tile(pin=tile)
    bufs = [np.ascontiguousarray(np.asarray(im, np.float32).ravel(order="F")) for im in imgs]
    offsets = np.zeros(len(bufs), np.int64)
    offsets[1:] = np.cumsum([b.size for b in bufs])[:-1]
    flat = torch.from_numpy(np.concatenate(bufs)).cuda()
    rows = [im.shape[0] for im in imgs]
    cols = [im.shape[1] for im in imgs]
    circ, sig = eng.transform_batch(flat, offsets, rows, cols, steps, tfs,
                                    [(k, -1, -1) for k in pfs])
    sino = eng.batch_sinograms(flat)
    torch.cuda.synchronize()
    if tile:
        assert eng.batch_tile() == tuple(tile)
    circ, sig, sino = circ.cpu().numpy(), sig.cpu().numpy(), sino.cpu().numpy()
    out, so, co = [], 0, 0
    for r, c, s in zip(rows, cols, steps):
        n = tt.pad_geometry(r, c)[0]
        a = 360 // s
        k = len(tfs) * a * n
        st = sino[so: so + k].reshape(len(tfs), a, n).transpose(0, 2, 1)
        m = len(tfs) * len(pfs) * a
        out.append((st, circ[co: co + m].reshape(len(tfs), len(pfs), a),
                    sig[co: co + m].reshape(len(tfs), len(pfs), a)))
        so += k
        co += m
    return out


def account_batch(O, name, imgs, steps, tfs, pfs, tile=None):
    pf = [(k, 0, 0) for k in pfs]
    totals = {"entries": 0, "median_ties": 0, "selection_ties": 0}
    results = run_batch(imgs, steps, tfs, pfs, tile)
    for i, (img, step, (sino, circ, sig)) in enumerate(zip(imgs, steps, results)):
        padded = O.pad(img)
        ang = O.angles_for_step(step)
        ref = O.sinograms(padded, ang, tfs)
        rs = account_sinograms(padded, ang, tfs, sino, ref)
        assert_accounted(rs, f"{name} image {i} {img.shape} step {step} sinograms")
        rc = account_circus(sino, pf, circ)
        assert_accounted(rc, f"{name} image {i} circus")
        assert zscore_mismatches(circ, sig) == 0, f"{name} image {i} signatures"
        ref_circ = np.stack([O.circus(ref[t], pf) for t in range(len(tfs))])
        re = account_circus(ref, pf, circ, ref=ref_circ, tie_columns=rs["tie_columns"],
                            key_rtol=1e-4)
        assert_accounted(re, f"{name} image {i} end to end")
        for k in totals:
            totals[k] += rs[k]
    record(name, totals)
    return totals


@pytest.mark.parametrize("tfs", [[0, 1, 2, 3, 4, 5], [0, 6, 7, 2]])
def test_batch_vs_oracle(oracle_lib, tfs):
    imgs, steps = _images()
    account_batch(oracle_lib, f"batch11_T{''.join(map(str, tfs))}", imgs, steps, tfs, [1, 2, 3])


@pytest.mark.parametrize("tile", [(8, 1, 0), (4, 2, 0), (4, 1, 1), (8, 1, 2), (16, 1, 4)])
def test_batch_every_tile_shape_vs_oracle(oracle_lib, tile):
    """Every tile shape the tuner can pick, pinned, T0-T5 (and T6/T7 for the
    CTA kernel's shapes)."""
    imgs, steps = _images()
    account_batch(oracle_lib, f"batch11_tile{tile}", imgs, steps, [0, 1, 2, 3, 4, 5], [1, 2, 3],
                  tile)
    if tile[2] == 0:
        account_batch(oracle_lib, f"batch11_T67_tile{tile}", imgs, steps, [6, 7, 1], [1],
                      tile)


def test_batch_pinned_warp_tile_rejects_t6():
    from tracetransform_gb300._native import TTError
    imgs, steps = _images()
    with pytest.raises(TTError):
        run_batch(imgs[:3], steps[:3], [0, 6], [1], (8, 1, 2))


def test_batch512_images_vs_oracle(oracle_lib):
    """20 images of the 512-image workload (sides 64-512 per axis, 180 or 360
    angles), T0-T5 x P1-P3, in one batched call."""
    from tracetransform_gb300.synthetic import workload
    items = workload("batch512")
    pick = list(range(0, 512, 26))[:20]
    imgs = [items[i][0] for i in pick]
    steps = [int(items[i][1]) for i in pick]
    tot = account_batch(oracle_lib, "batch512_sample", imgs, steps, [0, 1, 2, 3, 4, 5], [1, 2, 3])
    assert tot["median_ties"] + tot["selection_ties"] <= 0.002 * tot["entries"], tot


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
