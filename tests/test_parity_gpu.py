"""GPU parity: the CUDA engine, called through its C ABI, against the CPU
oracle (oracle/, pinned to the reference's own sources by
tests/test_oracle_golden.py) and against the golden fixtures directly.

Every entry must be within 1e-4 (relative, column guard) of the reference
or be a proven tie of the reference's own arithmetic (oracle/parity.py);
nothing is accepted by percentage.  The accounting is staged, as the path
is: sinograms against the reference's sinograms; circus functions against
the reference's P-stage applied to the engine's own sinograms; signatures
bit-identical to the reference's zscore of the engine's circus functions;
and end to end against the reference's circus functions, where an entry may
differ only in an angle whose sinogram column holds a proven tie.
"""
import glob
import os

import numpy as np
import pytest

import tracetransform_gb300 as tt
from tracetransform_gb300.synthetic import blob_image

from parity import (account_circus, account_sinograms, assert_accounted, engine_sinograms,
                    record, zscore_mismatches)

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(HERE, "golden", "*.npz"))
                if not p.endswith(("rotate9.npz", "image_io.npz")))
P123 = [(1, 0, 0), (2, 0, 0), (3, 0, 0)]


def load(name):
    return dict(np.load(os.path.join(HERE, "golden", name + ".npz")))


@pytest.fixture(scope="module")
def engine():
    import torch
    from tracetransform_gb300.device import Engine
    assert torch.cuda.is_available()
    return Engine(0)


def check_transform(oracle_lib, engine, name, img, step, tfs, pfs=P123, angles=None):
    """Staged accounting of one regular-mode transform (see module doc).
    Returns the sinogram report."""
    import torch
    padded = oracle_lib.pad(img)
    ang = oracle_lib.angles_for_step(step) if angles is None else angles
    ref, ref_med = oracle_lib.sinograms(padded, ang, tfs, with_medians=True)
    got, got_med = engine_sinograms(engine, img, ang, tfs)
    rs = account_sinograms(padded, ang, tfs, got, ref, got_med, ref_med)
    record(name + ":sinograms", rs)
    assert_accounted(rs, name + " sinograms")
    # P-stage on the engine's own sinograms
    dev = torch.from_numpy(np.ascontiguousarray(got.transpose(0, 2, 1))).cuda()
    circ = engine.circus(dev, [(k, o, -1) for k, o, _ in pfs])
    sig = engine.zscore(circ)
    torch.cuda.synchronize()
    circ, sig = circ.cpu().numpy(), sig.cpu().numpy()
    rc = account_circus(got, pfs, circ)
    record(name + ":circus", rc)
    assert_accounted(rc, name + " circus")
    assert zscore_mismatches(circ, sig) == 0, name + ": signatures differ from zscore(circus)"
    # end to end against the reference's own circus functions
    ref_circ = np.stack([oracle_lib.circus(ref[t], list(pfs)) for t in range(len(tfs))])
    re2e = account_circus(ref, pfs, circ, ref=ref_circ, tie_columns=rs["tie_columns"],
                          key_rtol=1e-4)
    record(name + ":end_to_end", re2e)
    assert_accounted(re2e, name + " end to end")
    return rs


def test_rotation_bit_exact_golden():
    g = load("rotate9")
    for a, want in zip(g["angles"], g["rotated"]):
        assert np.array_equal(tt.api.rotate(g["image"], float(a)), want), a


@pytest.mark.parametrize("shape,seed", [((47, 47), 1), ((20, 13), 2), ((13, 31), 3), ((91, 91), 4)])
def test_rotation_bit_exact_oracle(oracle_lib, shape, seed):
    img = blob_image(shape[0], shape[1], 4, (2, 9), (40, 200), seed)
    for a in (0.0, 0.5, 1.0, 13.0, 45.0, 89.0, 90.0, 91.0, 180.0, 233.5, 270.0, 359.0):
        assert np.array_equal(tt.api.rotate(img, a), oracle_lib.rotate(img, a)), a


@pytest.mark.parametrize("name", GOLDEN)
def test_golden_sinograms(oracle_lib, engine, name):
    """The reference's own sinograms (its sources built on the stand-ins)."""
    import torch
    g = load(name)
    tfs = [int(t) for t in g["tfuncs"]]
    padded = g["padded"]
    n = padded.shape[0]
    ang = oracle_lib.angles_for_step(int(g["step"]))
    dev = torch.from_numpy(np.ascontiguousarray(padded.T)).cuda()
    out, med = engine.sinograms(dev, n, n, ang, tfs, padded=True, medians=True)
    got, got_med = out.cpu().numpy().transpose(0, 2, 1), med.cpu().numpy().transpose(0, 2, 1)
    rep = account_sinograms(padded, ang, tfs, got, g["sino"], got_med, None)
    record("golden:" + name, rep)
    assert_accounted(rep, name)
    # the host drop-in entry point (which samples only the frame's non-zero
    # box, so its sums are chunked differently) is accounted the same way
    host = np.stack(tt.getSinograms(padded, int(g["step"]), [str(t) for t in tfs]))
    rep = account_sinograms(padded, ang, tfs, host, g["sino"])
    assert_accounted(rep, name + " (getSinograms)")


@pytest.mark.parametrize("name", [n for n in GOLDEN if "ortho" not in n])
def test_golden_transform(oracle_lib, engine, name):
    """Transformer.getTransform against the reference's own circus functions
    and signatures, staged as check_transform does."""
    g = load(name)
    tfs = [int(t) for t in g["tfuncs"]]
    pfs = [(int(k), int(o), 0) for k, o in zip(g["pkinds"], g["porders"])]
    step = int(g["step"])
    tr = tt.Transformer(g["image"], "golden", step, False)
    sig = tr.getTransform([str(t) for t in tfs], [str(k) for k, _, _ in pfs], write_data=False)
    # the drop-in's sinograms are the device call's (bit-identical circus)
    got, got_med = engine_sinograms(engine, g["image"], oracle_lib.angles_for_step(step), tfs)
    rs = account_sinograms(g["padded"], oracle_lib.angles_for_step(step), tfs, got, g["sino"],
                           got_med, None)
    assert_accounted(rs, name + " sinograms")
    staged = account_circus(got, pfs, tr.circus)
    assert_accounted(staged, name + " circus on the engine's sinograms")
    assert zscore_mismatches(tr.circus, sig.T.reshape(tr.circus.shape)) == 0
    rep = account_circus(g["sino"], pfs, tr.circus, ref=g["circus"],
                         tie_columns=rs["tie_columns"], key_rtol=1e-4)
    record("golden_transform:" + name, rep)
    assert_accounted(rep, name + " end to end")


@pytest.mark.parametrize("side,step", [(32, 2), (64, 3), (20, 1)])
def test_all_functionals_vs_oracle(oracle_lib, engine, side, step):
    img = blob_image(side, side + 3, 5, (3, 12), (40, 200), 100 + side)
    check_transform(oracle_lib, engine, f"blob{side}", img, step, [0, 1, 2, 3, 4, 5, 6, 7])


def test_single256_vs_oracle(oracle_lib, engine):
    """The 256x256 workload (N = 363, 360 angles), T0-T7 x P1-P3."""
    img = blob_image(256, 256, 8, (8, 40), (40, 200), 1)
    rep = check_transform(oracle_lib, engine, "single256", img, 1, [0, 1, 2, 3, 4, 5, 6, 7])
    assert rep["median_ties"] + rep["selection_ties"] <= 0.002 * rep["entries"], rep


def test_single1024_full_vs_oracle(oracle_lib, engine):
    """The 1024x1024 workload in full: N = 1449, all 360 angles, T0-T7 x
    P1-P3 -- every one of the 4.2 M sinogram and 8640 circus entries."""
    from tracetransform_gb300.synthetic import workload
    img, step = workload("single1024")[0]
    rep = check_transform(oracle_lib, engine, "single1024", img, int(step),
                          [0, 1, 2, 3, 4, 5, 6, 7])
    assert rep["median_ties"] + rep["selection_ties"] <= 0.002 * rep["entries"], rep


def test_single4096_angle_subset_vs_oracle(oracle_lib, engine):
    """The 4096x4096 workload (N = 5793, 0.5 degree steps): every 24th of its
    720 angles (30 angles, including the half-degree ones), T0-T7 x P1-P3."""
    from tracetransform_gb300.synthetic import workload
    img, step = workload("single4096")[0]
    idx = np.arange(0, 720, 24) + np.arange(30) % 2  # 15 whole and 15 half degrees
    ang = (idx.astype(np.float64) * 0.5).astype(np.float32)
    rep = check_transform(oracle_lib, engine, "single4096_subset", img, 0.5,
                          [0, 1, 2, 3, 4, 5, 6, 7], angles=ang)
    assert rep["median_ties"] + rep["selection_ties"] <= 0.002 * rep["entries"], rep


def test_circus_vs_oracle(oracle_lib):
    img = blob_image(64, 64, 6, (3, 12), (40, 200), 7)
    padded = oracle_lib.pad(img)
    ang = oracle_lib.angles_for_step(2)
    sino = oracle_lib.sinograms(padded, ang, [0, 1, 3])
    n = padded.shape[0]
    center = n // 2 - 3
    pf_ref = [(1, 0, 0), (2, 0, 0), (3, 0, 0)] + [(0, o, center) for o in (1, 2, 3, 4, 5)]
    pfs = [tt.PFunctionalWrapper.parse(s) for s in ("1", "2", "3", "H1", "H2", "H3", "H4", "H5")]
    for p in pfs[3:]:
        p.arguments.center = center
    got = np.stack([np.stack(tt.getCircusFunctions(sino[t], pfs)) for t in range(sino.shape[0])])
    rep = account_circus(sino, pf_ref, got)
    record("circus64", rep)
    assert_accounted(rep, "circus")


@pytest.mark.parametrize("rows,cols,ns", [(1, 5, 1), (2, 7, 2), (3, 130, 1), (17, 129, 3),
                                          (130, 257, 2), (1449, 40, 2), (2048, 131, 1)])
def test_p_stage_tensor_core_edges(oracle_lib, engine, rows, cols, ns):
    """P1-P3 of sinogram stacks through tt_circus_device -- P3 on the tensor
    cores with the precomputed twiddle blocks -- at its edges: the shortest
    columns (one to three frequencies: the smallest MMA width), column counts
    that leave partial 128-column tiles, and the longest columns the DFT path
    takes (2048 rows), against the oracle's P-stage, every entry accounted."""
    import torch
    rng = np.random.default_rng(rows * 1000 + cols)
    t = np.linspace(-1, 1, rows)
    sino = (np.exp(-(t[None, :, None] / rng.uniform(0.2, 0.6, (ns, 1, cols))) ** 2) *
            rng.uniform(1, 50, (ns, 1, cols)) + rng.uniform(0, 0.5, (ns, rows, cols)))
    sino = sino.astype(np.float32)
    dev = torch.from_numpy(np.ascontiguousarray(sino.transpose(0, 2, 1))).cuda()
    got = engine.circus(dev, [(k, -1, -1) for k in (1, 2, 3)])
    torch.cuda.synchronize()
    got = got.cpu().numpy()
    rep = account_circus(sino, P123, got)
    record(f"p_stage_edges_{rows}x{cols}x{ns}", rep)
    assert_accounted(rep, f"P-stage {rows} x {cols} x {ns}")


def test_zscore_bit_exact(oracle_lib):
    rng = np.random.default_rng(3)
    for n in (2, 7, 360, 720):
        x = (rng.random(n) * 100).astype(np.float32)
        assert np.array_equal(tt.zscore(x), oracle_lib.zscore(x))


@pytest.mark.parametrize("name", ["zeros", "const", "tiny3", "tiny5", "line1xN", "nonsquare"])
def test_edge_images(oracle_lib, engine, name):
    imgs = {
        "zeros": np.zeros((12, 12), np.float32, order="F"),
        "const": np.full((9, 9), 0.5, np.float32, order="F"),
        "tiny3": blob_image(3, 3, 1, (1, 2), (40, 200), 5),
        "tiny5": blob_image(5, 5, 2, (1, 2), (40, 200), 6),
        "line1xN": blob_image(1, 17, 2, (1, 3), (40, 200), 7),
        "nonsquare": blob_image(40, 9, 3, (1, 4), (40, 200), 8),
    }
    img = imgs[name]
    tfs = [0, 1, 2, 3, 4, 5, 6, 7]
    check_transform(oracle_lib, engine, name, img, 5, tfs)
    # the drop-in Transformer computes the same circus functions and signatures
    ref = oracle_lib.transform(img, 5, tfs, [(1, 0), (2, 0), (3, 0)])
    tr = tt.Transformer(img, name, 5, False)
    sig = tr.getTransform([str(t) for t in tfs], ["1", "2", "3"], write_data=False)
    assert zscore_mismatches(tr.circus, sig.T.reshape(tr.circus.shape)) == 0
    got, got_med = engine_sinograms(engine, img, oracle_lib.angles_for_step(5), tfs)
    assert account_circus(got, P123, tr.circus)["unexplained"] == 0
    assert tr.circus.shape == ref["circus"].shape


def test_invalid_arguments_raise():
    with pytest.raises(ValueError):
        tt.getSinograms(np.zeros((5, 6), np.float32), 1, ["0"])     # not square
    with pytest.raises(tt.ValidationError):
        tt.getSinograms(np.zeros((5, 5), np.float32), 1, ["9"])
    with pytest.raises(tt.ValidationError):
        tt.Transformer(np.zeros((5, 5), np.float32), "x", 1, False).getTransform(["0"], ["1", "H1"])
