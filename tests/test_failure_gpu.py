"""Failure behaviour of the C ABI, injected on the host (nothing here can
fault the GPU):

* device allocation failure: tt_debug_fail_allocations makes the library's
  next allocations fail as cudaMalloc would when the device is full; every
  entry point must report TT_ERR_OOM (the reference throws CUDAHelper::Error,
  cuda/src/cudahelper/errorhandling.hpp:24-31) and the plan must stay usable;
* non-finite and negative inputs: the reference does not check its inputs
  (c++/src/sinogram.cpp:67-178, circus.cpp:104-177), neither does the engine;
  every entry point must return TT_OK, and where the reference's result is
  determined by plain arithmetic the engine's is the same: the Radon
  sinogram's NaN pattern (the bilinear samples are bit-identical, so a NaN
  or infinite pixel poisons exactly the reference's samples) and the
  z-scores of a vector holding NaN;
* invalid ids and sizes: TT_ERR_INVALID_ARG from every entry point (the
  reference's validation_error / assert).
"""
import ctypes

import numpy as np
import pytest

import tracetransform_gb300 as tt
from tracetransform_gb300 import _native
from tracetransform_gb300.synthetic import blob_image

pytestmark = pytest.mark.gpu
OOM, INVALID = 5, 1


@pytest.fixture
def disarm():
    yield
    _native.lib().tt_debug_fail_allocations(0)


def _status(fn, *args):
    try:
        fn(*args)
    except _native.TTError as e:
        return e.status
    return 0


def test_allocation_failure_is_oom_and_the_plan_recovers(disarm):
    img = blob_image(40, 36, 4, (3, 9), (40, 200), 2)
    lib = _native.lib()
    for call in (
        lambda p: tt.Transformer(img, "x", 6, False, plan=p).getTransform(
            ["0", "1", "6"], ["1", "3"], write_data=False),
        lambda p: tt.transform_batch([img, img[:20]], [6, 9], ["0", "2"], ["1", "2"], plan=p),
        lambda p: tt.api.transform_extended(img, tt.angles_from_step(6), ["0"], ["1"], [1],
                                            plan=p),
    ):
        plan = tt.Plan(0)  # a fresh plan: its first call allocates
        assert lib.tt_debug_fail_allocations(1) == 0
        assert _status(call, plan) == OOM
        assert b"out of memory" in lib.tt_last_error().lower() or \
            b"memory" in lib.tt_last_error().lower()
        assert lib.tt_debug_fail_allocations(0) == 0
        assert _status(call, plan) == 0  # the same plan works once memory is there
    assert lib.tt_debug_fail_allocations(-1) == INVALID


def test_nan_inf_images_radon_pattern_matches_reference(oracle_lib):
    img = blob_image(30, 34, 4, (3, 9), (40, 200), 3).copy(order="F")
    img[5, 7] = np.nan
    img[20, 30] = np.inf
    img[12, 2] = -np.inf
    tfs = [0, 1, 2, 3, 4, 5, 6, 7]
    step = 5
    padded = oracle_lib.pad(img)
    ref = oracle_lib.sinograms(padded, oracle_lib.angles_for_step(step), [0])[0]
    got = np.stack(tt.getSinograms(padded, step, [str(t) for t in tfs]))  # TT_OK for all T
    assert np.array_equal(np.isnan(got[0]), np.isnan(ref))
    assert np.array_equal(np.isinf(got[0]), np.isinf(ref))
    tr = tt.Transformer(img, "nan", step, False)
    tr.getTransform([str(t) for t in tfs], ["1", "2", "3"], write_data=False)
    assert tr.circus.shape == (len(tfs), 3, 360 // step)
    tt.transform_batch([img, img], [step, step], [str(t) for t in tfs], ["1", "2", "3"])
    tt.api.transform_extended(img, tt.angles_from_step(step), ["0", "1"], ["1", "2", "3"],
                              [1, 2])


def test_negative_images_run_every_functional(oracle_lib):
    """Negative pixels reach the selections of T6 / T7 (negative keys) and P2's
    exact-sort fallback; every entry point returns, and the Radon sinogram --
    a plain sum -- is the reference's.  (Where the reference takes square roots
    of negative samples, T3-T7, its results are NaN-propagated; the engine's
    are not specified there.)"""
    from parity import close_mask
    img = (blob_image(33, 29, 4, (3, 9), (40, 200), 4) - 0.5).astype(np.float32, order="F")
    tfs = [str(t) for t in range(8)]
    tr = tt.Transformer(img, "neg", 4, False)
    sig = tr.getTransform(tfs, ["1", "2", "3"], write_data=False)
    assert sig.shape == (90, 24)
    tt.transform_batch([img, np.abs(img)], [4, 3], tfs, ["1", "2", "3"])
    padded = oracle_lib.pad(img)
    ref = oracle_lib.sinograms(padded, oracle_lib.angles_for_step(4), [0])[0]
    got = tt.getSinograms(padded, 4, ["0"])[0]
    assert close_mask(got.T, ref.T).all()


def test_nan_sinograms_through_the_p_stage_and_zscore(oracle_lib):
    rng = np.random.default_rng(5)
    sino = (rng.random((61, 40)) * 10).astype(np.float32, order="F")
    sino[3, 4] = np.nan
    sino[9, 11] = np.inf
    pfs = [tt.PFunctionalWrapper.parse(s) for s in ("1", "2", "3")]
    out = np.stack(tt.getCircusFunctions(sino, pfs))          # TT_OK
    assert np.isnan(out[0, 4]) and np.isinf(out[0, 11])       # P1 is a plain sum
    v = sino[:, 4].copy()
    assert np.array_equal(tt.zscore(v), oracle_lib.zscore(v), equal_nan=True)
    tt.nearest_orthonormal_sinogram(sino)                     # bounded sweeps: returns
    import torch
    d = torch.from_numpy(np.ascontiguousarray(sino.T)).cuda()
    res = torch.empty((1, 3, 40), device="cuda")
    pf = (_native.PFunctionalC * 3)()
    for i, k in enumerate((1, 2, 3)):
        pf[i].kind, pf[i].order, pf[i].center = k, -1, -1
    st = _native.lib().tt_circus_zscore_noalloc(ctypes.c_void_p(d.data_ptr()), 61, 40, 1, pf, 3,
                                                ctypes.c_void_p(res.data_ptr()), None)
    torch.cuda.synchronize()
    assert st == 0


def test_invalid_ids_and_sizes_every_entry_point():
    lib = _native.lib()
    F = ctypes.POINTER(ctypes.c_float)
    img = np.zeros((5, 5), np.float32)
    out = np.zeros(10000, np.float32)
    fp = lambda a: a.ctypes.data_as(F)
    bad_t = np.array([9], np.int32)
    ok_t = np.array([0], np.int32)
    pf_bad = (_native.PFunctionalC * 1)()
    pf_bad[0].kind, pf_bad[0].order, pf_bad[0].center = 7, -1, -1
    pf_ok = (_native.PFunctionalC * 1)()
    pf_ok[0].kind, pf_ok[0].order, pf_ok[0].center = 1, -1, -1
    ip = _native.iptr
    assert lib.tt_sinograms(None, fp(img), 5, 5, 1, ip(bad_t), 1, fp(out)) == INVALID
    assert lib.tt_sinograms(None, fp(img), 5, 6, 1, ip(ok_t), 1, fp(out)) == INVALID
    assert lib.tt_sinograms(None, fp(img), 5, 5, 0, ip(ok_t), 1, fp(out)) == INVALID
    assert lib.tt_circus(None, fp(img), 5, 5, pf_bad, 1, fp(out)) == INVALID
    assert lib.tt_transform(None, fp(img), 5, 5, 1, ip(bad_t), 1, pf_ok, 1, fp(out),
                            fp(out)) == INVALID
    assert lib.tt_transform(None, fp(img), 0, 5, 1, ip(ok_t), 1, pf_ok, 1, fp(out),
                            fp(out)) == INVALID
    assert lib.tt_zscore(None, fp(img), -1, 5, fp(out)) == INVALID
    assert lib.tt_rotate(None, fp(img), 0, 5, 1.0, fp(out)) == INVALID
    assert lib.tt_resize(None, fp(img), 5, 5, 0, 3, fp(out)) == INVALID
    ang = np.zeros(4, np.float32)
    orders = np.array([-1], np.int32)  # no Hermite order -1
    st = lib.tt_transform_extended(None, fp(img), 5, 5, fp(ang), 4, ip(ok_t), 1, pf_ok, 1,
                                   ip(orders), 1, fp(out), fp(out), fp(out), fp(out), None)
    assert st == INVALID
    off = np.zeros(1, np.int64)
    rows = np.array([5], np.int32)
    steps = np.array([0], np.int32)
    st = lib.tt_transform_batch(None, fp(img), off.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                ip(rows), ip(rows), ip(steps), 1, ip(ok_t), 1, pf_ok, 1,
                                fp(out), fp(out))
    assert st == INVALID
    tile = (ctypes.c_int32 * 3)(3, 1, 3)  # no such tile shape
    assert lib.tt_transform_batch_tile(None, tile, 1) == INVALID
