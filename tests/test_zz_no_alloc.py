"""The allocation-free entry point, tt_circus_zscore_noalloc.

It exists for callers that may not allocate device memory while they run (a
plugin whose host application's allocator owns the device memory, or a loop
that cannot take cudaMalloc/cudaFree stalls): it computes P1/P2/P3 circus
functions and their z-scores using only a fixed 4 MiB device array compiled
into the library.  These tests call it through the C ABI and compare it with
the allocating path (tt_circus_device + tt_zscore_device) on two calls in a
row, whose shared scratch must not leak from one call into the next.

The file sorts last on purpose, so that a failure here comes after every
other test has run; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from parity import close_mask

pytestmark = pytest.mark.gpu


def _pf(kinds):
    from tracetransform_gb300._native import PFunctionalC
    arr = (PFunctionalC * len(kinds))()
    for i, k in enumerate(kinds):
        arr[i].kind, arr[i].order, arr[i].center = k, -1, -1
    return arr


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_matches_allocating_path_twice():
    import torch
    from tracetransform_gb300 import _native
    from tracetransform_gb300.device import Engine, _stream

    lib = _native.lib()
    eng = Engine(0)
    kinds = [1, 2, 3]
    # two calls in a row with different shapes and data
    for seed, (ns, a, n) in ((1, (3, 90, 47)), (2, (2, 120, 93))):
        gen = torch.Generator(device="cuda").manual_seed(seed)
        sino = torch.rand((ns, a, n), generator=gen, device="cuda", dtype=torch.float32) * 50
        want = eng.zscore(eng.circus(sino, [(k, -1, -1) for k in kinds]))
        got = torch.full_like(want, float("nan"))
        st = lib.tt_circus_zscore_noalloc(_ptr(sino), n, a, ns, _pf(kinds), len(kinds), _ptr(got),
                                          _stream(sino))
        assert st == 0, lib.tt_last_error()
        torch.cuda.synchronize()
        g, w = got.cpu().numpy(), want.cpu().numpy()
        assert np.isfinite(g).all()
        assert close_mask(g, w).all()


def test_noalloc_rejects_what_it_cannot_hold():
    import torch
    from tracetransform_gb300 import _native
    from tracetransform_gb300.device import _stream

    lib = _native.lib()
    sino = torch.zeros((8, 720, 300), device="cuda")
    out = torch.empty((8, 3, 720), device="cuda")
    # 8 * 3 * 720 circus values fit; 3 * 400000 (over 1048576 floats) do not
    big = torch.zeros((1, 400000, 3), device="cuda")
    big_out = torch.empty((1, 3, 400000), device="cuda")
    st = lib.tt_circus_zscore_noalloc(_ptr(big), 3, 400000, 1, _pf([1, 2, 3]), 3, _ptr(big_out),
                                      _stream(big))
    assert st == 1 and b"4 MiB" in lib.tt_last_error()
    st = lib.tt_circus_zscore_noalloc(_ptr(sino), 300, 720, 8, _pf([0]), 1, _ptr(out), _stream(sino))
    assert st == 2  # Hermite needs per-sinogram bases
    st = lib.tt_circus_zscore_noalloc(_ptr(sino), 300, 720, 8, _pf([1, 2, 3]), 3, _ptr(out),
                                      _stream(sino))
    assert st == 0, lib.tt_last_error()
    torch.cuda.synchronize()
