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


def _call(lib, sino, rows, cols, ns, kinds, out):
    from tracetransform_gb300.device import _stream
    return lib.tt_circus_zscore_noalloc(_ptr(sino), rows, cols, ns, _pf(kinds), len(kinds),
                                        _ptr(out), _stream(sino))


def test_noalloc_matches_allocating_path_twice():
    """Same kernels as the allocating path, so the same bits; two calls in a
    row with different shapes and data, the second must not see the first's
    scratch."""
    import torch
    from tracetransform_gb300 import _native
    from tracetransform_gb300.device import Engine

    lib = _native.lib()
    eng = Engine(0)
    kinds = [1, 2, 3]
    for seed, (ns, a, n) in ((1, (3, 90, 47)), (2, (2, 120, 93))):
        gen = torch.Generator(device="cuda").manual_seed(seed)
        sino = torch.rand((ns, a, n), generator=gen, device="cuda", dtype=torch.float32) * 50
        want = eng.zscore(eng.circus(sino, [(k, -1, -1) for k in kinds]))
        got = torch.full_like(want, float("nan"))
        st = _call(lib, sino, n, a, ns, kinds, got)
        assert st == 0, lib.tt_last_error()
        torch.cuda.synchronize()
        g, w = got.cpu().numpy(), want.cpu().numpy()
        assert np.isfinite(g).all()
        assert close_mask(g, w).all()
        assert np.array_equal(g, w)


def test_noalloc_allocates_nothing():
    """After a first call (which may load the module), further calls leave
    the device's free memory unchanged."""
    import torch
    from tracetransform_gb300 import _native

    lib = _native.lib()
    sino = torch.rand((4, 180, 400), device="cuda") * 10
    out = torch.empty((4, 3, 180), device="cuda")
    assert _call(lib, sino, 400, 180, 4, [1, 2, 3], out) == 0, lib.tt_last_error()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert _call(lib, sino, 400, 180, 4, [1, 2, 3], out) == 0, lib.tt_last_error()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_p3_at_its_row_limit():
    import torch
    from tracetransform_gb300 import _native
    from tracetransform_gb300.device import Engine

    lib = _native.lib()
    eng = Engine(0)
    sino = torch.rand((2, 16, 2048), device="cuda") * 5
    want = eng.zscore(eng.circus(sino, [(3, -1, -1)]))
    got = torch.empty_like(want)
    assert _call(lib, sino, 2048, 16, 2, [3], got) == 0, lib.tt_last_error()
    torch.cuda.synchronize()
    assert np.array_equal(got.cpu().numpy(), want.cpu().numpy())
    longer = torch.rand((1, 16, 2049), device="cuda")
    out = torch.empty((1, 1, 16), device="cuda")
    assert _call(lib, longer, 2049, 16, 1, [3], out) == 1
    assert b"2048" in lib.tt_last_error()


def test_noalloc_rejects_what_it_cannot_hold():
    import torch
    from tracetransform_gb300 import _native

    lib = _native.lib()
    # P1 over one sinogram of 3 rows: cols + 2 (cols + 1) floats, each part
    # rounded up to 64, fill the 1048576-float array exactly at cols = 349504
    full = torch.rand((1, 349505, 3), device="cuda")
    out = torch.empty((1, 1, 349505), device="cuda")
    assert _call(lib, full, 3, 349504, 1, [1], out) == 0, lib.tt_last_error()
    assert _call(lib, full, 3, 349505, 1, [1], out) == 1
    assert b"4 MiB" in lib.tt_last_error()
    sino = torch.zeros((8, 720, 300), device="cuda")
    out = torch.empty((8, 3, 720), device="cuda")
    assert _call(lib, sino, 300, 720, 8, [0], out) == 2  # Hermite needs per-sinogram bases
    assert _call(lib, sino, 300, 720, 8, [1, 2, 3], out) == 0, lib.tt_last_error()
    torch.cuda.synchronize()
