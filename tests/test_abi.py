"""C ABI checks that need no GPU: the library loads, exports every symbol the
header declares, and its host-only entry points agree with the oracle."""
import re

import numpy as np
import pytest

import tracetransform_gb300 as tt
from tracetransform_gb300 import _native
from tracetransform_gb300.api import PFunctionalWrapper, TFunctionalWrapper, ValidationError


def header_symbols():
    import os
    path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                        "tracetransform.h")
    text = open(path).read()
    return set(re.findall(r"^(?:tt_status|const char \*)\s*(tt_\w+)\s*\(", text, re.M))


@pytest.fixture(scope="module")
def lib():
    from tracetransform_gb300 import build
    build.build()
    return _native.lib()


def test_exports_every_declared_symbol(lib):
    declared = header_symbols()
    assert declared, "no declarations parsed from include/tracetransform.h"
    assert declared == set(_native.EXPORTS)
    for name in declared:
        assert hasattr(lib, name), name


def test_version(lib):
    assert b"sm_103a" in lib.tt_version()


@pytest.mark.parametrize("shape", [(256, 256), (1024, 1024), (4096, 4096), (20, 13), (13, 20),
                                   (3, 3), (1, 1), (2, 7), (511, 64)])
def test_pad_geometry_matches_oracle(lib, oracle_lib, shape):
    assert tt.pad_geometry(*shape) == oracle_lib.pad_geometry(*shape)


def test_pad_places_image(lib, oracle_lib):
    img = np.asfortranarray(np.arange(20 * 13, dtype=np.float32).reshape(20, 13))
    assert np.array_equal(tt.pad(img), oracle_lib.pad(img))


@pytest.mark.parametrize("step", [1, 2, 3, 4, 7, 45, 360])
def test_angles_and_ortho_size(lib, oracle_lib, step):
    assert np.array_equal(tt.angles_from_step(step), oracle_lib.angles_for_step(step))
    assert tt.ortho_size(step) == oracle_lib.ortho_size(step)


def test_parsers_follow_reference():
    assert TFunctionalWrapper.parse("0").name == "Radon"
    assert int(TFunctionalWrapper.parse("7").functional) == 7
    for bad in ("8", "-1", "", "T1", "01"):
        with pytest.raises(ValidationError):
            TFunctionalWrapper.parse(bad)
    assert PFunctionalWrapper.parse("3").name == "P3"
    h = PFunctionalWrapper.parse("H12")
    assert h.arguments.order == 12 and int(h.functional) == 0
    for bad in ("H", "Hx", "4", "0", "P1"):
        with pytest.raises(ValidationError):
            PFunctionalWrapper.parse(bad)


def test_invalid_arguments_fail_before_compute(lib):
    # host-side validation happens before any device work, so these fail the
    # same way with or without a GPU (reference: assert / validation_error)
    n = ctypesint = None  # noqa: F841
    st = lib.tt_ortho_size(0, None)
    assert st == 1
    assert b"step" in lib.tt_last_error()
    st = lib.tt_pad_geometry(0, 5, None, None, None)
    assert st == 1


def test_compute_without_gpu_raises(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(_native.TTError):
        tt.getSinograms(np.zeros((5, 5), np.float32), 1, ["0"])
    with pytest.raises(_native.TTError):
        tt.resize(np.zeros((5, 5), np.float32), 3, 3)


def test_transformer_validation_before_compute():
    """Transformer checks its arguments on the host, as the reference's
    constructor and demo do (c++/src/transform.cpp:28-47,
    c++/src/demo.cpp:153-169), so these fail the same way without a GPU."""
    img = np.zeros((8, 8), np.float32)
    with pytest.raises(ValidationError):
        tt.Transformer(img, "x", 0, False)
    tr = tt.Transformer(img, "x", 4, False)
    with pytest.raises(ValidationError, match="Cannot mix"):
        tr.getTransform(["0"], ["1", "H2"], write_data=False)
    with pytest.raises(ValidationError, match="orthonormal"):
        tr.getTransform(["0"], ["H2"], write_data=False)
    with pytest.raises(ValidationError):
        tr.getTransform(["9"], ["1"], write_data=False)
