"""tt_transform_extended: P1-P3 and the orthonormal Hermite circus of the
same sinograms in one host-buffer call, equal bit for bit to the same work
done through the device entry points one stage at a time, and its regular
part equal to the drop-in tt_transform's."""
import numpy as np
import pytest

import tracetransform_gb300 as tt
from tracetransform_gb300.synthetic import blob_image

pytestmark = pytest.mark.gpu


def test_extended_equals_staged_device_calls():
    import torch
    from tracetransform_gb300.device import Engine, to_colmajor
    img = blob_image(64, 60, 5, (3, 10), (40, 200), 4)
    ang = tt.angles_from_step(5)
    tfs, pfs, orders = [0, 1, 3], [1, 2, 3], [1, 2, 3]
    ext = tt.api.transform_extended(img, ang, [str(t) for t in tfs], [str(p) for p in pfs],
                                    orders)
    eng = Engine(0)
    dev = to_colmajor(torch.from_numpy(np.ascontiguousarray(img)).cuda())
    sino = eng.sinograms(dev, 64, 60, ang, tfs)
    circ = eng.circus(sino, [(p, -1, -1) for p in pfs])
    hc, centers = eng.circus_orthonormal(sino, orders)
    torch.cuda.synchronize()
    assert np.array_equal(ext["circus"], circ.cpu().numpy())
    assert np.array_equal(ext["signatures"], eng.zscore(circ).cpu().numpy(), equal_nan=True)
    assert np.array_equal(ext["hermite_circus"], hc.cpu().numpy())
    assert np.array_equal(ext["hermite_signatures"], eng.zscore(hc).cpu().numpy(),
                          equal_nan=True)
    assert list(ext["centers"]) == list(centers)
    tr = tt.Transformer(img, "x", 5, False)
    tr.getTransform([str(t) for t in tfs], [str(p) for p in pfs], write_data=False)
    assert np.array_equal(ext["circus"], tr.circus)


def test_extended_rejects_hermite_in_pfuncs():
    img = np.ones((8, 8), np.float32)
    with pytest.raises(tt.api._native.InvalidArgument):
        tt.api.transform_extended(img, [0.0, 90.0], ["0"], ["H1"], [1])
