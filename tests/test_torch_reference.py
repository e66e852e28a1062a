"""The dense PyTorch-op restatement used as the reference gradient agrees with
the oracle's forward (T0-T2 sinograms, P1/P3 circus functions) on the CPU."""
import numpy as np
import torch

from tracetransform_gb300.synthetic import blob_image

import torch_reference as tref


def _check(O, rows, cols, step):
    img = np.ascontiguousarray(blob_image(rows, cols, 5, sigma=(2.0, 8.0), seed=rows * cols))
    angles = O.angles_for_step(step)
    sino, med = O.sinograms(O.pad(img), angles, [0, 1, 2], with_medians=True)
    ref = tref.sinograms(torch.from_numpy(img.astype(np.float64)), angles, [0, 1, 2],
                         torch.from_numpy(np.ascontiguousarray(med.transpose(0, 2, 1))))
    want = sino.transpose(0, 2, 1).astype(np.float64)
    assert np.abs(ref.numpy() - want).max() <= 1e-5 * np.abs(want).max()
    circ = tref.circus(ref, [1, 3]).numpy()
    for t in range(3):
        oc = O.circus(sino[t], [(1, -1, -1), (3, -1, -1)]).astype(np.float64)
        rel = np.abs(circ[t] - oc) / np.maximum(np.abs(oc), 1e-30)
        assert rel.max() <= 1e-4, (t, rel.max())


def test_torch_reference_square(oracle_lib):
    _check(oracle_lib, 20, 20, 7)


def test_torch_reference_ragged(oracle_lib):
    _check(oracle_lib, 13, 21, 3)
