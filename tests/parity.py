"""Parity helpers shared by the GPU tests: the accounting in oracle/parity.py
(every entry within 1e-4 of the oracle or a proven tie of the reference's
own arithmetic) plus the engine / oracle calls the tests repeat."""
from __future__ import annotations

import json
import os

import numpy as np

from oracle.parity import (EPS_FRAC, RTOL, account_circus, account_sinograms,  # noqa: F401
                           close_mask, median_tie, rel_err, selection_tie, tie_rows,
                           zscore_mismatches)


def engine_sinograms(engine, img, angles, tfs):
    """Sinograms and weighted-median rows of an unpadded image through
    tt_sinograms_device (the call tt_transform makes): (nT, N, A) each."""
    import torch
    from tracetransform_gb300.device import to_colmajor
    dev = to_colmajor(torch.from_numpy(np.ascontiguousarray(img, np.float32)).cuda())
    out, med = engine.sinograms(dev, img.shape[0], img.shape[1], angles, tfs, medians=True)
    torch.cuda.synchronize()
    return out.cpu().numpy().transpose(0, 2, 1), med.cpu().numpy().transpose(0, 2, 1)


def assert_accounted(rep, what=""):
    assert rep["unexplained"] == 0, f"{what}: {rep['unexplained']} entries unexplained: " \
                                    f"{rep['details']}"


def record(name, rep):
    """Append a report to $TT_PARITY_REPORT (JSON lines) when it is set."""
    path = os.environ.get("TT_PARITY_REPORT")
    if not path:
        return
    slim = {k: v for k, v in rep.items() if k not in ("tie_columns",)}
    with open(path, "a") as f:
        f.write(json.dumps({"case": name, **slim}) + "\n")
