"""Differentiable circus functions: torch.autograd over the engine's C ABI.

``circus(images, angles, tfuncs, pfuncs)`` returns the raw circus functions
(T-functional x P-functional x angle) of each image and back-propagates to the
images through the hand-written adjoint kernels (tt_circus_backward_device,
tt_sinograms_backward_device): P1/P3 adjoints per sinogram column, T0/T1/T2
adjoints with the weighted median held at the row the forward chose, and the
rotation adjoint gathered per pixel with the rotations recomputed.

float32 tensors run the fused forward kernel; float64 tensors run the
double-precision path (exact double coordinates), which is what
finite-difference checks use.  Differentiable functionals: T0, T1, T2 and
P1, P3.
"""
from __future__ import annotations

from typing import Dict, Sequence

import torch

from .device import Engine, to_colmajor

_engines: Dict[int, Engine] = {}


def engine_for(device: torch.device) -> Engine:
    idx = device.index if device.index is not None else torch.cuda.current_device()
    if idx not in _engines:
        _engines[idx] = Engine(idx)
    return _engines[idx]


class CircusFunction(torch.autograd.Function):
    """circus = P(T(rotate(pad(image)))) of one (rows, cols) image."""

    @staticmethod
    def forward(ctx, image, angles, tfuncs, pfuncs):
        eng = engine_for(image.device)
        rows, cols = image.shape
        cm = to_colmajor(image)
        pf = [(int(p), -1, -1) for p in pfuncs]
        if image.dtype == torch.float64:
            sino, med = eng.sinograms_f64(cm, rows, cols, angles, tfuncs)
            circ = eng.circus_f64(sino, pf)
        else:
            sino, med = eng.sinograms(cm, rows, cols, angles, tfuncs, medians=True)
            circ = eng.circus(sino, pf)
        ctx.save_for_backward(sino, med)
        ctx.meta = (rows, cols, tuple(angles), tuple(tfuncs), pf)
        return circ

    @staticmethod
    def backward(ctx, grad_circ):
        sino, med = ctx.saved_tensors
        rows, cols, angles, tfuncs, pf = ctx.meta
        eng = engine_for(sino.device)
        grad_sino = eng.circus_backward(sino, pf, grad_circ.to(sino.dtype).contiguous())
        grad_cm = eng.sinograms_backward(grad_sino, med, rows, cols, angles, tfuncs)
        return grad_cm.t(), None, None, None


def circus(images: torch.Tensor, angles: Sequence[float], tfuncs: Sequence[int],
           pfuncs: Sequence[int]) -> torch.Tensor:
    """Circus functions of a (rows, cols) image or a (B, rows, cols) batch:
    (nT, nP, A) or (B, nT, nP, A)."""
    angles = [float(a) for a in angles]
    tfuncs = [int(t) for t in tfuncs]
    pfuncs = [int(p) for p in pfuncs]
    if images.dim() == 2:
        return CircusFunction.apply(images, angles, tfuncs, pfuncs)
    return torch.stack([CircusFunction.apply(im, angles, tfuncs, pfuncs) for im in images])
