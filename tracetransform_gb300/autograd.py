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

from .api import pad_geometry
from .device import Engine

_engines: Dict[int, Engine] = {}


def engine_for(device: torch.device) -> Engine:
    idx = device.index if device.index is not None else torch.cuda.current_device()
    if idx not in _engines:
        _engines[idx] = Engine(idx)
    return _engines[idx]


class CircusFunction(torch.autograd.Function):
    """circus = P(T(rotate(pad(images)))) of a (B, rows, cols) batch of
    same-size images: one sinogram launch per image, then one P-stage launch,
    one P-stage adjoint launch and one rotation-adjoint launch for the whole
    batch."""

    @staticmethod
    def forward(ctx, images, angles, tfuncs, pfuncs):
        eng = engine_for(images.device)
        b, rows, cols = images.shape
        n = pad_geometry(rows, cols)[0]
        cm = images.transpose(1, 2).contiguous()  # (B, cols, rows): column-major images
        pf = [(int(p), -1, -1) for p in pfuncs]
        shape = (b, len(tfuncs), len(angles), n)
        sino = torch.empty(shape, dtype=images.dtype, device=images.device)
        med = torch.empty(shape, dtype=torch.int32, device=images.device)
        for i in range(b):
            if images.dtype == torch.float64:
                eng.sinograms_f64(cm[i], rows, cols, angles, tfuncs, out=sino[i],
                                  med_out=med[i])
            else:
                eng.sinograms(cm[i], rows, cols, angles, tfuncs, medians=True, out=sino[i],
                              med_out=med[i])
        flat = sino.view(b * len(tfuncs), len(angles), n)
        circ = eng.circus_f64(flat, pf) if images.dtype == torch.float64 else eng.circus(flat, pf)
        ctx.save_for_backward(sino, med)
        ctx.meta = (rows, cols, tuple(angles), tuple(tfuncs), pf)
        return circ.view(b, len(tfuncs), len(pf), len(angles))

    @staticmethod
    def backward(ctx, grad_circ):
        sino, med = ctx.saved_tensors
        rows, cols, angles, tfuncs, pf = ctx.meta
        eng = engine_for(sino.device)
        b, nt, a, n = sino.shape
        g = grad_circ.to(sino.dtype).contiguous().view(b * nt, len(pf), a)
        grad_sino = eng.circus_backward(sino.view(b * nt, a, n), pf, g)
        grad_cm = eng.sinograms_backward(grad_sino.view(b, nt, a, n), med, rows, cols, angles,
                                         tfuncs)
        return grad_cm.transpose(1, 2), None, None, None


def circus(images: torch.Tensor, angles: Sequence[float], tfuncs: Sequence[int],
           pfuncs: Sequence[int]) -> torch.Tensor:
    """Circus functions of a (rows, cols) image or a (B, rows, cols) batch:
    (nT, nP, A) or (B, nT, nP, A)."""
    angles = [float(a) for a in angles]
    tfuncs = [int(t) for t in tfuncs]
    pfuncs = [int(p) for p in pfuncs]
    if images.dim() == 2:
        return CircusFunction.apply(images.unsqueeze(0), angles, tfuncs, pfuncs)[0]
    return CircusFunction.apply(images, angles, tfuncs, pfuncs)
