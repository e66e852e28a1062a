"""Device-resident entry points on torch CUDA tensors (stream ordered).

Layouts (torch tensors are row-major, the engine is column-major):

* an image of R rows and C columns is a (C, R) contiguous tensor holding the
  column-major matrix -- ``to_colmajor`` / ``from_colmajor`` convert;
* a sinogram stack is (nT, A, N): ``sino[t, a]`` is column a (angle a) of
  sinogram t, i.e. the engine's nT x N x A column-major stack;
* circus functions are (nT, nP, A); signatures the same shape, z-scored.

Work is enqueued on torch's current CUDA stream of the tensor's device.
"""
from __future__ import annotations

import ctypes
from typing import Optional, Sequence

import numpy as np
import torch

from ._native import PFunctionalC, check, lib
from .api import Plan, angles_from_step, pad_geometry


def to_colmajor(image: torch.Tensor) -> torch.Tensor:
    """(R, C) tensor -> (C, R) contiguous tensor holding it column-major."""
    return image.t().contiguous()


def from_colmajor(buf: torch.Tensor) -> torch.Tensor:
    """(C, R) column-major storage -> (R, C) view."""
    return buf.t()


_CUDA_STREAM_LEGACY = 1  # cudaStreamLegacy: the NULL stream's explicit handle


def _stream(t: torch.Tensor):
    """Handle of torch's current stream.  torch's default stream is the legacy
    NULL stream (handle 0), which the C ABI would read as "the plan's own
    stream", so it is passed as cudaStreamLegacy."""
    h = torch.cuda.current_stream(t.device).cuda_stream
    return ctypes.c_void_p(h if h else _CUDA_STREAM_LEGACY)


def _ptr(t: Optional[torch.Tensor]):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _pf(pfuncs):
    arr = (PFunctionalC * max(len(pfuncs), 1))()
    for i, p in enumerate(pfuncs):
        kind, order, center = (tuple(p) + (-1, -1))[:3]
        arr[i].kind, arr[i].order, arr[i].center = int(kind), int(order), int(center)
    return arr


class Engine:
    """One device's plan plus tensor-level calls of the C ABI."""

    def __init__(self, device: int = 0):
        self.device = torch.device("cuda", device)
        self.plan = Plan(device)

    def sinograms(self, image_cm: torch.Tensor, rows: int, cols: int, angles_deg, tfuncs,
                  padded: bool = False, medians: bool = False,
                  out: Optional[torch.Tensor] = None, med_out: Optional[torch.Tensor] = None):
        """Sinograms of a column-major image (see module doc).

        padded=False: image_cm is the unpadded R x C image, placed in its pad()
        frame implicitly; padded=True: it already is the N x N frame."""
        if padded:
            n, ro, co = rows, 0, 0
            if rows != cols:
                raise ValueError("a padded image must be square")
        else:
            n, ro, co = pad_geometry(rows, cols)
        ang = np.ascontiguousarray(np.asarray(angles_deg, np.float32))
        ids = np.ascontiguousarray(np.asarray([int(t) for t in tfuncs], np.int32))
        if out is None:
            out = torch.empty((len(ids), len(ang), n), dtype=torch.float32, device=image_cm.device)
        med = None
        if medians:
            med = med_out if med_out is not None else torch.empty_like(out, dtype=torch.int32)
        check(lib().tt_sinograms_device(
            self.plan.handle, _ptr(image_cm), rows, cols, rows, n, ro, co,
            ang.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), len(ang),
            ids.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), len(ids), _ptr(out), _ptr(med),
            _stream(image_cm)))
        return (out, med) if medians else out

    def circus(self, sino: torch.Tensor, pfuncs: Sequence, centers=None,
               out: Optional[torch.Tensor] = None) -> torch.Tensor:
        """P-functionals of a (nS, A, N) sinogram stack -> (nS, nP, A).
        pfuncs: (kind, order, center) tuples; centers: per-sinogram Hermite
        centers overriding theirs."""
        ns, a, n = sino.shape
        if out is None:
            out = torch.empty((ns, len(pfuncs), a), dtype=torch.float32, device=sino.device)
        cptr = None
        if centers is not None:
            c = np.ascontiguousarray(np.asarray(centers, np.int32))
            cptr = c.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
        check(lib().tt_circus_device(self.plan.handle, _ptr(sino), n, a, ns, _pf(pfuncs),
                                     len(pfuncs), cptr, _ptr(out), _stream(sino)))
        return out

    def circus_orthonormal(self, sino: torch.Tensor, orders: Sequence[int],
                           out: Optional[torch.Tensor] = None):
        """Hermite circus of each sinogram's nearest orthonormal sinogram:
        (nS, A, N) -> ((nS, len(orders), A), centers); self.last_sweeps holds
        the Jacobi sweeps the call took."""
        ns, a, n = sino.shape
        if out is None:
            out = torch.empty((ns, len(orders), a), dtype=torch.float32, device=sino.device)
        centers = np.zeros(max(ns, 1), np.int32)
        sweeps = ctypes.c_int32(0)
        check(lib().tt_circus_orthonormal_device(
            self.plan.handle, _ptr(sino), n, a, ns, _pf([(0, int(o), -1) for o in orders]),
            len(orders), _ptr(out), centers.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
            ctypes.byref(sweeps), _stream(sino)))
        self.last_sweeps = sweeps.value
        return out, centers[:ns]

    def zscore(self, circus: torch.Tensor, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        length = circus.shape[-1]
        nvec = circus.numel() // max(length, 1)
        if out is None:
            out = torch.empty_like(circus)
        check(lib().tt_zscore_device(self.plan.handle, _ptr(circus), nvec, length, _ptr(out),
                                     _stream(circus)))
        return out

    # ---- backward and double precision -----------------------------------
    def circus_backward(self, sino: torch.Tensor, pfuncs, grad_circus: torch.Tensor):
        """Adjoint of circus(): (nS, nP, A) gradient -> (nS, A, N) gradient."""
        ns, a, n = sino.shape
        out = torch.empty_like(sino)
        fn = (lib().tt_circus_backward_f64_device if sino.dtype == torch.float64
              else lib().tt_circus_backward_device)
        check(fn(self.plan.handle, _ptr(sino), n, a, ns, _pf(pfuncs), len(pfuncs),
                 _ptr(grad_circus.contiguous()), _ptr(out), _stream(sino)))
        return out

    def sinograms_backward(self, grad_sino: torch.Tensor, medians: torch.Tensor, rows: int,
                           cols: int, angles_deg, tfuncs) -> torch.Tensor:
        """Adjoint of sinograms() for T0-T2.  grad_sino / medians: (nT, A, N)
        or a batch (B, nT, A, N) of same-size images; returns the column-major
        image gradient(s), (cols, rows) or (B, cols, rows)."""
        n, ro, co = pad_geometry(rows, cols)
        batch = grad_sino.dim() == 4
        b = grad_sino.shape[0] if batch else 1
        ang = np.ascontiguousarray(np.asarray(angles_deg, np.float32))
        ids = np.ascontiguousarray(np.asarray([int(t) for t in tfuncs], np.int32))
        out = torch.empty((b, cols, rows), dtype=grad_sino.dtype, device=grad_sino.device)
        fn = (lib().tt_sinograms_backward_f64_device if grad_sino.dtype == torch.float64
              else lib().tt_sinograms_backward_device)
        check(fn(self.plan.handle, b, rows, cols, n, ro, co,
                 ang.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), len(ang),
                 ids.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), len(ids),
                 _ptr(grad_sino.contiguous()), _ptr(medians.contiguous()), _ptr(out),
                 _stream(grad_sino)))
        return out if batch else out[0]

    def sinograms_f64(self, image_cm: torch.Tensor, rows: int, cols: int, angles_deg, tfuncs,
                      out: Optional[torch.Tensor] = None, med_out: Optional[torch.Tensor] = None):
        """T0-T2 sinograms of a double image in double: (nT, A, N) and medians."""
        n = pad_geometry(rows, cols)[0]
        ang = np.ascontiguousarray(np.asarray(angles_deg, np.float32))
        ids = np.ascontiguousarray(np.asarray([int(t) for t in tfuncs], np.int32))
        if out is None:
            out = torch.empty((len(ids), len(ang), n), dtype=torch.float64,
                              device=image_cm.device)
        med = med_out if med_out is not None else torch.empty(out.shape, dtype=torch.int32,
                                                                device=image_cm.device)
        check(lib().tt_sinograms_f64_device(
            self.plan.handle, _ptr(image_cm), rows, cols,
            ang.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), len(ang),
            ids.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), len(ids), _ptr(out), _ptr(med),
            _stream(image_cm)))
        return out, med

    def circus_f64(self, sino: torch.Tensor, pfuncs) -> torch.Tensor:
        ns, a, n = sino.shape
        out = torch.empty((ns, len(pfuncs), a), dtype=torch.float64, device=sino.device)
        check(lib().tt_circus_f64_device(self.plan.handle, _ptr(sino), n, a, ns, _pf(pfuncs),
                                         len(pfuncs), _ptr(out), _stream(sino)))
        return out

    def transform_batch(self, flat: torch.Tensor, offsets, rows, cols, steps, tfuncs, pfuncs,
                        circus: Optional[torch.Tensor] = None,
                        signatures: Optional[torch.Tensor] = None):
        """Batched engine on device: flat holds the column-major images at
        element offsets; returns flat circus and signature tensors (image after
        image, n_t x n_p x A_i each)."""
        off = np.ascontiguousarray(np.asarray(offsets, np.int64))
        r = np.ascontiguousarray(np.asarray(rows, np.int32))
        c = np.ascontiguousarray(np.asarray(cols, np.int32))
        s = np.ascontiguousarray(np.asarray(steps, np.int32))
        ids = np.ascontiguousarray(np.asarray([int(t) for t in tfuncs], np.int32))
        total = int(sum(len(ids) * len(pfuncs) * (360 // int(x)) for x in s))
        if circus is None:
            circus = torch.empty(max(total, 1), dtype=torch.float32, device=flat.device)
        if signatures is None:
            signatures = torch.empty(max(total, 1), dtype=torch.float32, device=flat.device)
        I32 = ctypes.POINTER(ctypes.c_int32)
        check(lib().tt_transform_batch_device(
            self.plan.handle, _ptr(flat), off.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
            r.ctypes.data_as(I32), c.ctypes.data_as(I32), s.ctypes.data_as(I32), len(r),
            ids.ctypes.data_as(I32), len(ids), _pf(pfuncs), len(pfuncs), _ptr(circus),
            _ptr(signatures), _stream(flat)))
        return circus, signatures

    def batch_sinograms(self, like: torch.Tensor) -> torch.Tensor:
        """The sinograms behind the last transform_batch call, flat: image
        after image in input order, each (nT, A_i, N_i)."""
        count = ctypes.c_int64(0)
        check(lib().tt_transform_batch_sinograms_device(self.plan.handle, None, 0,
                                                        ctypes.byref(count), _stream(like)))
        out = torch.empty(max(count.value, 1), dtype=torch.float32, device=like.device)
        check(lib().tt_transform_batch_sinograms_device(self.plan.handle, _ptr(out), out.numel(),
                                                        ctypes.byref(count), _stream(like)))
        return out[:count.value]

    def batch_stage_ms(self):
        """Device ms of the last transform_batch call's sinogram, P-functional
        and z-score kernels (waits for it)."""
        ms = (ctypes.c_float * 3)()
        check(lib().tt_transform_batch_stage_ms(self.plan.handle, ms))
        return [float(v) for v in ms]

    def batch_tile(self, pin=None):
        """The batched sinogram kernel's tile (lines per CTA, CTAs per SM,
        lines per warp) of the last batch; pin=(lines, ctas_per_sm,
        lines_per_warp) fixes it for the next batches (ctas_per_sm 0: tune)."""
        t = (ctypes.c_int32 * 3)(*(pin or (0, 0, 0)))
        check(lib().tt_transform_batch_tile(self.plan.handle, t, 1 if pin else 0))
        return tuple(int(v) for v in t)

    def transform(self, image_cm: torch.Tensor, rows: int, cols: int, angles_deg, tfuncs,
                  pfuncs, out_sino=None):
        """Regular (non-orthonormal) transform on the device: returns
        (sinograms, circus, signatures) tensors."""
        sino = self.sinograms(image_cm, rows, cols, angles_deg, tfuncs, out=out_sino)
        circ = self.circus(sino, [(k, o, -1) for k, o in pfuncs])
        return sino, circ, self.zscore(circ)


__all__ = ["Engine", "to_colmajor", "from_colmajor", "angles_from_step"]
