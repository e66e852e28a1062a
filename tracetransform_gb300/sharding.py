"""Multi-process sharding of the trace transform, one process per GPU.

Images are independent -- the reference's own multi-GPU mode gives each GPU
its own images (cuda/src/demo.cpp:258-266) -- and within one image every
circus entry depends only on its own angle's sinogram column
(c++/src/circus.cpp:129-154); only the z-score (c++/src/transform.cpp:95)
and the nearest orthonormal sinogram (c++/src/circus.cpp:68-102) need all
the angles of a sinogram.  Hence two partitionings:

* ``assign_images`` + ``transform_images_sharded``: the images of a batch
  to ranks, largest cost (4 A H W) first onto the least-loaded rank.  Every
  rank runs its images through the batched engine with no exchange; rank 0
  then gathers the finished per-image results.
* ``angle_ranges`` + ``transform_angle_sharded``: the angles of one large
  image in contiguous ranges, one per rank.  Each rank computes its sinogram
  columns and their raw circus entries; rank 0 gathers the raw circus
  vectors -- A floats per (T, P), the path's only exchange -- and z-scores
  them.  For the orthonormal (Hermite) circus it gathers the sinogram
  columns instead and runs the nearest orthonormal sinogram itself.

The exchange goes through ``torch.distributed`` (NCCL between GPUs, gloo in
the CPU tests).  The per-rank work is a ``Compute`` object; the default runs
the engine on this rank's GPU (and fails loudly without the CUDA library).
"""
from __future__ import annotations

from typing import List, Optional, Sequence, Tuple

import numpy as np

__all__ = ["angle_ranges", "assign_images", "image_cost", "EngineCompute",
           "transform_angle_sharded", "transform_images_sharded"]


def image_cost(rows: int, cols: int, n_angles: int) -> float:
    """Bytes one image's sinogram pass reads: 4 A H W."""
    return 4.0 * n_angles * rows * cols


def angle_ranges(n_angles: int, world: int) -> List[Tuple[int, int]]:
    """Contiguous [lo, hi) angle ranges, one per rank, sizes differing by at
    most one (the first n_angles % world ranks take the extra angle)."""
    if world < 1 or n_angles < 0:
        raise ValueError("need world >= 1 and n_angles >= 0")
    base, extra = divmod(n_angles, world)
    out, lo = [], 0
    for r in range(world):
        hi = lo + base + (1 if r < extra else 0)
        out.append((lo, hi))
        lo = hi
    return out


def assign_images(costs: Sequence[float], world: int) -> List[List[int]]:
    """Image indices per rank: greedy longest-processing-time order (largest
    cost first, ties by index) onto the least-loaded rank (ties by rank)."""
    if world < 1:
        raise ValueError("need world >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    load = [0.0] * world
    out: List[List[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda q: (load[q], q))
        out[r].append(i)
        load[r] += float(costs[i])
    return [sorted(o) for o in out]


class EngineCompute:
    """Per-rank work on this rank's GPU through the engine.  Arrays cross
    the host as numpy, angle axis last: sinograms (nT, N, A_r), circus
    (nT, nP, A_r)."""

    def __init__(self, device: int = 0):
        import torch
        from .device import Engine
        self._torch = torch
        self.engine = Engine(device)

    def sinograms(self, image: np.ndarray, angles_deg: np.ndarray, tfuncs) -> np.ndarray:
        from .device import to_colmajor
        torch = self._torch
        img = np.asarray(image, np.float32)
        dev = to_colmajor(torch.from_numpy(np.ascontiguousarray(img)).to(self.engine.device))
        s = self.engine.sinograms(dev, img.shape[0], img.shape[1], angles_deg, tfuncs)
        return s.transpose(1, 2).cpu().numpy()  # (nT, A, N) -> (nT, N, A)

    def circus(self, sino: np.ndarray, pfuncs) -> np.ndarray:
        torch = self._torch
        dev = torch.from_numpy(np.ascontiguousarray(sino.transpose(0, 2, 1))).to(self.engine.device)
        return self.engine.circus(dev, list(pfuncs)).cpu().numpy()

    def zscore(self, vectors: np.ndarray) -> np.ndarray:
        torch = self._torch
        dev = torch.from_numpy(np.ascontiguousarray(vectors, dtype=np.float32)).to(self.engine.device)
        return self.engine.zscore(dev).cpu().numpy()

    def transform_images(self, images, angle_steps, tfuncs, pfuncs):
        """The batched engine (regular P-functionals) on this rank's images:
        [(circus nT x nP x A_i, signatures A_i x (nT nP))] in input order."""
        torch = self._torch
        bufs = [np.ascontiguousarray(np.asarray(im, np.float32).ravel(order="F")) for im in images]
        offsets = np.zeros(len(bufs), np.int64)
        offsets[1:] = np.cumsum([b.size for b in bufs])[:-1]
        flat = torch.from_numpy(np.concatenate(bufs)).to(self.engine.device)
        circ, sig = self.engine.transform_batch(
            flat, offsets, [im.shape[0] for im in images], [im.shape[1] for im in images],
            [int(x) for x in angle_steps], tfuncs, list(pfuncs))
        circ, sig = circ.cpu().numpy(), sig.cpu().numpy()
        out, at = [], 0
        n_tp = len(tfuncs) * len(pfuncs)
        for x in angle_steps:
            a = 360 // int(x)
            out.append((circ[at:at + n_tp * a].reshape(len(tfuncs), len(pfuncs), a).copy(),
                        np.ascontiguousarray(sig[at:at + n_tp * a].reshape(n_tp, a).T)))
            at += n_tp * a
        return out

    def orthonormal(self, sino: np.ndarray, orders: Sequence[int]) -> np.ndarray:
        torch = self._torch
        dev = torch.from_numpy(np.ascontiguousarray(sino.transpose(0, 2, 1))).to(self.engine.device)
        circ, _ = self.engine.circus_orthonormal(dev, list(orders))
        return circ.cpu().numpy()


def _gather(obj, group):
    import torch.distributed as dist
    out = [None] * dist.get_world_size(group)
    dist.all_gather_object(out, obj, group=group)
    return out


def transform_angle_sharded(image, angle_stepsize: int, tfuncs: Sequence[int],
                            pfuncs: Sequence[Tuple[int, int, int]], rank: int, world: int,
                            group=None, compute=None):
    """Transformer::getTransform (c++/src/transform.cpp:49-112) of one image
    with its angles split over `world` ranks (call it on every rank).

    pfuncs: (kind, order, center) as tt_pfunctional (kind 0 = Hermite); all
    Hermite selects the orthonormal mode, as the reference's demo does
    (c++/src/demo.cpp:153-169), whose stretch to tt_ortho_size the caller
    applies to `image` first.  Returns, on rank 0, (circus nT x nP x A,
    signatures A x (nT nP)) -- column t nP + p of the signatures is the
    z-scored circus function (t, p) -- and None on every other rank."""
    from .api import angles_from_step
    compute = compute if compute is not None else EngineCompute()
    angles = np.asarray(angles_from_step(int(angle_stepsize)), np.float32)
    n_a = len(angles)
    lo, hi = angle_ranges(n_a, world)[rank]
    kinds = [int(p[0]) for p in pfuncs]
    n_herm = sum(1 for k in kinds if k == 0)
    if n_herm and n_herm != len(kinds):
        raise ValueError("Cannot mix regular and orthonormal P-functionals")
    sino = compute.sinograms(image, angles[lo:hi], tfuncs)  # (nT, N, A_r)
    if n_herm:
        # the nearest orthonormal sinogram needs every angle: gather the columns
        parts = _gather(sino, group) if world > 1 else [sino]
        if rank != 0:
            return None
        full = np.concatenate(parts, axis=2)
        circus = compute.orthonormal(full, [int(p[1]) for p in pfuncs])
    else:
        part = compute.circus(sino, pfuncs)  # (nT, nP, A_r)
        parts = _gather(part, group) if world > 1 else [part]
        if rank != 0:
            return None
        circus = np.concatenate(parts, axis=2)
    n_t, n_p = circus.shape[0], circus.shape[1]
    z = compute.zscore(circus.reshape(n_t * n_p, n_a))
    return circus, np.ascontiguousarray(z.reshape(n_t * n_p, n_a).T)


def transform_images_sharded(images, angle_steps, tfuncs: Sequence[int],
                             pfuncs: Sequence[Tuple[int, int, int]], rank: int, world: int,
                             group=None, compute=None):
    """A batch of independent images over `world` ranks (call it on every
    rank): each rank transforms its assign_images share (cost 4 A H W) in one
    batched call, and rank 0 gathers the per-image results.  Returns, on rank
    0, [(circus nT x nP x A_i, signatures A_i x (nT nP))] in input order, and
    None on every other rank."""
    compute = compute if compute is not None else EngineCompute()
    costs = [image_cost(im.shape[0], im.shape[1], 360 // int(st))
             for im, st in zip(images, angle_steps)]
    mine = assign_images(costs, world)[rank]
    results = (compute.transform_images([images[i] for i in mine],
                                        [angle_steps[i] for i in mine], tfuncs, pfuncs)
               if mine else [])
    local = list(zip(mine, results))
    parts = _gather(local, group) if world > 1 else [local]
    if rank != 0:
        return None
    out = [None] * len(images)
    for part in parts:
        for i, r in part:
            out[i] = r
    return out
