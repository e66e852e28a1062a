"""Seeded synthetic blob-plus-noise images.

The reference ships no test images (its README points at a missing
``../../test/Cam1_V1.pgm``), so every workload here is generated: a sum of
isotropic Gaussian blobs plus uniform noise in [0, 16), clipped to [0, 255],
quantised to uint8 (round half to even) and scaled by 1/255 in double then
stored as float32 -- exactly what ``gray2mat`` does to a PGM
(c++/src/auxiliary.cpp:148-157), so every path sees identical floats.

Images are returned as float32 arrays of shape (rows, cols) in Fortran
(column-major) order, the storage order of the reference's Eigen matrices.
"""
from __future__ import annotations

import numpy as np

__all__ = ["blob_image", "blob_image_u8", "workload", "workload_u8", "write_pgm"]


def blob_image_u8(rows: int, cols: int, n_blobs: int, sigma: tuple[float, float],
                  amplitude: tuple[float, float], rng: np.random.Generator) -> np.ndarray:
    """uint8 image of shape (rows, cols): Gaussian blobs + U[0,16) noise."""
    cx = rng.uniform(0, cols, n_blobs)
    cy = rng.uniform(0, rows, n_blobs)
    sg = rng.uniform(sigma[0], sigma[1], n_blobs)
    am = rng.uniform(amplitude[0], amplitude[1], n_blobs)
    noise = rng.uniform(0.0, 16.0, size=(rows, cols))
    y = np.arange(rows, dtype=np.float64)[:, None]
    x = np.arange(cols, dtype=np.float64)[:, None]
    # separable blobs: image = Gy diag(a) Gx^T, one GEMM instead of n_blobs passes
    gy = np.exp(-((y - cy[None, :]) ** 2) / (2 * sg[None, :] ** 2))
    gx = np.exp(-((x - cx[None, :]) ** 2) / (2 * sg[None, :] ** 2))
    img = (gy * am[None, :]) @ gx.T + noise
    return np.rint(np.clip(img, 0.0, 255.0)).astype(np.uint8)


def _u8(rows, cols, n_blobs, sigma, amplitude, seed):
    return blob_image_u8(rows, cols, n_blobs, sigma, amplitude, np.random.default_rng(seed))


def blob_image(rows: int, cols: int, n_blobs: int, sigma=(8.0, 40.0),
               amplitude=(40.0, 200.0), seed: int = 1) -> np.ndarray:
    """float32 (rows, cols) Fortran-order image in [0, 1], as gray2mat gives."""
    rng = np.random.default_rng(seed)
    u8 = blob_image_u8(rows, cols, n_blobs, sigma, amplitude, rng)
    return np.asfortranarray((u8.astype(np.float64) / 255.0).astype(np.float32))


def workload(name: str):
    """The named workloads as gray2mat floats: [(image, angle_step), ...]
    (the pixels of workload_u8 / 255 in double, stored as float32)."""
    return [(np.asfortranarray((u8.astype(np.float64) / 255.0).astype(np.float32)), step)
            for u8, step in workload_u8(name)]


def write_pgm(name: str, directory: str):
    """Writes the named workload's images as ASCII PGM (P2) files
    <name>_<i>.pgm -- the input format of the reference's demo
    (c++/src/demo.cpp:190-194, readnetpbm) -- and returns their paths with
    the angle steps."""
    import os
    from .api import writepgm
    out = []
    for i, (u8, step) in enumerate(workload_u8(name)):
        path = os.path.join(directory, f"{name}_{i}.pgm")
        writepgm(path, u8.astype(np.int32))
        out.append((path, step))
    return out


def workload_u8(name: str):
    """The named benchmark workloads, as uint8 pixels.

    ``single256``  256x256, 8 blobs (sigma 8-40, amplitude 40-200), seed 1
    ``single1024`` 1024x1024, 32 blobs (sigma 16-160), seed 2
    ``single4096`` 4096x4096, 256 blobs (sigma 32-640), seed 6
    ``batch512``   512 images, sides U{64..512} per axis, 4-16 blobs, step 1
                   or 2 degrees with equal probability; seed 3 (image i uses
                   sub-seed 3000 + i)
    Returns a list of (image, angle_step_degrees) pairs.
    """
    if name == "single256":
        return [(_u8(256, 256, 8, (8, 40), (40, 200), 1), 1.0)]
    if name == "single1024":
        return [(_u8(1024, 1024, 32, (16, 160), (40, 200), 2), 1.0)]
    if name == "single4096":
        return [(_u8(4096, 4096, 256, (32, 640), (40, 200), 6), 0.5)]
    if name == "batch512":
        rng = np.random.default_rng(3)
        rows = rng.integers(64, 513, 512)
        cols = rng.integers(64, 513, 512)
        nb = rng.integers(4, 17, 512)
        steps = np.where(rng.random(512) < 0.5, 1.0, 2.0)
        return [(_u8(int(rows[i]), int(cols[i]), int(nb[i]), (8, 40), (40, 200), 3000 + i),
                 float(steps[i])) for i in range(512)]
    raise ValueError(f"unknown workload {name!r}")
