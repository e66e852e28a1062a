"""Dense PyTorch-op restatement of the differentiable forward path.

T0/T1/T2 sinograms and P1/P3 circus functions of one image, written with
plain tensor ops (gather, sums, torch.fft.rfft) in float64 so that torch's own
autograd gives a reference gradient for the engine's hand-written adjoint
kernels.  The rotation follows the engine's float coordinate arithmetic
(c++/src/auxiliary.cpp:182-255: q = (X c + Y s) + o in float32, bilinear
weights from the float fractional parts), the weighted medians are taken from
the engine's forward pass and held fixed (c++/src/functionals.cpp:95-129), and
P1/P3 follow c++/src/functionals.cpp:287-360 (P3: |F_m(p) / N|^4 with the
mirrored index, integrated by trapz over linspace(-1, 1, N)).

Test infrastructure only: the engine never calls this.
"""
from __future__ import annotations

import numpy as np
import torch

from tracetransform_gb300.api import pad_geometry


def line_samples(img: torch.Tensor, angles_deg, n: int, ro: int, co: int) -> torch.Tensor:
    """(A, N columns, N samples) rotated-frame samples of a (rows, cols) image
    placed at (ro, co) in the N x N frame; differentiable in img."""
    rows, cols = img.shape
    dev = img.device
    ang = np.asarray(angles_deg, np.float32)
    rad = (ang.astype(np.float64) * np.pi / 180).astype(np.float32)
    c = torch.from_numpy(np.cos(-rad).astype(np.float32)).to(dev)
    s = torch.from_numpy(np.sin(-rad).astype(np.float32)).to(dev)
    o = torch.tensor((n - 1) * 0.5, dtype=torch.float32, device=dev)
    grid = torch.arange(n, dtype=torch.float32, device=dev) - o
    X = grid.view(1, n, 1)  # column index of the rotated frame
    Y = grid.view(1, 1, n)  # sample (row) index along the column
    cc, ss = c.view(-1, 1, 1), s.view(-1, 1, 1)
    qx = ((X * cc) + (Y * ss)) + o
    qy = ((X * (-ss)) + (Y * cc)) + o
    valid = (qx >= 0) & (qx < n - 1) & (qy >= 0) & (qy < n - 1)
    xi, yi = torch.trunc(qx), torch.trunc(qy)
    xf, yf = (qx - xi).double(), (qy - yi).double()
    x0 = xi.long() - co
    y0 = yi.long() - ro
    flat = img.reshape(-1)
    out = torch.zeros(qx.shape, dtype=img.dtype, device=dev)
    for dx, dy, w in ((0, 0, (1 - xf) * (1 - yf)), (1, 0, xf * (1 - yf)),
                      (0, 1, (1 - xf) * yf), (1, 1, xf * yf)):
        xx, yy = x0 + dx, y0 + dy
        ok = valid & (xx >= 0) & (xx < cols) & (yy >= 0) & (yy < rows)
        idx = torch.where(ok, yy * cols + xx, torch.zeros_like(xx))
        out = out + torch.where(ok, flat[idx] * w, torch.zeros_like(w))
    return out


def sinograms(img: torch.Tensor, angles_deg, tfuncs, medians: torch.Tensor) -> torch.Tensor:
    """(nT, A, N) T0/T1/T2 sinograms; medians (nT, A, N) from the engine."""
    rows, cols = img.shape
    n, ro, co = pad_geometry(rows, cols)
    x = line_samples(img, angles_deg, n, ro, co)  # (A, N, N)
    j = torch.arange(n, device=img.device, dtype=torch.float64).view(1, 1, n)
    out = []
    for t, f in enumerate(tfuncs):
        if f == 0:
            out.append(x.sum(-1))
            continue
        m = medians[t].to(torch.float64).unsqueeze(-1)
        r = torch.clamp(j - m, min=0)
        out.append((x * (r if f == 1 else r * r)).sum(-1))
    return torch.stack(out)


def circus(sino: torch.Tensor, pfuncs) -> torch.Tensor:
    """(nS, A, N) sinograms -> (nS, nP, A) P1/P3 circus functions."""
    n = sino.shape[-1]
    out = []
    for p in pfuncs:
        if p == 1:
            out.append((sino[..., 1:] - sino[..., :-1]).abs().sum(-1))
        elif p == 3:
            F = torch.fft.rfft(sino, dim=-1)
            h = (F.real / n) ** 2 + (F.imag / n) ** 2
            y_half = h * h
            mirror = [k if k <= n // 2 else n - k for k in range(n)]
            y = y_half[..., mirror]
            lin = torch.from_numpy(
                (-1 + np.arange(n) * 2.0 / (n - 1)).astype(np.float32).astype(np.float64)
            ).to(sino.device)
            out.append((0.5 * (lin[1:] - lin[:-1]) * (y[..., 1:] + y[..., :-1])).sum(-1))
        else:
            raise ValueError(f"no reference for P{p}")
    return torch.stack(out, dim=1)
