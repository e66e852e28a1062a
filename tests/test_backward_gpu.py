"""Gradient checks of the hand-written adjoint kernels.

* FP64 finite differences: circus functions (T0, T1, T2 x P1, P3) of 32 x 32
  synthetic blob images over 90 angles, every pixel perturbed by
  h = 1e-6 * max(1, |x|) with central differences, against the float64
  adjoint; a pixel whose perturbation moves a weighted median or flips the
  sign of a P1 difference (the functionals' non-differentiable points) is
  skipped and counted.  Bar: max |fd - grad| <= 1e-6 * max |grad| per
  functional pair.
* Dense PyTorch-op reference gradient: the float32 engine's gradient against
  torch autograd through a float64 tensor-op restatement of the same forward
  (tests/torch_reference.py) with the engine's medians.
"""
import numpy as np
import pytest
import torch

from tracetransform_gb300 import autograd as tta
from tracetransform_gb300.api import angles_from_step, pad_geometry
from tracetransform_gb300.synthetic import blob_image

import torch_reference as tref

pytestmark = pytest.mark.gpu

TF = [0, 1, 2]
PF = [1, 3]


def _blob(rows, cols, seed):
    """(rows, cols) C-ordered blob + noise image in [0, 1]."""
    s = max(rows, cols)
    return np.ascontiguousarray(blob_image(rows, cols, 4 + seed % 5, sigma=(s / 16, s / 4),
                                           seed=seed))


def _image(rows, cols, seed, jitter=1e-3):
    """float64 blob image plus a small continuous jitter that breaks the
    uint8 quantisation's exact ties."""
    rng = np.random.default_rng(seed + 1000)
    return _blob(rows, cols, seed).astype(np.float64) + rng.uniform(0, jitter, (rows, cols))


def _fd_check(rows, cols, step, seed):
    dev = torch.device("cuda", 0)
    angles = angles_from_step(step)
    eng = tta.engine_for(dev)
    img = torch.from_numpy(_image(rows, cols, seed)).to(dev)
    W = torch.from_numpy(np.random.default_rng(seed).standard_normal(
        (len(TF), len(PF), len(angles)))).to(dev)

    # analytic gradients, one per (T, P) pair
    x = img.clone().requires_grad_(True)
    circ = tta.circus(x, angles, TF, PF)
    grads = torch.stack([
        torch.autograd.grad((circ[t, p] * W[t, p]).sum(), x, retain_graph=True)[0]
        for t in range(len(TF)) for p in range(len(PF))]).view(len(TF), len(PF), rows, cols)

    def fwd(im):
        sino, med = eng.sinograms_f64(im.t().contiguous(), rows, cols, angles, TF)
        return sino, med, (eng.circus_f64(sino, [(p, -1, -1) for p in PF]) * W).sum(-1)

    _, med0, _ = fwd(img)
    fd = torch.empty((rows * cols, len(TF), len(PF)), dtype=torch.float64, device=dev)
    skip = torch.zeros(rows * cols, dtype=torch.bool, device=dev)
    flat = img.reshape(-1).cpu()
    for i in range(rows * cols):
        h = 1e-6 * max(1.0, abs(float(flat[i])))
        ip, im_ = img.clone(), img.clone()
        ip.view(-1)[i] += h
        im_.view(-1)[i] -= h
        sp, mp, lp = fwd(ip)
        sm, mm, lm = fwd(im_)
        fd[i] = (lp - lm) / (2 * h)
        flip = (torch.sign(sp[..., 1:] - sp[..., :-1]) != torch.sign(sm[..., 1:] - sm[..., :-1]))
        skip[i] = (mp != med0).any() | (mm != med0).any() | flip.any()
    fd = fd.permute(1, 2, 0).reshape(len(TF), len(PF), rows, cols)
    keep = ~skip.view(rows, cols)
    n_skip = int(skip.sum())
    assert n_skip <= 0.1 * rows * cols, f"{n_skip} of {rows * cols} pixels at kinks"
    worst = 0.0
    for t in range(len(TF)):
        for p in range(len(PF)):
            g, f = grads[t, p][keep], fd[t, p][keep]
            scale = float(g.abs().max())
            err = float((f - g).abs().max()) / scale
            worst = max(worst, err)
            assert err <= 1e-6, f"T{TF[t]} x P{PF[p]}: fd error {err:.3g} of max |grad|"
    return worst, n_skip


@pytest.mark.parametrize("rows,cols,seed", [(32, 32, 1), (32, 24, 2)])
def test_fd_fp64(rows, cols, seed):
    _fd_check(rows, cols, 4, seed)  # 90 angles


@pytest.mark.parametrize("rows,cols,step", [(32, 32, 4), (64, 48, 1), (256, 256, 10)])
def test_reference_gradient_float(rows, cols, step):
    dev = torch.device("cuda", 0)
    angles = angles_from_step(step)
    img = torch.from_numpy(_blob(rows, cols, rows + cols)).to(dev)
    W = torch.from_numpy(np.random.default_rng(7).standard_normal(
        (len(TF), len(PF), len(angles)))).to(dev)

    x = img.clone().requires_grad_(True)
    circ = tta.circus(x, angles, TF, PF)
    (circ.double() * W).sum().backward()
    g_eng = x.grad.double()

    eng = tta.engine_for(dev)
    sino32, med = eng.sinograms(img.t().contiguous(), rows, cols, angles, TF, medians=True)
    xr = img.double().clone().requires_grad_(True)
    sino_ref = tref.sinograms(xr, angles, TF, med)
    circ_ref = tref.circus(sino_ref, PF)
    # the forward agrees before the gradients are compared
    assert float((sino_ref.detach() - sino32.double()).abs().max()) <= \
        1e-5 * float(sino_ref.detach().abs().max())
    (circ_ref * W).sum().backward()
    g_ref = xr.grad
    err = float((g_eng - g_ref).abs().max()) / float(g_ref.abs().max())
    assert err <= 1e-4, f"gradient differs from the dense reference by {err:.3g} of max"


def test_mse_loss_batch():
    """MSE between circus functions and a second seed's targets, over a
    batch; the batched gradient equals the per-image ones."""
    dev = torch.device("cuda", 0)
    angles = angles_from_step(8)
    imgs = torch.stack([torch.from_numpy(_blob(40, 40, s))
                        for s in range(3)]).to(dev)
    tgt_imgs = torch.stack([torch.from_numpy(_blob(40, 40, 100 + s))
                            for s in range(3)]).to(dev)
    with torch.no_grad():
        target = tta.circus(tgt_imgs, angles, TF, PF)
    x = imgs.clone().requires_grad_(True)
    loss = torch.nn.functional.mse_loss(tta.circus(x, angles, TF, PF), target)
    loss.backward()
    assert torch.isfinite(x.grad).all() and float(x.grad.abs().max()) > 0
    for b in range(3):
        xb = imgs[b].clone().requires_grad_(True)
        cb = tta.circus(xb, angles, TF, PF)
        ((cb - target[b]) ** 2).sum().div(target.numel()).backward()
        torch.testing.assert_close(xb.grad, x.grad[b], rtol=1e-5, atol=1e-7 * float(xb.grad.abs().max()))


def test_unsupported_functionals_raise():
    dev = torch.device("cuda", 0)
    img = torch.rand(16, 16, device=dev, dtype=torch.float64)
    with pytest.raises(Exception, match="T0, T1 and T2"):
        tta.circus(img, angles_from_step(30), [3], [1])
    with pytest.raises(Exception, match="P1 and P3"):
        tta.circus(img, angles_from_step(30), [0], [2])


@pytest.mark.parametrize("rows", [7, 363, 1449, 2500, 5793])
def test_p_stage_adjoint_float_matches_f64(rows):
    """The float P-stage adjoint (both DFTs of a column by the chirp-z FFT)
    against the float64 one (direct DFT sums) on the same sinogram columns:
    the sinograms of a smooth blob at the sizes of the 256^2, 1024^2 and
    4096^2 workloads and between them.  Bar: 1e-4 of the largest gradient
    entry, per column kind (P1 only, P3 only, both)."""
    from tracetransform_gb300.device import Engine
    eng = tta.engine_for(torch.device("cuda", 0))
    assert isinstance(eng, Engine)
    rng = np.random.default_rng(rows)
    cols, ns = 12, 2
    t = np.linspace(-1, 1, rows)
    base = np.exp(-(t[None, None, :] / rng.uniform(0.2, 0.5, (ns, cols, 1))) ** 2)
    sino = torch.from_numpy(base * rows * rng.uniform(0.1, 1, (ns, cols, 1)) +
                            rng.uniform(0, 1, (ns, cols, rows))).cuda()
    pf = [(1, -1, -1), (3, -1, -1)]
    g = torch.from_numpy(rng.standard_normal((ns, 2, cols))).cuda()
    g[0, 0, :4] = 0  # P3 only
    g[0, 1, 4:8] = 0  # P1 only
    got = eng.circus_backward(sino.float().contiguous(), pf, g.float().contiguous()).double()
    want = eng.circus_backward(sino.float().double().contiguous(), pf, g.contiguous())
    for sl in (slice(0, 4), slice(4, 8), slice(8, cols)):
        w = want[:, sl]
        err = float((got[:, sl] - w).abs().max()) / float(w.abs().max())
        assert err <= 1e-4, f"rows {rows}: float adjoint off by {err:.3g} of max"
