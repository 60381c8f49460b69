"""Differentiable predict on the GPU gridder.

``predict(image, plan)`` is dirty2ms, linear in the real image x:
V = M A x (A the degridding operator per polarisation, M the image-to-
visibility polarisation matrix).  For a real loss L, PyTorch hands back
G = dL/dRe(V) + i dL/dIm(V), and dL/dx = Re(A^H M^H G), which is exactly
ms2dirty of G on the same plan with the matrix M^H -- so the backward pass
is the gridder itself, and the w-planes are recomputed rather than stored.

``apply_gains(vis, gains, ant1, ant2)`` multiplies each visibility by
g[ant1] conj(g[ant2]) (per-antenna, per-channel complex gains); its
backward uses a hand-written kernel that reduces the gain gradient over
the baseline rows (``gb_gain_gradient`` in the C-ABI).
"""
import numpy
import torch

from . import _lib
from .wgridder import _ptr, _stream


class _Predict(torch.autograd.Function):
    @staticmethod
    def forward(ctx, image, plan, polmat, npol_vis):
        ctx.plan = plan
        ctx.polmat_h = None if polmat is None else numpy.conj(numpy.asarray(polmat)).T.copy()
        return plan.dirty2ms(image.detach().contiguous(), polmat=polmat, npol_vis=npol_vis,
                             layout="yx")

    @staticmethod
    def backward(ctx, grad):
        plan = ctx.plan
        g = grad.detach().to(plan.complex_dtype).contiguous()
        img = plan.ms2dirty(g, polmat=ctx.polmat_h, layout="yx")
        return img, None, None, None


def predict(image, plan, polmat=None, npol_vis=None):
    """Differentiable dirty2ms: image [npol][ny][nx] (plan's real dtype) ->
    visibilities [nrows][nchan][npol_vis]."""
    return _Predict.apply(image, plan, polmat, npol_vis)


def _precision_of(t):
    if t.dtype in (torch.complex128, torch.float64):
        return _lib.GB_FP64
    return _lib.GB_FP32


def _apply_gains_raw(vis, gains, ant1, ant2):
    lib = _lib.load()
    nrows, nchan, npol = vis.shape
    out = torch.empty_like(vis)
    with torch.cuda.device(vis.device):
        _lib.check(lib.gb_apply_gains(_ptr(vis), _ptr(gains), _ptr(ant1), _ptr(ant2), nrows,
                                      nchan, npol, _precision_of(vis), _ptr(out),
                                      _stream(vis.device)), "gb_apply_gains")
    return out


class _ApplyGains(torch.autograd.Function):
    @staticmethod
    def forward(ctx, vis, gains, ant1, ant2):
        vis = vis.detach().contiguous()
        gains = gains.detach().to(torch.complex128).contiguous()
        ctx.save_for_backward(vis, gains, ant1, ant2)
        return _apply_gains_raw(vis, gains, ant1, ant2)

    @staticmethod
    def backward(ctx, grad):
        vis, gains, ant1, ant2 = ctx.saved_tensors
        grad = grad.detach().to(vis.dtype).contiguous()
        grad_vis = None
        if ctx.needs_input_grad[0]:
            grad_vis = _apply_gains_raw(grad, gains.conj().resolve_conj().contiguous(), ant1,
                                        ant2)
        grad_gains = None
        if ctx.needs_input_grad[1]:
            lib = _lib.load()
            nrows, nchan, npol = vis.shape
            nant = gains.shape[0]
            grad_gains = torch.zeros_like(gains)
            with torch.cuda.device(vis.device):
                _lib.check(lib.gb_gain_gradient(_ptr(vis), _ptr(grad), _ptr(gains), _ptr(ant1),
                                                _ptr(ant2), nrows, nchan, npol, nant,
                                                _precision_of(vis), _ptr(grad_gains),
                                                _stream(vis.device)), "gb_gain_gradient")
        return grad_vis, grad_gains, None, None


def apply_gains(vis, gains, ant1, ant2):
    """V' = g[ant1] conj(g[ant2]) V.

    :param vis: [nrows, nchan, npol] complex CUDA tensor
    :param gains: [nant, nchan] complex128 CUDA tensor (may require grad)
    :param ant1, ant2: [nrows] int32 CUDA tensors
    """
    return _ApplyGains.apply(vis, gains, ant1, ant2)


def baseline_antennas(nants, ntimes, device):
    """ant1, ant2 per row for rows ordered [time][baseline], baselines ant1 < ant2."""
    a1, a2 = numpy.triu_indices(nants, k=1)
    a1 = numpy.tile(a1, ntimes).astype(numpy.int32)
    a2 = numpy.tile(a2, ntimes).astype(numpy.int32)
    return torch.from_numpy(a1).to(device), torch.from_numpy(a2).to(device)
