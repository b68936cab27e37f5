"""Differentiable predict / invert and the gain chi^2, on the GB300 kernels.

ARL has no derivatives on this path; the adjoint pairs follow from its
conventions (``processing_components/griddata/gridding.py``):

* predict  V = D F (gcf * I): F the unnormalised centred FFT of
  ``fft_image_to_griddata`` (:292-302), D the degridder (:233-267, no conjugate).
  Its adjoint is gcf * F^H G: G the gridder (:99-133, conjugated taps, unit
  weights) and F^H = nx ny * ifft, the transform of ``fft_griddata_to_image``
  (:270-289).  So the backward pass of predict is invert's gridder + FFT and the
  backward pass of invert is predict's FFT + degridder; taps are re-read from
  the oversampled table, nothing per visibility is stored except the row plan.
* chi^2 = sum w |Vobs - g[a2] conj(g[a1]) M|^2 with the g_i g_j* convention of
  ``apply_gaintable`` (``processing_components/calibration/operations.py:134-137``);
  its Wirtinger derivatives come from ``arlgpu_gain_chi2``.

Gradients follow torch's complex convention (2 * dL/d conj(z)).
"""
import ctypes

import numpy
import torch

from . import _native as nat
from . import device as dv
from .gridding import DeviceVisibility, _gcf_t, _rows
from .kernels import _grid_wcs


class GriddingOperator:
    """The rows, convolution function and image geometry of a predict / invert
    pair, with the row plan (FP64 mapping + tile binning) built once."""

    def __init__(self, vis, im, gcfcf, precision=None):
        self.precision = dv.resolve_precision(precision)
        device = dv.require_cuda()
        self.device = device
        gcf, cf = gcfcf
        self.uvw, self.f, v, w = _rows(vis, self.precision, device)
        self.weight = w
        nchan, npol, ny, nx = im.shape
        self.shape = (nchan, npol, ny, nx)
        self.npol = npol
        self.gd = dv.grid_desc(_grid_wcs(im, 1, 1e15), (nchan, npol, 1, ny, nx))
        self.cf_t, cs, ps, psup = dv.device_cf(cf, self.precision, device)
        self._psup = psup
        self.cd = dv.cf_desc(cf.grid_wcs, cf.data.shape, cs, ps, psup, table=self.cf_t)
        self.gcf = _gcf_t(gcf, device)
        self.n = self.uvw.shape[0]
        self.ws = torch.empty(dv.plan_bytes(self.n, self.gd, self.cd), dtype=torch.uint8, device=device)
        n_bad = torch.zeros(1, dtype=torch.int64, device=device)
        nat.call('arlgpu_plan_build', nat.ptr(self.uvw), nat.ptr(self.f), self.n, ctypes.byref(self.gd),
                 ctypes.byref(self.cd), nat.ptr(self.ws), self.ws.numel(), nat.ptr(n_bad), nat.stream_ptr())
        nb = int(n_bad.item())
        assert nb == 0, "%d visibilities fall outside the grid or convolution function" % nb
        self.ones = torch.ones((self.n, npol), dtype=dv.RDTYPE[self.precision], device=device)
        self.sumwt = None

    # -- building blocks --------------------------------------------------
    def _grid(self, v, w):
        g = torch.empty((self.shape[0], self.shape[1], 1, self.shape[2], self.shape[3]),
                        dtype=dv.CDTYPE[self.precision], device=self.device)
        sw = torch.empty((self.shape[0], self.shape[1]), dtype=torch.float64, device=self.device)
        v = v.contiguous()
        w = w.contiguous()
        nat.call('arlgpu_grid_planned', nat.ptr(v), nat.ptr(w), self.n,
                 nat.PRECISIONS[self.precision], nat.ptr(self.cf_t), ctypes.byref(self.cd), nat.ptr(g),
                 ctypes.byref(self.gd), nat.ptr(sw), nat.ptr(self.ws), self.ws.numel(), nat.stream_ptr())
        return g, sw

    def _degrid(self, g):
        out = torch.empty((self.n, self.npol), dtype=dv.CDTYPE[self.precision], device=self.device)
        nat.call('arlgpu_degrid_planned', self.n, nat.PRECISIONS[self.precision], nat.ptr(self.cf_t),
                 ctypes.byref(self.cd), nat.ptr(g), ctypes.byref(self.gd), nat.ptr(out), nat.ptr(self.ws),
                 self.ws.numel(), nat.stream_ptr())
        return out

    def _image_to_grid(self, image):
        return dv.fft_image_to_grid(image.to(torch.float64).contiguous(), self.gcf, self.gd, self.precision)

    def _grid_to_image(self, g, sumwt=None):
        re, _ = dv.fft_grid_to_image(g, self.gd, self.gcf, self.precision, sumwt=sumwt, buf=g)
        return re

    # -- operators ----------------------------------------------------------
    def predict(self, image):
        """V = degrid(F(gcf * image)) (ARL predict_2d with coincident phase centres)."""
        return self._degrid(self._image_to_grid(image))

    def predict_adjoint(self, grad_v):
        """gcf * Re(F^H grid(grad_v)), the vector-Jacobian product of predict."""
        g, _ = self._grid(grad_v.to(dv.CDTYPE[self.precision]), self.ones)
        return self._grid_to_image(g)

    def invert(self, vis):
        """Re(F^H grid(vis * weight)) * gcf / sumwt (ARL invert_2d, normalize=True)."""
        g, sw = self._grid(vis.to(dv.CDTYPE[self.precision]), self.weight)
        self.sumwt = sw
        return self._grid_to_image(g, sw)

    def invert_adjoint(self, grad_image):
        """weight * degrid(F(gcf * grad_image / sumwt)), the vector-Jacobian product of invert."""
        if self.sumwt is None:
            _, self.sumwt = self._grid(torch.zeros((self.n, self.npol), dtype=dv.CDTYPE[self.precision],
                                                   device=self.device), self.weight)
        sw = self.sumwt
        scale = torch.where(sw > 0, 1.0 / sw.clamp_min(1e-300), torch.zeros_like(sw))[:, :, None, None]
        v = self._degrid(self._image_to_grid(grad_image * scale))
        return v * self.weight


class Predict(torch.autograd.Function):
    """image [nchan, npol, ny, nx] (float64) -> visibilities [nvis, npol]."""

    @staticmethod
    def forward(ctx, image, op):
        ctx.op = op
        return op.predict(image)

    @staticmethod
    def backward(ctx, grad_v):
        return ctx.op.predict_adjoint(grad_v), None


class Invert(torch.autograd.Function):
    """visibilities [nvis, npol] -> normalised dirty image [nchan, npol, ny, nx]."""

    @staticmethod
    def forward(ctx, vis, op):
        ctx.op = op
        return op.invert(vis)

    @staticmethod
    def backward(ctx, grad_image):
        return ctx.op.invert_adjoint(grad_image.to(torch.float64)).to(dv.CDTYPE[ctx.op.precision]), None


class GainChi2(torch.autograd.Function):
    """chi^2 = sum w |Vobs - g[a2] conj(g[a1]) M|^2 -> scalar float64; gradients
    to the model visibilities M and the complex gains g."""

    @staticmethod
    def forward(ctx, model, gains, vobs, a1, a2, weight):
        prec = 'fp64' if model.dtype == torch.complex128 else 'fp32c'
        dev = model.device
        chi2 = torch.zeros(1, dtype=torch.float64, device=dev)
        grad_m = torch.empty_like(model) if ctx.needs_input_grad[0] else None
        grad_g = torch.empty(gains.shape, dtype=torch.complex128, device=dev) if ctx.needs_input_grad[1] else None
        g = gains.detach().to(torch.complex128).contiguous()
        vo = vobs.to(model.dtype).contiguous()
        mo = model.contiguous()
        nat.call('arlgpu_gain_chi2', nat.ptr(vo), nat.ptr(mo),
                 nat.ptr(weight), model.shape[0], model.shape[1], nat.PRECISIONS[prec], nat.ptr(a1), nat.ptr(a2),
                 nat.ptr(g), g.shape[0], nat.ptr(chi2), nat.ptr(grad_m), nat.ptr(grad_g), nat.stream_ptr())
        ctx.save_for_backward(*(t for t in (grad_m, grad_g) if t is not None))
        ctx.has = (grad_m is not None, grad_g is not None)
        return chi2[0]

    @staticmethod
    def backward(ctx, gout):
        saved = list(ctx.saved_tensors)
        gm = 2.0 * gout * saved.pop(0) if ctx.has[0] else None
        gg = (2.0 * gout * saved.pop(0)) if ctx.has[1] else None
        return gm, gg, None, None, None, None


def chi2(image, gains, vobs, op, a1, a2, weight=None):
    """chi^2 of predict(image) corrupted by per-antenna gains against vobs;
    differentiable in image (float64 tensor) and gains (complex128 tensor)."""
    m = Predict.apply(image, op)
    return GainChi2.apply(m, gains, vobs, a1, a2, weight)


def gain_chi2_step(image, gains, vobs, op, a1, a2, weight=None):
    """One gradient step's worth of work: chi^2 and its gradients with respect
    to the image and the gains (each a fresh tensor)."""
    x = image.detach().requires_grad_(True)
    g = gains.detach().requires_grad_(True)
    c = chi2(x, g, vobs, op, a1, a2, weight)
    c.backward()
    return c.detach(), x.grad, g.grad
