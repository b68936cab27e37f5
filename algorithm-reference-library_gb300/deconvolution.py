"""Hogbom and multiscale CLEAN on the GB300 kernels.

Reference behaviour:
  hogbom, overlapIndices    processing_library/arrays/cleaners.py:12-69, :134-154
  msclean and its helpers   processing_library/arrays/cleaners.py:165-440
  deconvolve_cube           processing_components/image/deconvolution.py:43-300 ('hogbom', 'msclean')

The minor cycles run on the device (``csrc/clean.cu``) in FP64 with the
reference's operation order, so components and residuals equal NumPy's bit
for bit.  The multiscale set-up (scale images, their FFT convolutions with
the dirty image and the PSF, the coupling matrix) is NumPy on the host, as
the reference computes it, so the device loop starts from identical values.
deconvolve_cube's other algorithms raise NotImplementedError.
"""
import ctypes

import numpy
import torch

from . import _native as nat
from . import device as dv
from .data_models import Image, create_image_from_array
from .imaging import get_parameter


def _plane(a, device):
    if isinstance(a, torch.Tensor):
        return a.to(device=device, dtype=torch.float64).contiguous()
    return dv.to_device(numpy.asarray(a, dtype=numpy.float64), torch.float64, device)


def hogbom_device(dirty, psf, window, gain, thresh, niter, fracthresh):
    """One plane on the device; dirty / psf / window are CUDA tensors or arrays.
    Returns (components, residual, iterations) with device tensors."""
    assert 0.0 < gain < 2.0
    assert niter > 0
    device = dv.require_cuda()
    d = _plane(dirty, device)
    p = _plane(psf, device)
    w = None if window is None else _plane(window, device)
    nx, ny = d.shape
    comps = torch.empty_like(d)
    res = torch.empty_like(d)
    dmax = float(d.abs().max().item())
    pmax = float(p.max().item())
    assert pmax > 0.0
    iters = ctypes.c_int32(0)
    nat.call('arlgpu_hogbom', nat.ptr(d), nat.ptr(p), nat.ptr(w), nx, ny, p.shape[0], p.shape[1], float(gain),
             float(thresh), int(niter), float(fracthresh), dmax, pmax, nat.ptr(comps), nat.ptr(res),
             ctypes.byref(iters), nat.stream_ptr())
    return comps, res, iters.value


def hogbom(dirty, psf, window, gain, thresh, niter, fracthresh, prefix=''):
    """``cleaners.py:12-69``: (component array, residual array)."""
    comps, res, _ = hogbom_device(dirty, psf, window, gain, thresh, niter, fracthresh)
    if isinstance(dirty, torch.Tensor):
        return comps, res
    return comps.cpu().numpy(), res.cpu().numpy()


# Schwab's rational approximation (m = 6, alpha = 1) as msclean evaluates it
# (``cleaners.py:398-440``), one scalar at a time.
_SPH_P = ((8.203343e-2, -3.644705e-1, 6.278660e-1, -5.335581e-1, 2.312756e-1),
          (4.028559e-3, -3.697768e-2, 1.021332e-1, -1.201436e-1, 6.412774e-2))
_SPH_Q = ((1.0000000, 8.212018e-1, 2.078043e-1), (1.0000000, 9.599102e-1, 2.918724e-1))


def _spheroidal(vnu):
    if 0.0 <= vnu < 0.75:
        part, nuend = 0, 0.75
    elif 0.75 <= vnu <= 1.0:
        part, nuend = 1, 1.0
    else:
        return 0.0
    top = _SPH_P[part][0]
    bot = _SPH_Q[part][0]
    d = vnu ** 2 - nuend ** 2
    for k in range(1, 5):
        top += _SPH_P[part][k] * d ** k
    for k in range(1, 3):
        bot += _SPH_Q[part][k] * d ** k
    value = top / bot if bot != 0.0 else 0.0
    return value if value >= 0.0 else 0.0


def create_scalestack(scaleshape, scales, norm=True):
    """``cleaners.py:283-316``: [nscales, nx, ny] stack of the scale basis images."""
    assert scaleshape[0] == len(scales)
    basis = numpy.zeros(scaleshape)
    nx, ny = scaleshape[1], scaleshape[2]
    xcen = int(numpy.ceil(float(nx) / 2.0))
    ycen = int(numpy.ceil(float(ny) / 2.0))
    for iscale in numpy.arange(0, len(scales)):
        halfscale = int(numpy.ceil(scales[iscale] / 2.0))
        if scales[iscale] > 0.0:
            rscale2 = 1.0 / (float(scales[iscale]) / 2.0) ** 2
            for y in range(ycen - halfscale - 1, ycen + halfscale + 1):
                for x in range(xcen - halfscale - 1, xcen + halfscale + 1):
                    fx = float(x - xcen)
                    fy = float(y - ycen)
                    r2 = rscale2 * (fx * fx + fy * fy)
                    r = numpy.sqrt(r2)
                    basis[iscale, x, y] = _spheroidal(r) * (1.0 - r ** 2)
            basis[basis < 0.0] = 0.0
            if norm:
                basis[iscale, :, :] /= numpy.sum(basis[iscale, :, :])
        else:
            basis[iscale, xcen, ycen] = 1.0
    return basis


def _fft2c(a):
    return numpy.fft.fftshift(numpy.fft.fft2(numpy.fft.fftshift(a)))


def convolve_scalestack(scalestack, img):
    """``cleaners.py:319-335``."""
    convolved = numpy.zeros(scalestack.shape)
    ximg = _fft2c(img)
    for iscale in range(scalestack.shape[0]):
        xmult = ximg * numpy.conjugate(_fft2c(scalestack[iscale, :, :]))
        convolved[iscale, :, :] = numpy.real(numpy.fft.ifftshift(numpy.fft.ifft2(numpy.fft.ifftshift(xmult))))
    return convolved


def convolve_convolve_scalestack(scalestack, img):
    """``cleaners.py:338-360``: [nscales, nscales, nx, ny]."""
    nscales, nx, ny = scalestack.shape
    convolved = numpy.zeros([nscales, nscales, nx, ny])
    ximg = _fft2c(img)
    xscale = numpy.zeros([nscales, nx, ny], dtype='complex')
    for s in range(nscales):
        xscale[s] = _fft2c(scalestack[s, ...])
    for s in range(nscales):
        for p in range(nscales):
            xmult = ximg * xscale[p] * numpy.conjugate(xscale[s])
            convolved[s, p, ...] = numpy.real(numpy.fft.ifftshift(numpy.fft.ifft2(numpy.fft.ifftshift(xmult))))
    return convolved


def msclean(dirty, psf, window, gain, thresh, niter, scales, fracthresh, prefix=''):
    """``cleaners.py:165-280``: (component array, residual array); the set-up on
    the host as the reference forms it, the minor cycle on the device."""
    assert 0.0 < gain < 2.0
    assert niter > 0
    assert len(scales) > 0
    device = dv.require_cuda()
    dirty = numpy.asarray(dirty, dtype=numpy.float64)
    psf = numpy.asarray(psf, dtype=numpy.float64)
    pmax = psf.max()
    assert pmax > 0.0
    lpsf = psf / pmax
    ldirty = dirty / pmax
    scalestack = create_scalestack([len(scales), ldirty.shape[0], ldirty.shape[1]], scales, norm=True)
    pscalestack = create_scalestack([len(scales), lpsf.shape[0], lpsf.shape[1]], scales, norm=True)
    res_scalestack = convolve_scalestack(scalestack, numpy.array(ldirty))
    psf_scalescalestack = convolve_convolve_scalestack(pscalestack, numpy.array(lpsf))
    ns = len(scales)
    coupling = numpy.zeros([ns, ns])
    for i in range(ns):
        for j in range(ns):
            coupling[i, j] = numpy.max(psf_scalescalestack[i, j, :, :])
    if window is None:
        windowstack = None
    else:
        windowstack = numpy.zeros_like(scalestack)
        windowstack[convolve_scalestack(scalestack, window) > 0.9] = 1.0
        assert numpy.sum(windowstack) > 0
    absolutethresh = max(thresh, fracthresh * numpy.fabs(res_scalestack[0, :, :]).max())
    stack_t = torch.as_tensor(res_scalestack).to(device)
    pss_t = torch.as_tensor(psf_scalescalestack).to(device)
    ps_t = torch.as_tensor(pscalestack).to(device)
    ws_t = None if windowstack is None else torch.as_tensor(windowstack).to(device)
    cm_t = torch.as_tensor(coupling).to(device)
    comps = torch.empty(dirty.shape, dtype=torch.float64, device=device)
    iters = ctypes.c_int32(0)
    nat.call('arlgpu_msclean', nat.ptr(stack_t), nat.ptr(pss_t), nat.ptr(ps_t), nat.ptr(ws_t), nat.ptr(cm_t), ns,
             dirty.shape[0], dirty.shape[1], psf.shape[0], psf.shape[1], float(gain), float(absolutethresh),
             int(niter), nat.ptr(comps), ctypes.byref(iters), nat.stream_ptr())
    return comps.cpu().numpy(), pmax * stack_t[0].cpu().numpy()


def deconvolve_cube(dirty, psf, prefix='', **kwargs):
    """``deconvolution.py:43-300`` with algorithm='hogbom': window shapes
    'quarter' / 'no_edge' / None or a mask Image, PSF cropped to psf_support,
    one CLEAN per (channel, polarisation).  Returns (component Image,
    residual Image).  ``psf.data`` is cropped in place, as in the reference."""
    assert isinstance(dirty, Image), dirty
    assert isinstance(psf, Image), psf
    dd = dirty.data.cpu().numpy() if isinstance(dirty.data, torch.Tensor) else numpy.asarray(dirty.data)
    window_shape = get_parameter(kwargs, 'window_shape', None)
    ny, nx = dd.shape[2], dd.shape[3]
    if window_shape == 'quarter':
        qx, qy = nx // 4, ny // 4
        window = numpy.zeros_like(dd)
        window[..., (qy + 1):3 * qy, (qx + 1):3 * qx] = 1.0
    elif window_shape == 'no_edge':
        edge = get_parameter(kwargs, 'window_edge', 16)
        window = numpy.zeros_like(dd)
        window[..., (edge + 1):(ny - edge), (edge + 1):(nx - edge)] = 1.0
    elif window_shape is None:
        window = None
    else:
        raise ValueError("Window shape %s is not recognized" % window_shape)
    mask = get_parameter(kwargs, 'mask', None)
    if isinstance(mask, Image):
        window = numpy.asarray(mask.data)
    psf_support = get_parameter(kwargs, 'psf_support', max(dd.shape[2] // 2, dd.shape[3] // 2))
    if psf_support <= psf.data.shape[2] // 2 and psf_support <= psf.data.shape[3] // 2:
        c = [psf.data.shape[2] // 2, psf.data.shape[3] // 2]
        psf.data = psf.data[..., (c[0] - psf_support):(c[0] + psf_support), (c[1] - psf_support):(c[1] + psf_support)]
    algorithm = get_parameter(kwargs, 'algorithm', 'msclean')
    if algorithm not in ('hogbom', 'msclean'):
        raise NotImplementedError("deconvolve_cube algorithm %r is outside the GB300 path ('hogbom', 'msclean')"
                                  % algorithm)
    gain = get_parameter(kwargs, 'gain', 0.7)
    assert 0.0 < gain < 2.0, "Loop gain must be between 0 and 2"
    thresh = get_parameter(kwargs, 'threshold', 0.0)
    assert thresh >= 0.0
    niter = get_parameter(kwargs, 'niter', 100)
    assert niter > 0
    if algorithm == 'msclean':
        scales = get_parameter(kwargs, 'scales', [0, 3, 10, 30])
        fracthresh = get_parameter(kwargs, 'fractional_threshold', 0.01)
    else:
        fracthresh = get_parameter(kwargs, 'fractional_threshold', 0.1)
    assert 0.0 < fracthresh < 1.0
    pd = psf.data.cpu().numpy() if isinstance(psf.data, torch.Tensor) else numpy.asarray(psf.data)
    comp = numpy.zeros(dd.shape)
    resid = numpy.zeros(dd.shape)
    for ch in range(dd.shape[0]):
        for pol in range(dd.shape[1]):
            if pd[ch, pol].max():
                w = None if window is None else window[ch, pol]
                if algorithm == 'msclean':
                    comp[ch, pol], resid[ch, pol] = msclean(dd[ch, pol], pd[ch, pol], w, gain, thresh, niter,
                                                            scales, fracthresh, prefix)
                else:
                    comp[ch, pol], resid[ch, pol] = hogbom(dd[ch, pol], pd[ch, pol], w, gain, thresh, niter,
                                                           fracthresh, prefix)
    return (create_image_from_array(comp, dirty.wcs, dirty.polarisation_frame),
            create_image_from_array(resid, dirty.wcs, dirty.polarisation_frame))
