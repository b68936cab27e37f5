"""Hogbom CLEAN on the GB300 kernels.

Reference behaviour:
  hogbom, overlapIndices    processing_library/arrays/cleaners.py:12-69, :134-154
  deconvolve_cube           processing_components/image/deconvolution.py:43-300 ('hogbom')

The minor cycle runs on the device (``csrc/clean.cu``) in FP64 with the
reference's operation order, so components and residuals equal NumPy's bit
for bit.  Of deconvolve_cube's algorithms only 'hogbom' is on the GPU path;
the others raise NotImplementedError.
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
    if algorithm != 'hogbom':
        raise NotImplementedError("deconvolve_cube algorithm %r is outside the GB300 path (only 'hogbom')"
                                  % algorithm)
    gain = get_parameter(kwargs, 'gain', 0.7)
    assert 0.0 < gain < 2.0, "Loop gain must be between 0 and 2"
    thresh = get_parameter(kwargs, 'threshold', 0.0)
    assert thresh >= 0.0
    niter = get_parameter(kwargs, 'niter', 100)
    assert niter > 0
    fracthresh = get_parameter(kwargs, 'fractional_threshold', 0.1)
    assert 0.0 < fracthresh < 1.0
    pd = psf.data.cpu().numpy() if isinstance(psf.data, torch.Tensor) else numpy.asarray(psf.data)
    comp = numpy.zeros(dd.shape)
    resid = numpy.zeros(dd.shape)
    for ch in range(dd.shape[0]):
        for pol in range(dd.shape[1]):
            if pd[ch, pol].max():
                comp[ch, pol], resid[ch, pol] = hogbom(dd[ch, pol], pd[ch, pol],
                                                       None if window is None else window[ch, pol], gain, thresh,
                                                       niter, fracthresh, prefix)
    return (create_image_from_array(comp, dirty.wcs, dirty.polarisation_frame),
            create_image_from_array(resid, dirty.wcs, dirty.polarisation_frame))
