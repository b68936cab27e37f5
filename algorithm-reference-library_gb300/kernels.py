"""ConvolutionFunction and GridData builders and the gridding kernels.

Mirrors ARL's ``processing_components/griddata/kernels.py``,
``griddata/convolution_functions.py`` and ``griddata/operations.py``.  The PSWF
and w-kernel tables are generated in FP64 on the GPU (``arlgpu_make_pswf``,
``arlgpu_make_wkernels``); the WCS bookkeeping is plain Python.
"""
import copy
import ctypes

import numpy
import torch

from . import _native as nat
from . import device as dv
from .data_models import ConvolutionFunction, GridData, Image
from .wcs import WCS

D2R = numpy.pi / 180.0


def create_convolutionfunction_from_image(im, nz=1, zstep=1e15, ztype='WW', oversampling=8, support=16):
    """Empty cf [nchan, npol, nz, O, O, S, S] and its WCS (UU, VV, DUU, DVV, WW,
    STOKES, FREQ) (``convolution_functions.py:62-147``)."""
    assert len(im.shape) == 4
    assert im.wcs.wcs.ctype[0] == 'RA---SIN'
    assert im.wcs.wcs.ctype[1] == 'DEC--SIN'
    w = WCS(7)
    w.wcs.ctype = ['UU', 'VV', 'DUU', 'DVV', ztype, im.wcs.wcs.ctype[2], im.wcs.wcs.ctype[3]]
    w.wcs.crval = [0.0, 0.0, 0.0, 0.0, 0.0, im.wcs.wcs.crval[2], im.wcs.wcs.crval[3]]
    w.wcs.crpix = [float(support // 2) + 1.0, float(support // 2) + 1.0, float(oversampling // 2) + 1.0,
                   float(oversampling // 2) + 1.0, float(nz // 2 + 1), im.wcs.wcs.crpix[2], im.wcs.wcs.crpix[3]]
    cu = 1.0 / (im.shape[3] * D2R * im.wcs.wcs.cdelt[0])
    cv = 1.0 / (im.shape[2] * D2R * im.wcs.wcs.cdelt[1])
    w.wcs.cdelt = [cu, cv, cu / oversampling, cv / oversampling, zstep, im.wcs.wcs.cdelt[2], im.wcs.wcs.cdelt[3]]
    nchan, npol, ny, nx = im.shape
    cf = ConvolutionFunction(numpy.zeros([nchan, npol, nz, oversampling, oversampling, support, support],
                                         dtype='complex'), w, im.wcs.deepcopy(), im.polarisation_frame)
    return cf


def _grid_wcs(im, nw, wstep):
    w = WCS(5)
    w.wcs.crval = [0.0, 0.0, 0.0, im.wcs.wcs.crval[2], im.wcs.wcs.crval[3]]
    w.wcs.crpix = [im.shape[3] // 2 + 1, im.shape[2] // 2 + 1, nw // 2 + 1, im.wcs.wcs.crpix[2],
                   im.wcs.wcs.crpix[3]]
    w.wcs.ctype = ['UU', 'VV', 'WW', im.wcs.wcs.ctype[2], im.wcs.wcs.ctype[3]]
    w.wcs.cdelt = [1.0 / (im.shape[3] * D2R * im.wcs.wcs.cdelt[0]), 1.0 / (im.shape[2] * D2R * im.wcs.wcs.cdelt[1]),
                   wstep, im.wcs.wcs.cdelt[2], im.wcs.wcs.cdelt[3]]
    return w


def create_griddata_from_image(im, nw=1, wstep=1e15):
    """Zero grid [nchan, npol, nw, ny, nx] with WCS UU, VV, WW, STOKES, FREQ
    (``griddata/operations.py:91-145``)."""
    assert len(im.shape) == 4
    nchan, npol, ny, nx = im.shape
    return GridData(numpy.zeros([nchan, npol, nw, ny, nx], dtype='complex'), _grid_wcs(im, nw, wstep),
                    im.wcs.deepcopy(), im.polarisation_frame)


def create_griddata_on_device(im, nw=1, wstep=1e15, precision=None):
    """As create_griddata_from_image, with ``data`` a zeroed CUDA tensor of the precision's dtype."""
    precision = dv.resolve_precision(precision)
    nchan, npol, ny, nx = im.shape
    data = torch.zeros((nchan, npol, nw, ny, nx), dtype=dv.CDTYPE[precision], device=dv.require_cuda())
    return GridData(data, _grid_wcs(im, nw, wstep), im.wcs.deepcopy(), im.polarisation_frame)


def create_box_convolutionfunction(im, oversampling=1, support=1):
    """``kernels.py:19-49``: unit tap at (2, 2) of a 4 x 4 kernel; gcf = 1 / sinc^2."""
    cf = create_convolutionfunction_from_image(im, oversampling=1, support=4)
    cf.data[...] = 0.0
    cf.data[..., 2, 2] = 1.0
    nchan, npol, ny, nx = im.data.shape
    nu = numpy.abs((numpy.arange(nx) - nx // 2) / nx)
    g1 = numpy.sinc(nu)
    gcf = 1.0 / numpy.outer(g1, g1)
    return Image(numpy.broadcast_to(gcf, im.data.shape).copy(), cf.projection_wcs.deepcopy(),
                 im.polarisation_frame), cf


def _pswf_on_device(oversampling, support, n):
    device = dv.require_cuda()
    cf = torch.empty((oversampling, oversampling, support, support), dtype=torch.complex128, device=device)
    gcf = torch.empty((n, n), dtype=torch.float64, device=device) if n else None
    nat.call('arlgpu_make_pswf', oversampling, support, n, n, nat.ptr(cf), nat.ptr(gcf), nat.stream_ptr())
    return cf, gcf


def create_pswf_convolutionfunction(im, oversampling=8, support=6):
    """``kernels.py:52-97``: PSWF anti-aliasing kernel (FP64, generated on the
    GPU) and its grid-correction image."""
    assert isinstance(im, Image), im
    cf = create_convolutionfunction_from_image(im, oversampling=oversampling, support=support)
    nchan, npol, ny, nx = im.data.shape
    assert ny == nx, "ARL's PSWF grid correction needs a square image"
    k, g = _pswf_on_device(oversampling, support, nx)
    k = k.cpu().numpy()
    g = g.cpu().numpy()
    cf.data = numpy.broadcast_to(k[None, None, None], (nchan, npol, 1) + k.shape).astype('complex')
    gcf = Image(numpy.broadcast_to(g, (nchan, npol, ny, nx)).copy(), cf.projection_wcs.deepcopy(),
                im.polarisation_frame)
    return gcf, cf


def create_awterm_convolutionfunction(im, make_pb=None, nw=1, wstep=1e15, oversampling=8, support=6, use_aaf=True,
                                      maxsupport=512, plane_support=None):
    """``kernels.py:100-200`` without a primary beam: the w-kernel stack
    [nchan, npol, nw, O, O, S, S] generated in FP64 on the GPU, the w-screens
    divided by the anti-aliasing function (use_aaf, the default; the returned
    gcf is then the PSWF grid correction) or not (gcf all ones).
    ``plane_support`` (optional, even values <= support) crops plane z to its
    central plane_support[z] taps (see ``set_plane_support``)."""
    if make_pb is not None:
        raise NotImplementedError('primary-beam (A-term) kernels are outside the GB300 path')
    assert isinstance(oversampling, int) and oversampling > 0
    nchan, npol, ony, onx = im.data.shape
    cf = create_convolutionfunction_from_image(im, oversampling=oversampling, support=support)
    cf.grid_wcs.wcs.crpix[4] = nw // 2 + 1.0
    cf.grid_wcs.wcs.cdelt[4] = wstep
    cf.grid_wcs.wcs.ctype[4] = 'WW'
    device = dv.require_cuda()
    t = torch.empty((nw, oversampling, oversampling, support, support), dtype=torch.complex128, device=device)
    nat.call('arlgpu_make_wkernels', nw, float(wstep), oversampling, support, maxsupport, onx,
             float(im.wcs.wcs.cdelt[0]), int(bool(use_aaf)), nat.ptr(t), nat.stream_ptr())
    k = t.cpu().numpy()
    cf.data = numpy.broadcast_to(k[None, None], (nchan, npol) + k.shape).copy()
    if plane_support is not None:
        set_plane_support(cf, plane_support)
    if use_aaf:
        _, g = _pswf_on_device(1, 6, onx)
        gdata = numpy.broadcast_to(g.cpu().numpy(), (nchan, npol, ony, onx)).copy()
    else:
        gdata = numpy.ones((nchan, npol, ony, onx))
    gcf = Image(gdata, cf.projection_wcs.deepcopy(), im.polarisation_frame)
    return gcf, cf


def set_plane_support(cf, supports):
    """Crop each z-plane of ``cf`` to its central supports[z] x supports[z] taps:
    the taps outside are zeroed in ``cf.data`` (so ARL-style code sees the same
    kernel) and the GPU skips them."""
    S = cf.shape[-1]
    supports = numpy.asarray(supports, dtype=numpy.int32)
    assert supports.shape == (cf.shape[2],)
    assert numpy.all(supports % 2 == 0) and numpy.all(supports >= 2) and numpy.all(supports <= S)
    data = numpy.array(cf.data, copy=True)
    for z, sz in enumerate(supports):
        lo = S // 2 - sz // 2
        m = numpy.ones((S, S), dtype=bool)
        m[lo:lo + sz, lo:lo + sz] = False
        data[:, :, z, :, :, m] = 0.0
    cf.data = data
    cf.plane_support = supports


def support_schedule(w_planes, smin, smax):
    """Even support growing linearly with |w| from smin (w = 0) to smax (max |w|)."""
    w = numpy.abs(numpy.asarray(w_planes, dtype=float))
    wmax = w.max() if w.max() > 0 else 1.0
    s = smin + (smax - smin) * w / wmax
    return (2 * numpy.ceil(s / 2)).astype(numpy.int32).clip(smin, smax)


def apply_bounding_box_convolutionfunction(cf, fractional_level=1e-4):
    """``convolution_functions.py:159-184``: crop all planes to a common box."""
    newcf = copy_convolutionfunction(cf)
    nx = newcf.data.shape[-1]
    ny = newcf.data.shape[-2]
    mask = numpy.max(numpy.abs(newcf.data), axis=(0, 1, 2, 3, 4))
    coords = numpy.argwhere(mask > fractional_level * numpy.max(numpy.abs(cf.data)))
    crpx = int(numpy.round(cf.grid_wcs.wcs.crpix[0]))
    crpy = int(numpy.round(cf.grid_wcs.wcs.crpix[1]))
    x0, y0 = coords.min(axis=0)
    dx = crpx - x0
    dy = crpy - y0
    x0 -= 1
    y0 -= 1
    x1 = crpx + dx - 1
    y1 = crpy + dy - 1
    newcf.data = newcf.data[..., y0:y1, x0:x1]
    nny, nnx = newcf.data.shape[-2], newcf.data.shape[-1]
    newcf.grid_wcs.wcs.crpix[0] += nnx / 2 - nx / 2
    newcf.grid_wcs.wcs.crpix[1] += nny / 2 - ny / 2
    return newcf


def calculate_bounding_box_convolutionfunction(cf, fractional_level=1e-4):
    """``convolution_functions.py:187-207``: per-plane (z, (y0, y1), (x0, x1))."""
    bboxes = []
    threshold = fractional_level * numpy.max(numpy.abs(cf.data))
    for z in range(cf.data.shape[2]):
        mask = numpy.max(numpy.abs(cf.data[:, :, z, ...]), axis=(0, 1, 2, 3))
        coords = numpy.argwhere(mask > threshold)
        x0, y0 = coords.min(axis=0)
        x1, y1 = coords.max(axis=0)
        bboxes.append((z, (y0, y1), (x0, x1)))
    return bboxes


def copy_convolutionfunction(cf):
    """``convolution_functions.py:228-244``."""
    fcf = ConvolutionFunction(copy.deepcopy(cf.data), copy.deepcopy(cf.grid_wcs), copy.deepcopy(cf.projection_wcs),
                              cf.polarisation_frame)
    fcf.plane_support = None if cf.plane_support is None else numpy.array(cf.plane_support)
    return fcf


def copy_griddata(gd):
    """``griddata/operations.py:29-51``."""
    return GridData(gd.data.clone() if isinstance(gd.data, torch.Tensor) else copy.deepcopy(gd.data),
                    copy.deepcopy(gd.grid_wcs), copy.deepcopy(gd.projection_wcs), gd.polarisation_frame)
