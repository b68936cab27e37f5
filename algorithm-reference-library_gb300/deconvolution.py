"""Hogbom and multiscale CLEAN on the GB300 kernels.

Reference behaviour:
  hogbom, overlapIndices    processing_library/arrays/cleaners.py:12-69, :134-154
  hogbom_complex            processing_library/arrays/cleaners.py:72-131
  msmfsclean and helpers    processing_library/arrays/cleaners.py:469-760
  image frequency moments   processing_components/image/operations.py:239-330
  msclean and its helpers   processing_library/arrays/cleaners.py:165-440
  deconvolve_cube           processing_components/image/deconvolution.py:43-300 ('hogbom', 'msclean')

Everything runs on the device.  The Hogbom minor cycle (``csrc/clean.cu``)
is FP64 in the reference's operation order, so components and residuals
equal NumPy's bit for bit.  The multiscale set-up (scale images, their
convolutions with the dirty image and the PSF as complex128 cuFFT transforms,
the coupling matrix, the window stack) is ``csrc/msclean_setup.cu``; it
rounds differently from NumPy's FFTs, so msclean agrees with the reference to
a stated FP64 tolerance rather than bit for bit.  The complex Hogbom of
Q + iU (``cleaners.py:72-131``, deconvolve_cube 'hogbom-complex') runs the
same way on two residual planes.  The multi-scale multi-frequency CLEAN
('msmfsclean', 'mfsmsclean', 'mmclean') cleans the frequency moments of the
cube: its set-up (scale stacks, the scale-moment residuals and the
scale-scale-moment-moment PSF by complex128 cuFFT convolutions, the
moment-moment Hessians and their inverses) and minor cycle run on the device,
within a stated FP64 tolerance of the reference.  Unknown algorithms raise
ValueError, as in the reference.
"""
import ctypes

import numpy
import torch

from . import _native as nat
from . import device as dv
from .data_models import Image, PolarisationFrame, create_image_from_array
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


def hogbom_complex(dirty_q, dirty_u, psf_q, psf_u, window, gain, thresh, niter, fracthresh):
    """``cleaners.py:72-131``: complex Hogbom CLEAN of Q + iU with the (common)
    PSF; returns (Q components, U components, Q residual, U residual).  Inputs
    are arrays or CUDA tensors; the minor cycle runs on the device
    (``arlgpu_hogbom_complex``)."""
    assert 0.0 < gain < 2.0
    assert niter > 0
    device = dv.require_cuda()
    dq, du = _plane(dirty_q, device), _plane(dirty_u, device)
    pq, pu = _plane(psf_q, device), _plane(psf_u, device)
    assert bool(torch.equal(pq, pu))
    w = None if window is None else _plane(window, device)
    nx, ny = dq.shape
    pmax = float(pq.max().item())
    assert pmax > 0.0
    dmax = float(torch.hypot(dq, du).max().item())
    cq, cu, rq, ru = (torch.empty_like(dq) for _ in range(4))
    iters = ctypes.c_int32(0)
    nat.call('arlgpu_hogbom_complex', nat.ptr(dq), nat.ptr(du), nat.ptr(pq), nat.ptr(w), nx, ny, pq.shape[0],
             pq.shape[1], float(gain), float(thresh), int(niter), float(fracthresh), dmax, pmax, nat.ptr(cq),
             nat.ptr(cu), nat.ptr(rq), nat.ptr(ru), ctypes.byref(iters), nat.stream_ptr())
    if isinstance(dirty_q, torch.Tensor):
        return cq, cu, rq, ru
    return cq.cpu().numpy(), cu.cpu().numpy(), rq.cpu().numpy(), ru.cpu().numpy()


def msclean(dirty, psf, window, gain, thresh, niter, scales, fracthresh, prefix=''):
    """``cleaners.py:165-280``: (component array, residual array).  The set-up
    (``arlgpu_msclean_setup``) and the minor cycle (``arlgpu_msclean``) run on
    the device; dirty / psf / window are arrays or CUDA tensors."""
    assert 0.0 < gain < 2.0
    assert niter > 0
    assert len(scales) > 0
    device = dv.require_cuda()
    d = _plane(dirty, device)
    p = _plane(psf, device)
    w = None if window is None else _plane(window, device)
    ns = len(scales)
    nx, ny = d.shape
    pnx, pny = p.shape
    sc = (ctypes.c_double * ns)(*[float(x) for x in scales])
    nb = ctypes.c_size_t(0)
    nat.call('arlgpu_msclean_setup_bytes', nx, ny, pnx, pny, ns, ctypes.byref(nb))
    ws = dv.WORKSPACE.get(nb.value, device)
    f64 = dict(dtype=torch.float64, device=device)
    stack = torch.empty((ns, nx, ny), **f64)
    pss = torch.empty((ns, ns, pnx, pny), **f64)
    pscale = torch.empty((ns, pnx, pny), **f64)
    wstack = None if w is None else torch.empty((ns, nx, ny), **f64)
    coupling = torch.empty((ns, ns), **f64)
    scalars = torch.empty(2, **f64)
    nat.call('arlgpu_msclean_setup', nat.ptr(d), nx, ny, nat.ptr(p), pnx, pny, nat.ptr(w), sc, ns, nat.ptr(stack),
             nat.ptr(pss), nat.ptr(pscale), nat.ptr(wstack), nat.ptr(coupling), nat.ptr(scalars), nat.ptr(ws),
             ws.numel(), nat.stream_ptr())
    pmax, res0max = (float(x) for x in scalars.cpu())
    assert pmax > 0.0
    if wstack is not None:
        assert float(wstack.sum().item()) > 0
    absolutethresh = max(thresh, fracthresh * res0max)
    comps = torch.empty((nx, ny), **f64)
    iters = ctypes.c_int32(0)
    nat.call('arlgpu_msclean', nat.ptr(stack), nat.ptr(pss), nat.ptr(pscale), nat.ptr(wstack), nat.ptr(coupling), ns,
             nx, ny, pnx, pny, float(gain), float(absolutethresh), int(niter), nat.ptr(comps), ctypes.byref(iters),
             nat.stream_ptr())
    res = stack[0] * pmax
    if isinstance(dirty, torch.Tensor):
        return comps, res
    return comps.cpu().numpy(), res.cpu().numpy()


def _band(n, lo, hi):
    """Boolean mask of the indices lo <= i < hi of an axis of length n."""
    i = numpy.arange(n)
    return (i >= lo) & (i < hi)


def clean_window(shape, window_shape, edge=16):
    """The CLEAN window of each (channel, polarisation) plane, as
    ``deconvolution.py:82-100`` defines them: 'quarter' keeps rows and columns
    q + 1 .. 3 q - 1 with q a quarter of the axis, 'no_edge' drops the first
    edge + 1 and the last edge of each axis, None cleans everywhere (returns
    None).  Other names raise ValueError."""
    if window_shape is None:
        return None
    ny, nx = shape[-2], shape[-1]
    if window_shape == 'quarter':
        rows, cols = _band(ny, ny // 4 + 1, 3 * (ny // 4)), _band(nx, nx // 4 + 1, 3 * (nx // 4))
    elif window_shape == 'no_edge':
        rows, cols = _band(ny, edge + 1, ny - edge), _band(nx, edge + 1, nx - edge)
    else:
        raise ValueError("Window shape %s is not recognized" % window_shape)
    return numpy.broadcast_to(numpy.outer(rows, cols).astype(numpy.float64), tuple(shape)).copy()


def crop_psf_to_support(psf, support):
    """Keep the 2 support x 2 support pixels around the PSF's centre pixel
    (``deconvolution.py:108-113``), in place, when both axes are at least that
    large."""
    ny, nx = psf.data.shape[2], psf.data.shape[3]
    if support <= ny // 2 and support <= nx // 2:
        y0, x0 = ny // 2 - support, nx // 2 - support
        psf.data = psf.data[..., y0:y0 + 2 * support, x0:x0 + 2 * support]


# ---------------------------------------------------------------------------
# Multi-scale multi-frequency CLEAN (cleaners.py:469-760) and the frequency
# moments it works on (processing_components/image/operations.py:239-330)
# ---------------------------------------------------------------------------
_FINDPEAK = {'ARL': 0, 'Algorithm1': 1, 'CASA': 2}


def _channel_frequencies(im):
    return numpy.asarray(im.wcs.sub([4]).wcs_pix2world(numpy.arange(im.data.shape[0]), 0)[0], dtype=numpy.float64)


def _moment_weights(freq, nmoment, reference_frequency):
    return [[float(numpy.power((f - reference_frequency) / reference_frequency, m)) for f in freq]
            for m in range(nmoment)]


def calculate_image_frequency_moments(im, reference_frequency=None, nmoment=1):
    """``image/operations.py:239-282``: moment m of the cube is the sum over
    channels of plane * ((f - f0) / f0)^m, f0 the mean channel frequency by
    default; the frequency axis becomes a MOMENT axis.  Summed on the device in
    channel order."""
    assert isinstance(im, Image)
    assert nmoment > 0
    nchan = im.data.shape[0]
    assert nmoment <= nchan, "Number of moments %d cannot exceed the number of channels %d" % (nmoment, nchan)
    freq = _channel_frequencies(im)
    f0 = float(numpy.average(freq)) if reference_frequency is None else reference_frequency
    device = dv.require_cuda()
    cube = _plane(im.data, device)
    out = torch.zeros((nmoment,) + tuple(cube.shape[1:]), dtype=torch.float64, device=device)
    for m, ws in enumerate(_moment_weights(freq, nmoment, f0)):
        for c, w in enumerate(ws):
            out[m] = out[m] + cube[c] * w
    wcs = im.wcs.deepcopy()
    wcs.wcs.ctype[3] = 'MOMENT'
    wcs.wcs.crval[3] = 0.0
    wcs.wcs.crpix[3] = 1.0
    wcs.wcs.cdelt[3] = 1.0
    data = out if isinstance(im.data, torch.Tensor) else out.cpu().numpy()
    return create_image_from_array(data, wcs, im.polarisation_frame)


def calculate_image_from_frequency_moments(im, moment_image, reference_frequency=None):
    """``image/operations.py:285-330``: channel c of the new cube is the sum
    over moments of moment_m * ((f_c - f0) / f0)^m, on im's channels."""
    assert isinstance(im, Image)
    nchan, npol, ny, nx = im.data.shape
    nmoment, mnpol, mny, mnx = moment_image.data.shape
    assert nmoment > 0 and npol == mnpol and ny == mny and nx == mnx
    assert moment_image.wcs.wcs.ctype[3] == 'MOMENT', "Second image should be a moment image"
    freq = _channel_frequencies(im)
    f0 = float(numpy.average(freq)) if reference_frequency is None else reference_frequency
    device = dv.require_cuda()
    mom = _plane(moment_image.data, device)
    out = torch.zeros((nchan, npol, ny, nx), dtype=torch.float64, device=device)
    for m, ws in enumerate(_moment_weights(freq, nmoment, f0)):
        for c, w in enumerate(ws):
            out[c] = out[c] + mom[m] * w
    data = out if isinstance(im.data, torch.Tensor) else out.cpu().numpy()
    return create_image_from_array(data, im.wcs, im.polarisation_frame)


def _scale_stack(scales, n0, n1, device):
    out = torch.empty((len(scales), n0, n1), dtype=torch.float64, device=device)
    sc = (ctypes.c_double * len(scales))(*[float(x) for x in scales])
    nat.call('arlgpu_scale_stack', sc, len(scales), n0, n1, nat.ptr(out), nat.stream_ptr())
    return out


def _scale_convolve(imgs, stack, twice=False, thresh=-1.0):
    """imgs [k, n0, n1] convolved with every plane of stack (convolve_scalestack)
    -> [k, ns, n0, n1], or twice (convolve_convolve_scalestack) -> [k, ns, ns,
    n0, n1]; thresh >= 0 turns the once-convolved result into 1 above it, 0
    elsewhere."""
    k, n0, n1 = imgs.shape
    ns = stack.shape[0]
    nb = ctypes.c_size_t(0)
    nat.call('arlgpu_scale_convolve_bytes', n0, n1, ns, ctypes.byref(nb))
    ws = dv.WORKSPACE.get(nb.value, imgs.device)
    shape = (k, ns, ns, n0, n1) if twice else (k, ns, n0, n1)
    out = torch.empty(shape, dtype=torch.float64, device=imgs.device)
    nat.call('arlgpu_scale_convolve', nat.ptr(imgs.contiguous()), k, n0, n1, nat.ptr(stack), ns, int(twice),
             float(thresh), nat.ptr(out), nat.ptr(ws), ws.numel(), nat.stream_ptr())
    return out


def msmfsclean(dirty, psf, window, gain, thresh, niter, scales, fracthresh, findpeak='ARL', prefix=''):
    """``cleaners.py:469-600``: multi-scale multi-frequency CLEAN of the moment
    images dirty [nmoment, n0, n1] with the PSF moments [2 nmoment (or 1),
    p0, p1]; returns (model moments, residual moments).  The set-up (scale
    stacks, scale-moment residuals, scale-scale-moment-moment PSF, Hessians,
    window stack) and the minor cycle (``arlgpu_msmfsclean``) run on the
    device."""
    assert 0.0 < gain < 2.0
    assert niter > 0
    assert len(scales) > 0
    assert findpeak in _FINDPEAK, findpeak
    device = dv.require_cuda()
    d = _plane(dirty, device)
    p = _plane(psf, device)
    nmoment, n0, n1 = d.shape
    pn, p0, p1 = p.shape
    ns = len(scales)
    pmax = float(p.max().item())
    assert pmax > 0.0
    if nmoment > 1:
        assert pn == 2 * nmoment
    lpsf, ldirty = p / pmax, d / pmax
    scalestack = _scale_stack(scales, n0, n1, device)
    pscalestack = _scale_stack(scales, p0, p1, device)
    smres = _scale_convolve(ldirty, scalestack).transpose(0, 1).contiguous()  # [ns, nmoment, n0, n1]
    nm = max(pn // 2, 1)
    cc = _scale_convolve(lpsf[:2 * nm - 1], pscalestack, twice=True)  # [t + q][s][p]
    ssm = torch.empty((ns, ns, nm, nm, p0, p1), dtype=torch.float64, device=device)
    for t in range(nm):
        for q in range(nm):
            ssm[:, :, t, q] = cc[t + q]
    hess = torch.stack([ssm[s, s, :, :, p0 // 2, p1 // 2] for s in range(ns)]).contiguous()
    ihess = torch.linalg.inv(hess).contiguous()
    wstack = None
    if window is not None:
        wstack = _scale_convolve(_plane(window, device)[None], scalestack, thresh=0.9)[0].contiguous()
    absolutethresh = max(thresh, fracthresh * float(smres[0, 0].abs().max().item()))
    model = torch.empty((nmoment, n0, n1), dtype=torch.float64, device=device)
    iters = ctypes.c_int32(0)
    nat.call('arlgpu_msmfsclean', nat.ptr(smres), nat.ptr(ssm), nat.ptr(pscalestack), nat.ptr(wstack), nat.ptr(hess),
             nat.ptr(ihess), ns, nmoment, n0, n1, p0, p1, float(gain), float(absolutethresh), int(niter),
             _FINDPEAK[findpeak], nat.ptr(model), ctypes.byref(iters), nat.stream_ptr())
    res = smres[0] * pmax
    if isinstance(dirty, torch.Tensor):
        return model, res
    return model.cpu().numpy(), res.cpu().numpy()


def _deconvolve_cube_msmfs(dirty, psf, window, kwargs):
    """``deconvolution.py:156-210`` ('msmfsclean', 'mfsmsclean', 'mmclean'):
    moment images of the cube (nmoment, default 3; the PSF with 2 nmoment),
    both divided by the PSF moments' peak, one msmfsclean per polarisation,
    then the component and residual moments back to cubes on the dirty
    image's channels unless return_moments."""
    findpeak = get_parameter(kwargs, 'findpeak', 'ARL')
    nmoment = get_parameter(kwargs, 'nmoment', 3)
    assert nmoment >= 1, "Number of frequency moments must be greater than or equal to one"
    nchan = dirty.data.shape[0]
    assert nchan > 2 * (nmoment - 1), "Require nchan %d > 2 * (nmoment %d - 1)" % (nchan, 2 * (nmoment - 1))
    dirty_taylor = calculate_image_frequency_moments(dirty, nmoment=nmoment)
    psf_taylor = calculate_image_frequency_moments(psf, nmoment=2 * nmoment if nmoment > 1 else 1)
    dt, pt = _plane(dirty_taylor.data, dv.require_cuda()), _plane(psf_taylor.data, dv.require_cuda())
    psf_peak = float(pt.max().item())
    dt, pt = dt / psf_peak, pt / psf_peak
    gain = get_parameter(kwargs, 'gain', 0.7)
    assert 0.0 < gain < 2.0, "Loop gain must be between 0 and 2"
    thresh = get_parameter(kwargs, 'threshold', 0.0)
    assert thresh >= 0.0
    niter = get_parameter(kwargs, 'niter', 100)
    assert niter > 0
    scales = get_parameter(kwargs, 'scales', [0, 3, 10, 30])
    fracthresh = get_parameter(kwargs, 'fractional_threshold', 0.1)
    assert 0.0 < fracthresh < 1.0
    comp = torch.zeros_like(dt)
    resid = torch.zeros_like(dt)
    for pol in range(dt.shape[1]):
        if float(pt[0, pol].max().item()):
            w = None if window is None else window[0, pol]
            comp[:, pol], resid[:, pol] = msmfsclean(dt[:, pol], pt[:, pol], w, gain, thresh, niter, scales,
                                                     fracthresh, findpeak)
    host = not isinstance(dirty.data, torch.Tensor)
    comp_image = create_image_from_array(comp.cpu().numpy() if host else comp, dirty_taylor.wcs,
                                         dirty.polarisation_frame)
    resid_image = create_image_from_array(resid.cpu().numpy() if host else resid, dirty_taylor.wcs,
                                          dirty.polarisation_frame)
    if not get_parameter(kwargs, 'return_moments', False):
        comp_image = calculate_image_from_frequency_moments(dirty, comp_image)
        resid_image = calculate_image_from_frequency_moments(dirty, resid_image)
    return comp_image, resid_image


def _deconvolve_cube_complex(dd, psf, window, kwargs, wcs):
    """``deconvolution.py:244-292``: per channel, polarisations 0 and 3 by
    Hogbom, 1 and 2 together as Q + iU by complex Hogbom (with polarisation 1's
    window); components and residuals in the stokesIQUV frame."""
    gain = get_parameter(kwargs, 'gain', 0.7)
    assert 0.0 < gain < 2.0, "Loop gain must be between 0 and 2"
    thresh = get_parameter(kwargs, 'threshold', 0.0)
    assert thresh >= 0.0
    niter = get_parameter(kwargs, 'niter', 100)
    assert niter > 0
    fracthresh = get_parameter(kwargs, 'fractional_threshold', 0.1)
    assert 0.0 <= fracthresh < 1.0
    pd = psf.data.cpu().numpy() if isinstance(psf.data, torch.Tensor) else numpy.asarray(psf.data)
    comp = numpy.zeros(dd.shape)
    resid = numpy.zeros(dd.shape)
    for ch in range(dd.shape[0]):
        for pol in (0, 3):
            if pol < dd.shape[1] and pd[ch, pol].max():
                w = None if window is None else window[ch, pol]
                comp[ch, pol], resid[ch, pol] = hogbom(dd[ch, pol], pd[ch, pol], w, gain, thresh, niter, fracthresh)
        if dd.shape[1] > 2 and pd[ch, 1:2].max():
            w = None if window is None else window[ch, 1]
            comp[ch, 1], comp[ch, 2], resid[ch, 1], resid[ch, 2] = hogbom_complex(
                dd[ch, 1], dd[ch, 2], pd[ch, 1], pd[ch, 2], w, gain, thresh, niter, fracthresh)
    frame = PolarisationFrame('stokesIQUV')
    return create_image_from_array(comp, wcs, frame), create_image_from_array(resid, wcs, frame)


def deconvolve_cube(dirty, psf, prefix='', **kwargs):
    """``deconvolution.py:43-300`` with algorithm='hogbom': window shapes
    'quarter' / 'no_edge' / None or a mask Image, PSF cropped to psf_support,
    one CLEAN per (channel, polarisation).  Returns (component Image,
    residual Image).  ``psf.data`` is cropped in place, as in the reference."""
    assert isinstance(dirty, Image), dirty
    assert isinstance(psf, Image), psf
    dd = dirty.data.cpu().numpy() if isinstance(dirty.data, torch.Tensor) else numpy.asarray(dirty.data)
    window = clean_window(dd.shape, get_parameter(kwargs, 'window_shape', None),
                          get_parameter(kwargs, 'window_edge', 16))
    mask = get_parameter(kwargs, 'mask', None)
    if isinstance(mask, Image):
        window = numpy.asarray(mask.data)
    crop_psf_to_support(psf, get_parameter(kwargs, 'psf_support', max(dd.shape[2] // 2, dd.shape[3] // 2)))
    algorithm = get_parameter(kwargs, 'algorithm', 'msclean')
    if algorithm == 'hogbom-complex':
        return _deconvolve_cube_complex(dd, psf, window, kwargs, dirty.wcs)
    if algorithm in ('msmfsclean', 'mfsmsclean', 'mmclean'):
        return _deconvolve_cube_msmfs(dirty, psf, window, kwargs)
    if algorithm not in ('hogbom', 'msclean'):
        raise ValueError('deconvolve_cube %s: Unknown algorithm %s' % (prefix, algorithm))
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
