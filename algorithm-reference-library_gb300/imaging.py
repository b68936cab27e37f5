"""invert_2d / predict_2d, w-stacking and the imaging-context registry on the
GB300 kernels.

Reference behaviour:
  shift_vis_to_image, normalize_sumwt, predict_2d, invert_2d
                                  processing_components/imaging/base.py:50-189
  predict_wstack_single, invert_wstack_single
                                  processing_components/imaging/wstack_single.py:26-96
  vis_null_iter, vis_wslice_iter  processing_components/visibility/iterators.py:23-109
  imaging_contexts, imaging_context
                                  workflows/shared/imaging/imaging_shared.py:21-94
  invert_list_serial_workflow, predict_list_serial_workflow
                                  workflows/serial/imaging/imaging_serial.py:41-216

invert_2d keeps the grid in HBM between the gridder and the FFT: one host->device
copy of the rows in, one device->host copy of the image out.
"""
import numpy
import torch

from . import _native as nat
from . import device as dv
from .data_models import Image, Visibility, copy_visibility, create_empty_image_like, create_visibility_from_rows
from .gridding import DeviceVisibility, _assert_in_grid, _gcf_t, _rows
from .kernels import create_pswf_convolutionfunction, _grid_wcs


def get_parameter(kwargs, key, default=None):
    """``data_models/parameters.py:79-96``."""
    if kwargs is None:
        return default
    value = kwargs.get(key, default)
    return default if value is None else value


def normalize_sumwt(im, sumwt):
    """``imaging/base.py:84-101``: divide each (chan, pol) plane by sumwt, zero if sumwt <= 0."""
    nchan, npol = im.data.shape[:2]
    assert sumwt is not None and sumwt.shape[0] == nchan and sumwt.shape[1] == npol
    for c in range(nchan):
        for p in range(npol):
            if sumwt[c, p] > 0.0:
                im.data[c, p] = im.data[c, p] / sumwt[c, p]
            else:
                im.data[c, p] = 0.0
    return im


def _image_phasecentre_offset(vis, im):
    pc = getattr(vis, 'phasecentre', None)
    if pc is None:
        return None
    ipc = im.phasecentre
    if ipc.separation_rad(pc) > 1e-15:
        return ipc.lmn(pc)
    return None


def shift_vis_to_image(vis, im, tangent=True, inverse=False):
    """``imaging/base.py:50-81``: phase-rotate rows to the image's FFT phase
    centre (a no-op when the phase centres coincide).  Rotation runs on the GPU."""
    lmn = _image_phasecentre_offset(vis, im)
    if lmn is None:
        return vis
    l, m, _ = lmn
    device = dv.require_cuda()
    if isinstance(vis, DeviceVisibility):
        prec = vis.precision
        out = vis.vis.clone()
        nat.call('arlgpu_phaserotate', nat.ptr(out), nat.ptr(vis.uvw), vis.nvis, vis.npol,
                 nat.PRECISIONS[prec], float(l), float(m), int(inverse), nat.stream_ptr())
        return DeviceVisibility(vis.uvw, vis.frequency, out, vis.imaging_weight, vis.polarisation_frame,
                                im.phasecentre)
    newvis = copy_visibility(vis)
    v = dv.to_device(vis.vis, torch.complex128, device)
    uvw = dv.to_device(vis.uvw, torch.float64, device)
    nat.call('arlgpu_phaserotate', nat.ptr(v), nat.ptr(uvw), vis.nvis, vis.npol, nat.FP64, float(l), float(m),
             int(inverse), nat.stream_ptr())
    newvis.data['vis'][...] = v.cpu().numpy()
    newvis.phasecentre = im.phasecentre
    return newvis


def _default_gcfcf(im, kwargs):
    return create_pswf_convolutionfunction(im, support=get_parameter(kwargs, 'support', 6),
                                           oversampling=get_parameter(kwargs, 'oversampling', 128))


def invert_2d(vis, im, dopsf=False, normalize=True, gcfcf=None, precision=None, **kwargs):
    """``imaging/base.py:141-189``: (image, sumwt) or, with imaginary=True,
    (image, sumwt, imaginary image).  Host inputs give host outputs; a
    DeviceVisibility gives images whose data are CUDA tensors."""
    precision = dv.resolve_precision(precision)
    device = dv.require_cuda()
    svis = shift_vis_to_image(vis, im, tangent=True, inverse=False)
    gcf, cf = gcfcf if gcfcf is not None else _default_gcfcf(im, kwargs)
    uvw, f, v, w = _rows(svis, precision, device)
    if dopsf:
        v = torch.ones_like(v)
    nchan, npol, ny, nx = im.shape
    gd = dv.grid_desc(_grid_wcs(im, 1, 1e15), (nchan, npol, 1, ny, nx))
    cf_t, cs, ps, psup = dv.device_cf(cf, precision, device)
    cd = dv.cf_desc(cf.grid_wcs, cf.data.shape, cs, ps, psup)
    grid_t, sumwt, n_bad = dv.grid(uvw, f, v, w, cf_t, cd, gd, precision)
    _assert_in_grid(n_bad)
    imaginary = get_parameter(kwargs, 'imaginary', False)
    # The grid is consumed in place as the FFT buffer (nw == 1).
    re, imag = dv.fft_grid_to_image(grid_t, gd, _gcf_t(gcf, device), precision,
                                    sumwt=sumwt if normalize else None, imaginary=imaginary, buf=grid_t)
    host = not isinstance(vis, DeviceVisibility)
    wcs = im.wcs.deepcopy()
    sw = sumwt.cpu().numpy() if host else sumwt
    if host:
        re = re.cpu().numpy()
        imag = imag.cpu().numpy() if imag is not None else None
    result = Image(re, wcs, im.polarisation_frame)
    if imaginary:
        return result, sw, Image(imag, wcs.deepcopy(), im.polarisation_frame)
    return result, sw


def predict_2d(vis, model, gcfcf=None, precision=None, **kwargs):
    """``imaging/base.py:104-138``: a new Visibility with the model's predicted vis."""
    if model is None:
        return vis
    precision = dv.resolve_precision(precision)
    device = dv.require_cuda()
    gcf, cf = gcfcf if gcfcf is not None else _default_gcfcf(model, kwargs)
    nchan, npol, ny, nx = model.shape
    gd = dv.grid_desc(_grid_wcs(model, 1, 1e15), (nchan, npol, 1, ny, nx))
    d = model.data
    m_t = d.to(device=device, dtype=torch.float64).contiguous() if isinstance(d, torch.Tensor) else \
        dv.to_device(numpy.asarray(d, numpy.float64), torch.float64, device)
    grid_t = dv.fft_image_to_grid(m_t, _gcf_t(gcf, device), gd, precision)
    cf_t, cs, ps, psup = dv.device_cf(cf, precision, device)
    cd = dv.cf_desc(cf.grid_wcs, cf.data.shape, cs, ps, psup)
    uvw, f, _, _ = _rows(vis, precision, device, need_vis=False)
    out, n_bad = dv.degrid(uvw, f, grid_t, cf_t, cd, gd, precision)
    _assert_in_grid(n_bad)
    if isinstance(vis, DeviceVisibility):
        newvis = DeviceVisibility(vis.uvw, vis.frequency, out, vis.imaging_weight, vis.polarisation_frame,
                                  vis.phasecentre)
    else:
        newvis = copy_visibility(vis, zero=True)
        newvis.data['vis'][...] = out.cpu().numpy()
    return shift_vis_to_image(newvis, model, tangent=True, inverse=True)


# ---------------------------------------------------------------------------
# Iterators and contexts
# ---------------------------------------------------------------------------
def vis_null_iter(vis, vis_slices=1):
    """``visibility/iterators.py:23-32``: all rows at once."""
    yield numpy.ones(vis.nvis, dtype=bool)


def vis_wslice_iter(vis, vis_slices=1):
    """``visibility/iterators.py:91-109``: boolean row masks of w-slices."""
    w = vis.w if isinstance(vis, Visibility) else vis.uvw[:, 2].cpu().numpy()
    wmaxabs = numpy.max(numpy.abs(w))
    boxes = numpy.linspace(-wmaxabs, +wmaxabs, vis_slices)
    wstack = boxes[1] - boxes[0] if vis_slices > 1 else 2 * wmaxabs
    for box in boxes:
        yield numpy.abs(w - box) < 0.5 * wstack
