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
import ctypes

import numpy
import torch

from . import _native as nat
from . import device as dv
from .data_models import Image, Visibility, copy_visibility, create_empty_image_like, create_visibility_from_rows
from .gridding import DeviceVisibility, _assert_in_grid, _gcf_t, _rows
from .kernels import create_pswf_convolutionfunction, _grid_wcs
from .wstack import WStackImager, invert_to_host, slice_axis as _slice_axis


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


def _reproject_uvw(uvw, old, new):
    """uvw [..., 3] on the tangent plane of ``old`` re-expressed on that of
    ``new``: ``uvw_to_xyz`` with (ha, dec) = (-ra, dec) of ``old``, then
    ``xyz_to_uvw`` with those of ``new`` (``util/coordinate_support.py:59-113``),
    each product and sum rounded on its own as there.  On the device."""
    c0, s0 = float(numpy.cos(-old.ra_rad)), float(numpy.sin(-old.ra_rad))
    cd0, sd0 = float(numpy.cos(old.dec_rad)), float(numpy.sin(old.dec_rad))
    c1, s1 = float(numpy.cos(-new.ra_rad)), float(numpy.sin(-new.ra_rad))
    cd1, sd1 = float(numpy.cos(new.dec_rad)), float(numpy.sin(new.dec_rad))
    u, v, w = uvw[..., 0], uvw[..., 1], uvw[..., 2]
    v0 = v * sd0 - w * cd0
    z = v * cd0 + w * sd0
    x = u * c0 + v0 * s0
    y = -u * s0 + v0 * c0
    v0 = x * s1 + y * c1
    return torch.stack([x * c1 - y * s1, z * cd1 + v0 * sd1, z * sd1 - v0 * cd1], dim=-1)


def phaserotate_visibility(vis, newphasecentre, tangent=True, inverse=False):
    """``visibility/base.py:295-381``: a copy of ``vis`` whose rows are
    multiplied by conj(exp(-2 pi i (u l + v m + w (n - 1)))) (by the phasor
    itself with ``inverse``), (l, m, n - 1) the direction cosines of
    ``newphasecentre`` relative to ``vis.phasecentre``; ``vis`` itself when
    |n - 1| < 1e-15.  With ``tangent=False`` the uvw are then re-projected onto
    the new phase centre's tangent plane and the copy takes that phase centre.
    Visibility, DeviceVisibility or BlockVisibility (per channel uvw = metres x
    f / c).  Runs on the GPU in FP64."""
    l, m, n1 = newphasecentre.lmn(vis.phasecentre)
    if numpy.abs(n1) < 1e-15:
        return vis
    device = dv.require_cuda()
    if isinstance(vis, DeviceVisibility):
        out = vis.vis.clone()
        nat.call('arlgpu_phaserotate', nat.ptr(out), nat.ptr(vis.uvw), vis.nvis, vis.npol,
                 nat.PRECISIONS[vis.precision], float(l), float(m), int(inverse), nat.stream_ptr())
        if tangent:
            return DeviceVisibility(vis.uvw, vis.frequency, out, vis.imaging_weight, vis.polarisation_frame,
                                    vis.phasecentre)
        return DeviceVisibility(_reproject_uvw(vis.uvw, vis.phasecentre, newphasecentre).contiguous(),
                                vis.frequency, out, vis.imaging_weight, vis.polarisation_frame, newphasecentre)
    if isinstance(vis, Visibility):
        newvis = copy_visibility(vis)
        v = dv.to_device(vis.vis, torch.complex128, device)
        uvw = dv.to_device(vis.uvw, torch.float64, device)
        nat.call('arlgpu_phaserotate', nat.ptr(v), nat.ptr(uvw), vis.nvis, vis.npol, nat.FP64, float(l), float(m),
                 int(inverse), nat.stream_ptr())
        newvis.data['vis'][...] = v.cpu().numpy()
        if not tangent:
            newvis.data['uvw'][...] = _reproject_uvw(uvw, vis.phasecentre, newphasecentre).cpu().numpy()
            newvis.phasecentre = newphasecentre
        return newvis
    from .data_models import BlockVisibility, copy_blockvisibility
    from .skycomponents import C_M_S
    assert isinstance(vis, BlockVisibility), 'vis argument neither Visibility or BlockVisibility'
    newvis = copy_blockvisibility(vis)
    ntimes, nant, _, nchan, npol = vis.vis.shape
    k = torch.as_tensor(vis.frequency / C_M_S, device=device)
    buvw = dv.to_device(vis.uvw, torch.float64, device)                      # [t, i, j, 3], metres
    uvw = (buvw[..., None, :] * k[:, None]).reshape(-1, 3).contiguous()     # [t, i, j, c, 3], wavelengths
    v = dv.to_device(vis.vis, torch.complex128, device).reshape(-1, npol).contiguous()
    nat.call('arlgpu_phaserotate', nat.ptr(v), nat.ptr(uvw), uvw.shape[0], npol, nat.FP64, float(l), float(m),
             int(inverse), nat.stream_ptr())
    newvis.data['vis'][...] = v.cpu().numpy().reshape(vis.vis.shape)
    if not tangent:
        newvis.data['uvw'][...] = _reproject_uvw(buvw, vis.phasecentre, newphasecentre).cpu().numpy()
        newvis.phasecentre = newphasecentre
    return newvis


def shift_vis_to_image(vis, im, tangent=True, inverse=False):
    """``imaging/base.py:50-81``: phase-rotate rows to the image's FFT phase
    centre (a no-op when the phase centres coincide).  Rotation runs on the GPU."""
    pc = getattr(vis, 'phasecentre', None)
    if pc is None or im.phasecentre.separation_rad(pc) <= 1e-15:
        return vis
    newvis = phaserotate_visibility(vis, im.phasecentre, tangent=tangent, inverse=inverse)
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
    cd = dv.cf_desc(cf.grid_wcs, cf.data.shape, cs, ps, psup, table=cf_t)
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
    cd = dv.cf_desc(cf.grid_wcs, cf.data.shape, cs, ps, psup, table=cf_t)
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


# ---------------------------------------------------------------------------
# W-stacking
# ---------------------------------------------------------------------------
def invert_wstack(vis, im, vis_slices, dopsf=False, normalize=True, gcfcf=None, precision=None, **kwargs):
    """W-stack invert over all slices at once: equals ``invert_list_serial_workflow``
    with context 'wstack' (imaging_serial.py:186-197): sum_s sumwt_s * invert_wstack_single_s,
    normalised by sum_s sumwt_s.  One gridder launch, batched FFTs, one combine."""
    imager = WStackImager(vis, im, vis_slices, gcfcf=gcfcf, precision=precision)
    image, sumwt = invert_to_host(imager, vis, dopsf, normalize)
    return Image(image, im.wcs.deepcopy(), im.polarisation_frame), sumwt


def predict_wstack(vis, model, vis_slices, gcfcf=None, precision=None, **kwargs):
    """W-stack predict over all slices at once: equals ``predict_list_serial_workflow``
    with context 'wstack' (each slice's rows get predict_wstack_single's values)."""
    imager = WStackImager(vis, model, vis_slices, gcfcf=gcfcf, precision=precision)
    out = imager.predict(model.data)
    if isinstance(vis, DeviceVisibility):
        return DeviceVisibility(vis.uvw, vis.frequency, out.clone(), vis.imaging_weight, vis.polarisation_frame,
                                vis.phasecentre)
    newvis = copy_visibility(vis, zero=True)
    newvis.data['vis'][...] = out.cpu().numpy()
    return newvis


def _wstack_fftbuf(gd, grid_t, precision, device):
    """FP64 transform scratch of the w-stack invert: the grid itself on the FP64
    path, else a buffer of the size the library asks for (one group of planes)."""
    if precision == 'fp64':
        return grid_t
    nbytes = ctypes.c_size_t(0)
    nat.call('arlgpu_wstack_fftbuf_bytes', ctypes.byref(gd), ctypes.byref(nbytes))
    return torch.empty(nbytes.value // 16, dtype=torch.complex128, device=device)


def invert_wstack_single(vis, im, dopsf, normalize=True, remove=True, gcfcf=None, precision=None, **kwargs):
    """``wstack_single.py:67-96``: (Re(wb * I), sumwt) for one slice, wb the
    w-beam of the slice's mean w and I the complex invert_2d image."""
    return _single_slice_invert(vis, im, dopsf, normalize, gcfcf, precision)


def _single_slice(vis, im, gcfcf, precision, device):
    gcf, cf = gcfcf if gcfcf is not None else create_pswf_convolutionfunction(im)
    if cf.shape[2] != 1:
        raise NotImplementedError('w-stacking with w-projection kernels is outside the GB300 path')
    uvw, f, v, w = _rows(vis, precision, device)
    nchan, npol, ny, nx = im.shape
    gd = dv.grid_desc(_grid_wcs(im, 1, 1e15), (nchan, npol, 1, ny, nx))
    cf_t, cs, ps, psup = dv.device_cf(cf, precision, device)
    cd = dv.cf_desc(cf.grid_wcs, cf.data.shape, cs, ps, psup, table=cf_t)
    ws = dv.WORKSPACE.get(dv.plan_bytes(uvw.shape[0], gd, cd), device)
    n_bad = torch.zeros(1, dtype=torch.int64, device=device)
    nat.call('arlgpu_plan_build', nat.ptr(uvw), nat.ptr(f), uvw.shape[0], ctypes.byref(gd), ctypes.byref(cd),
             nat.ptr(ws), ws.numel(), nat.ptr(n_bad), nat.stream_ptr())
    _assert_in_grid(n_bad)
    wmean = torch.empty(1, dtype=torch.float64, device=device)
    nat.call('arlgpu_plan_plane_mean_w', nat.ptr(uvw), uvw.shape[0], ctypes.byref(gd), ctypes.byref(cd),
             nat.ptr(ws), ws.numel(), nat.ptr(wmean), nat.stream_ptr())
    cellsize = abs(float(im.wcs.wcs.cdelt[0])) * numpy.pi / 180.0
    return dict(gcf=gcf, cf=cf, uvw=uvw, f=f, v=v, w=w, gd=gd, cd=cd, cf_t=cf_t, ws=ws, wmean=wmean,
                cellsize=cellsize)


def _single_slice_invert(vis, im, dopsf, normalize, gcfcf, precision):
    precision = dv.resolve_precision(precision)
    device = dv.require_cuda()
    s = _single_slice(vis, im, gcfcf, precision, device)
    gd, cd = s['gd'], s['cd']
    nchan, npol, ny, nx = im.shape
    v = torch.ones_like(s['v']) if dopsf else s['v']
    grid_t = torch.empty((nchan, npol, 1, ny, nx), dtype=dv.CDTYPE[precision], device=device)
    sumwt = torch.empty((nchan, npol), dtype=torch.float64, device=device)
    nat.call('arlgpu_grid_planned', nat.ptr(v), nat.ptr(s['w']), s['uvw'].shape[0], nat.PRECISIONS[precision],
             nat.ptr(s['cf_t']), ctypes.byref(cd), nat.ptr(grid_t), ctypes.byref(gd), nat.ptr(sumwt),
             nat.ptr(s['ws']), s['ws'].numel(), nat.stream_ptr())
    image = torch.empty((nchan, npol, ny, nx), dtype=torch.float64, device=device)
    norm = sumwt if normalize else torch.ones_like(sumwt)
    fftbuf = _wstack_fftbuf(gd, grid_t, precision, device)
    gcf_d = _gcf_t(s['gcf'], device)
    nat.call('arlgpu_wstack_grid_to_image', nat.ptr(grid_t), ctypes.byref(gd), nat.PRECISIONS[precision],
             nat.ptr(gcf_d), nat.ptr(s['wmean']), s['cellsize'], nat.ptr(norm), nat.ptr(image),
             nat.ptr(fftbuf), nat.stream_ptr())
    host = not isinstance(vis, DeviceVisibility)
    out = Image(image.cpu().numpy() if host else image, im.wcs.deepcopy(), im.polarisation_frame)
    return out, (sumwt.cpu().numpy() if host else sumwt)


def predict_wstack_single(vis, model, remove=True, gcfcf=None, precision=None, **kwargs):
    """``wstack_single.py:26-64``: V = predict_2d(conj(w-beam of the mean w) * model).
    As in ARL the input's vis column is zeroed."""
    precision = dv.resolve_precision(precision)
    device = dv.require_cuda()
    if isinstance(vis, Visibility):
        vis.data['vis'][...] = 0.0
    s = _single_slice(vis, model, gcfcf, precision, device)
    gd, cd = s['gd'], s['cd']
    nchan, npol, ny, nx = model.shape
    d = model.data
    m_t = d.to(device=device, dtype=torch.float64).contiguous() if isinstance(d, torch.Tensor) else \
        dv.to_device(numpy.asarray(d, numpy.float64), torch.float64, device)
    grid_t = torch.empty((nchan, npol, 1, ny, nx), dtype=dv.CDTYPE[precision], device=device)
    gcf_d = _gcf_t(s['gcf'], device)
    nat.call('arlgpu_wstack_image_to_grid', nat.ptr(m_t), nat.ptr(gcf_d), nat.ptr(s['wmean']),
             s['cellsize'], ctypes.byref(gd), nat.PRECISIONS[precision], nat.ptr(grid_t), nat.stream_ptr())
    out = torch.empty((s['uvw'].shape[0], npol), dtype=dv.CDTYPE[precision], device=device)
    nat.call('arlgpu_degrid_planned', s['uvw'].shape[0], nat.PRECISIONS[precision], nat.ptr(s['cf_t']),
             ctypes.byref(cd), nat.ptr(grid_t), ctypes.byref(gd), nat.ptr(out), nat.ptr(s['ws']), s['ws'].numel(),
             nat.stream_ptr())
    if isinstance(vis, DeviceVisibility):
        return DeviceVisibility(vis.uvw, vis.frequency, out, vis.imaging_weight, vis.polarisation_frame,
                                vis.phasecentre)
    newvis = copy_visibility(vis, zero=True)
    newvis.data['vis'][...] = out.cpu().numpy()
    return newvis


# ---------------------------------------------------------------------------
# Contexts and serial workflows
# ---------------------------------------------------------------------------
def imaging_contexts():
    """``workflows/shared/imaging/imaging_shared.py:21-88``, restricted to the
    contexts on the GB300 path."""
    return {'2d': {'predict': predict_2d, 'invert': invert_2d, 'vis_iterator': vis_null_iter},
            'wprojection': {'predict': predict_2d, 'invert': invert_2d, 'vis_iterator': vis_null_iter},
            'wstack': {'predict': predict_wstack_single, 'invert': invert_wstack_single,
                       'vis_iterator': vis_wslice_iter}}


def imaging_context(context='2d'):
    contexts = imaging_contexts()
    assert context in contexts.keys(), context
    return contexts[context]


def invert_list_serial_workflow(vis_list, template_model_imagelist, dopsf=False, normalize=True, facets=1,
                                vis_slices=1, context='2d', gcfcf=None, precision=None, **kwargs):
    """``imaging_serial.py:125-216`` for facets == 1: one (image, sumwt) per vis.
    The 'wstack' context runs all slices in one batched pass."""
    if facets != 1:
        raise NotImplementedError('facets are outside the GB300 path')
    if not isinstance(template_model_imagelist, (list, tuple)):
        template_model_imagelist = [template_model_imagelist]
    imaging_context(context)
    if gcfcf is None:
        gcfcf = [create_pswf_convolutionfunction(template_model_imagelist[0])]
    out = []
    for i, vis in enumerate(vis_list):
        g = gcfcf[i] if len(gcfcf) > 1 else gcfcf[0]
        im = template_model_imagelist[i]
        if context == 'wstack' and normalize:
            out.append(invert_wstack(vis, im, vis_slices, dopsf=dopsf, normalize=True, gcfcf=g,
                                     precision=precision))
        elif context == 'wstack':
            out.append(_invert_wstack_slices_unnormalised(vis, im, vis_slices, dopsf, g, precision))
        else:
            out.append(invert_2d(vis, im, dopsf=dopsf, normalize=normalize, gcfcf=g, precision=precision))
    return out


def _invert_wstack_slices_unnormalised(vis, im, vis_slices, dopsf, gcfcf, precision):
    """The serial w-stack workflow with normalize=False (``imaging_serial.py:186-197``):
    each slice's rows are inverted without normalisation
    (``invert_wstack_single``), the slice image is weighted by the slice's own
    sumwt, and the sum is divided by the total sumwt.  Slices without rows
    contribute nothing, as ``create_visibility_from_rows`` returns None for
    them.  One GPU invert per slice; the weighted sum stays on the device
    (FP64) and comes back once."""
    if not isinstance(vis, Visibility):
        raise NotImplementedError('the unnormalised w-stack workflow takes a host Visibility')
    device = dv.require_cuda()
    nchan, npol = im.shape[:2]
    acc = torch.zeros(im.shape, dtype=torch.float64, device=device)
    total = torch.zeros((nchan, npol), dtype=torch.float64, device=device)
    for rows in vis_wslice_iter(vis, vis_slices):
        row_vis = create_visibility_from_rows(vis, rows)
        if row_vis is None:
            continue
        dvis = DeviceVisibility.from_visibility(row_vis, precision, device)
        img, sw = invert_wstack_single(dvis, im, dopsf, normalize=False, gcfcf=gcfcf, precision=precision)
        acc += sw[:, :, None, None] * img.data
        total += sw
    acc = torch.where(total[:, :, None, None] > 0, acc / torch.where(total > 0, total, 1.0)[:, :, None, None],
                      torch.zeros_like(acc))
    return Image(acc.cpu().numpy(), im.wcs.deepcopy(), im.polarisation_frame), total.cpu().numpy()


def predict_list_serial_workflow(vis_list, model_imagelist, context, vis_slices=1, facets=1, gcfcf=None,
                                 precision=None, **kwargs):
    """``imaging_serial.py:41-122`` for facets == 1: predicted copies of each vis."""
    if facets != 1:
        raise NotImplementedError('facets are outside the GB300 path')
    imaging_context(context)
    if gcfcf is None:
        gcfcf = [create_pswf_convolutionfunction(m) for m in model_imagelist]
    out = []
    for i, vis in enumerate(vis_list):
        g = gcfcf[i] if len(gcfcf) > 1 else gcfcf[0]
        if context == 'wstack':
            out.append(predict_wstack(vis, model_imagelist[i], vis_slices, gcfcf=g, precision=precision))
        else:
            out.append(predict_2d(vis, model_imagelist[i], gcfcf=g, precision=precision))
    return out
