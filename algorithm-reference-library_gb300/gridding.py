"""Gridding, degridding and the FFT stages: ARL's ``griddata/gridding.py`` API
on the GB300 kernels.

Every function keeps the reference's name, arguments and result types
(``processing_components/griddata/gridding.py``).  Inputs may be host (NumPy)
data models, in which case they are copied to HBM and results copied back in
ARL's dtypes, or device-resident (``DeviceVisibility`` rows; CUDA tensors in
``GridData.data`` / ``Image.data``), in which case nothing leaves the GPU.
``precision`` selects 'fp32c' (complex64 storage, compensated FP32
accumulation) or 'fp64' (complex128 throughout); the default is set with
``set_default_precision``.
"""
import ctypes

import numpy
import torch

from . import _native as nat
from . import device as dv
from .data_models import GridData, Image, Visibility, copy_visibility


class DeviceVisibility:
    """Row columns resident in HBM: uvw [nvis, 3] f64, frequency [nvis] f64,
    vis [nvis, npol] complex, imaging_weight [nvis, npol] real (precision dtypes)."""

    def __init__(self, uvw, frequency, vis, imaging_weight, polarisation_frame=None, phasecentre=None):
        self.uvw = uvw
        self.frequency = frequency
        self.vis = vis
        self.imaging_weight = imaging_weight
        self.polarisation_frame = polarisation_frame
        self.phasecentre = phasecentre

    @property
    def nvis(self):
        return self.vis.shape[0]

    @property
    def npol(self):
        return self.vis.shape[1]

    @property
    def precision(self):
        return 'fp64' if self.vis.dtype == torch.complex128 else 'fp32c'

    @classmethod
    def from_blockvisibility(cls, bvis, precision=None):
        """Rows formed on the device from an uploaded BlockVisibility
        (``convert_blocks``, ``visibility/coalesce.py:331-443``)."""
        from .coalesce import device_rows_from_blocks
        return device_rows_from_blocks(bvis, precision)

    @classmethod
    def from_visibility(cls, vis, precision=None, device=None):
        precision = dv.resolve_precision(precision)
        device = device or dv.require_cuda()
        return cls(dv.to_device(vis.uvw, torch.float64, device),
                   dv.to_device(vis.frequency, torch.float64, device),
                   dv.to_device(vis.vis, torch.complex128, device).to(dv.CDTYPE[precision]),
                   dv.to_device(vis.imaging_weight, torch.float64, device).to(dv.RDTYPE[precision]),
                   vis.polarisation_frame, vis.phasecentre)


def _rows(vis, precision, device, need_vis=True):
    if isinstance(vis, DeviceVisibility):
        v = vis.vis.to(dv.CDTYPE[precision]) if need_vis else None
        w = vis.imaging_weight.to(dv.RDTYPE[precision]) if need_vis else None
        return vis.uvw, vis.frequency, v, w
    assert isinstance(vis, Visibility), vis
    uvw = dv.to_device(vis.uvw, torch.float64, device)
    f = dv.to_device(vis.frequency, torch.float64, device)
    if not need_vis:
        return uvw, f, None, None
    v = dv.to_device(vis.vis, torch.complex128, device).to(dv.CDTYPE[precision])
    w = dv.to_device(vis.imaging_weight, torch.float64, device).to(dv.RDTYPE[precision])
    return uvw, f, v, w


def _descs(griddata, cf, precision, device):
    gd = dv.grid_desc(griddata.grid_wcs, griddata.data.shape)
    t, cs, ps, psup = dv.device_cf(cf, precision, device)
    cd = dv.cf_desc(cf.grid_wcs, cf.data.shape, cs, ps, psup, table=t)
    return gd, cd, t


def _assert_in_grid(n_bad):
    n = int(n_bad.item())
    assert n == 0, "%d visibilities fall outside the grid or convolution function" % n


def convolution_mapping(vis, griddata, cf, channel_tolerance=1e-8):
    """``gridding.py:24-96``: returns (pu_grid, pu_offset, pv_grid, pv_offset,
    pwg_grid, pwg_fraction, pwc_grid, pwc_fraction, pfreq_grid); the integer
    indices come from the GPU's FP64 mapping, bit-identical to NumPy's."""
    device = dv.require_cuda()
    numpy.testing.assert_almost_equal(griddata.grid_wcs.wcs.cdelt[0], cf.grid_wcs.wcs.cdelt[0], 7)
    numpy.testing.assert_almost_equal(griddata.grid_wcs.wcs.cdelt[1], cf.grid_wcs.wcs.cdelt[1], 7)
    uvw, f, _, _ = _rows(vis, 'fp64', device, need_vis=False)
    n = uvw.shape[0]
    gd = dv.grid_desc(griddata.grid_wcs, griddata.data.shape)
    cd = dv.cf_desc(cf.grid_wcs, cf.data.shape, 0, 0, None)
    outs = [torch.empty(n, dtype=torch.int32, device=device) for _ in range(7)]
    nbad = ctypes.c_int64()
    nat.call('arlgpu_convolution_mapping', nat.ptr(uvw), nat.ptr(f), n, ctypes.byref(gd), ctypes.byref(cd),
             *[nat.ptr(o) for o in outs], ctypes.byref(nbad), nat.stream_ptr())
    pu, puo, pv, pvo, pwg, pwc, pf = (o.cpu().numpy().astype(int) for o in outs)
    assert numpy.min(pu) >= 0, "U axis underflows: %f" % numpy.min(pu)
    assert numpy.max(pu) < griddata.shape[3], "U axis overflows: %f" % numpy.max(pu)
    assert numpy.min(pv) >= 0, "V axis underflows: %f" % numpy.min(pv)
    assert numpy.max(pv) < griddata.shape[4], "V axis overflows: %f" % numpy.max(pv)
    assert numpy.min(pwg) >= 0, "W axis underflows: %f" % numpy.min(pwg)
    assert numpy.max(pwg) < cf.shape[2], "W axis overflows: %f" % numpy.max(pwg)
    assert numpy.min(pwc) >= 0, "W axis underflows: %f" % numpy.min(pwc)
    assert numpy.max(pwc) < cf.shape[2], "W axis overflows: %f" % numpy.max(pwc)
    assert numpy.min(pf) >= 0, "Frequency axis underflows: %f" % numpy.max(pf)
    assert numpy.max(pf) < cf.shape[0], "Frequency axis overflows: %f" % numpy.max(pf)
    w = numpy.asarray(vis.uvw[:, 2].cpu() if isinstance(vis, DeviceVisibility) else vis.uvw[:, 2])
    pwg_fraction = griddata.grid_wcs.sub([3]).wcs_world2pix(w, 0)[0] - pwg
    pwc_fraction = cf.grid_wcs.sub([5]).wcs_world2pix(w, 0)[0] - pwc
    return pu, puo, pv, pvo, pwg, pwg_fraction, pwc, pwc_fraction, pf


def grid_visibility_to_griddata(vis, griddata, cf, precision=None, check=True):
    """``gridding.py:99-133``: zero ``griddata.data`` and grid vis * imaging_weight
    with conj(cf); returns (griddata, sumwt[nchan, npol])."""
    precision = dv.resolve_precision(precision)
    device = dv.require_cuda()
    gd, cd, cf_t = _descs(griddata, cf, precision, device)
    uvw, f, v, w = _rows(vis, precision, device)
    target = griddata.data
    in_place = isinstance(target, torch.Tensor) and target.is_cuda and target.dtype == dv.CDTYPE[precision]
    out, sumwt, n_bad = dv.grid(uvw, f, v, w, cf_t, cd, gd, precision, out=target if in_place else None)
    if check:
        _assert_in_grid(n_bad)
    if not in_place:
        if isinstance(target, torch.Tensor):
            target.copy_(out)
        else:
            griddata.data[...] = out.cpu().numpy()
    return griddata, (sumwt if isinstance(vis, DeviceVisibility) else sumwt.cpu().numpy())


def degrid_visibility_from_griddata(vis, griddata, cf, precision=None, check=True, **kwargs):
    """``gridding.py:233-267``: a new Visibility whose vis column is
    sum(grid window * cf) (no conjugate)."""
    precision = dv.resolve_precision(precision)
    device = dv.require_cuda()
    gd, cd, cf_t = _descs(griddata, cf, precision, device)
    uvw, f, _, _ = _rows(vis, precision, device, need_vis=False)
    g = griddata.data
    if isinstance(g, torch.Tensor):
        g_t = g.to(device=device, dtype=dv.CDTYPE[precision]).contiguous()
    else:
        g_t = dv.to_device(g, torch.complex128, device).to(dv.CDTYPE[precision])
    out, n_bad = dv.degrid(uvw, f, g_t, cf_t, cd, gd, precision)
    if check:
        _assert_in_grid(n_bad)
    if isinstance(vis, DeviceVisibility):
        return DeviceVisibility(vis.uvw, vis.frequency, out, vis.imaging_weight, vis.polarisation_frame,
                                vis.phasecentre)
    newvis = copy_visibility(vis, zero=True)
    newvis.data['vis'][...] = out.cpu().numpy()
    return newvis


def _gcf_t(gcf, device):
    d = gcf.data
    if isinstance(d, torch.Tensor):
        return d.to(device=device, dtype=torch.float64).contiguous()
    return dv.to_device(numpy.asarray(d, dtype=numpy.float64), torch.float64, device)


def fft_griddata_to_image(griddata, gcf, imaginary=False, precision=None, sumwt=None):
    """``gridding.py:270-289``: Re (and Im) of ifft(sum_w grid) * gcf * nx * ny.
    With ``sumwt`` the result is also normalised as ``normalize_sumwt`` does."""
    precision = dv.resolve_precision(precision)
    device = dv.require_cuda()
    g = griddata.data
    host = not isinstance(g, torch.Tensor)
    g_t = dv.to_device(g, torch.complex128, device).to(dv.CDTYPE[precision]) if host else \
        g.to(device=device, dtype=dv.CDTYPE[precision]).contiguous()
    gd = dv.grid_desc(griddata.grid_wcs, g_t.shape)
    sw = None
    if sumwt is not None:
        sw = sumwt if isinstance(sumwt, torch.Tensor) else dv.to_device(numpy.asarray(sumwt, float), torch.float64,
                                                                          device)
    re, im = dv.fft_grid_to_image(g_t, gd, _gcf_t(gcf, device), precision, sumwt=sw, imaginary=imaginary)
    wcs = griddata.projection_wcs
    pf = griddata.polarisation_frame
    if host:
        re = re.cpu().numpy()
        im = im.cpu().numpy() if im is not None else None
    if imaginary:
        return Image(re, wcs.deepcopy(), pf), Image(im, wcs.deepcopy(), pf)
    return Image(re, wcs.deepcopy(), pf)


def fft_image_to_griddata(im, griddata, gcf, precision=None):
    """``gridding.py:292-302``: griddata.data[:, :, z] = fft(im * gcf) for every z."""
    precision = dv.resolve_precision(precision)
    device = dv.require_cuda()
    d = im.data
    im_t = d.to(device=device, dtype=torch.float64) if isinstance(d, torch.Tensor) else \
        dv.to_device(numpy.asarray(d, numpy.float64), torch.float64, device)
    gd = dv.grid_desc(griddata.grid_wcs, griddata.data.shape)
    target = griddata.data
    in_place = isinstance(target, torch.Tensor) and target.is_cuda and target.dtype == dv.CDTYPE[precision]
    out = dv.fft_image_to_grid(im_t, _gcf_t(gcf, device), gd, precision, out=target if in_place else None)
    if not in_place:
        if isinstance(target, torch.Tensor):
            target.copy_(out)
        else:
            griddata.data[...] = out.cpu().numpy()
    return griddata
