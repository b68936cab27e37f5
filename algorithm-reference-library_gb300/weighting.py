"""Uniform weighting on the GB300 kernels.

Reference behaviour:
  grid_weight_to_griddata   processing_components/griddata/gridding.py:161-183
  griddata_merge_weights    processing_components/griddata/gridding.py:186-210
  griddata_reweight         processing_components/griddata/gridding.py:213-230
  weight_visibility         processing_components/imaging/weighting.py:19-40

The weight grid is summed on the device in FP64 (atomics, so sums of
non-integer weights may differ from NumPy's sequential sums in the last bit);
the reweighting divides each row's imaging weights by its cell's sum.
"""
import ctypes

import numpy
import torch

from . import _native as nat
from . import device as dv
from .data_models import Visibility
from .gridding import DeviceVisibility
from .kernels import copy_griddata, create_pswf_convolutionfunction


def _weight_rows(vis, precision, device):
    """(uvw, frequency, imaging weight) device tensors; the weights are the
    caller's own tensor for a DeviceVisibility (updated in place by reweight)."""
    if isinstance(vis, DeviceVisibility):
        return vis.uvw, vis.frequency, vis.imaging_weight
    assert isinstance(vis, Visibility), vis
    uvw = dv.to_device(vis.uvw, torch.float64, device)
    f = dv.to_device(vis.frequency, torch.float64, device)
    w = dv.to_device(vis.imaging_weight, torch.float64, device).to(dv.RDTYPE[precision])
    return uvw, f, w


def _precision_of(vis, precision):
    if isinstance(vis, DeviceVisibility):
        return 'fp64' if vis.imaging_weight.dtype == torch.float64 else 'fp32c'
    return dv.resolve_precision(precision) if precision is not None else 'fp64'


def _grid_weights(uvw, f, w, gd, cd, precision, device):
    shape = (gd.nchan, gd.npol, gd.nw, gd.ny, gd.nx)
    wgrid = torch.empty(shape, dtype=torch.float64, device=device)
    sumwt = torch.empty((gd.nchan, gd.npol), dtype=torch.float64, device=device)
    n_bad = torch.zeros(1, dtype=torch.int64, device=device)
    w = w.contiguous()
    nat.call('arlgpu_grid_weights', nat.ptr(uvw), nat.ptr(f), nat.ptr(w), uvw.shape[0], nat.PRECISIONS[precision],
             ctypes.byref(cd), nat.ptr(wgrid), ctypes.byref(gd), nat.ptr(sumwt), nat.ptr(n_bad), nat.stream_ptr())
    nb = int(n_bad.item())
    assert nb == 0, "%d visibilities fall outside the grid" % nb
    return wgrid, sumwt


def grid_weight_to_griddata(vis, griddata, cf, precision=None):
    """``gridding.py:161-183``: zero ``griddata.data`` and add each row's imaging
    weight to its nearest cell; returns (griddata, sumwt[nchan, npol])."""
    precision = _precision_of(vis, precision)
    device = dv.require_cuda()
    gd = dv.grid_desc(griddata.grid_wcs, griddata.data.shape)
    cd = dv.cf_desc(cf.grid_wcs, cf.data.shape, 0, 0, None)
    uvw, f, w = _weight_rows(vis, precision, device)
    wgrid, sumwt = _grid_weights(uvw, f, w, gd, cd, precision, device)
    target = griddata.data
    if isinstance(target, torch.Tensor):
        target.copy_(wgrid.to(target.dtype))
    else:
        target[...] = wgrid.cpu().numpy()
    return griddata, (sumwt if isinstance(vis, DeviceVisibility) else sumwt.cpu().numpy())


def griddata_merge_weights(gd_list, algorithm='uniform'):
    """``gridding.py:186-210``: sum the (griddata, sumwt) pairs into a copy of
    the centre one; its FREQ axis gets the summed bandwidth and mean frequency."""
    centre = len(gd_list) // 2
    gd = copy_griddata(gd_list[centre][0])
    sumwt = gd_list[centre][1]
    frequency = 0.0
    bandwidth = 0.0
    for i, g in enumerate(gd_list):
        if i != centre:
            gd.data += g[0].data
            sumwt += g[1]
        frequency += g[0].grid_wcs.wcs.crval[4]
        bandwidth += g[0].grid_wcs.wcs.cdelt[4]
    gd.grid_wcs.wcs.cdelt[4] = bandwidth
    gd.grid_wcs.wcs.crval[4] = frequency / len(gd_list)
    return gd, sumwt


def griddata_reweight(vis, griddata, cf, precision=None):
    """``gridding.py:213-230``: each row's imaging weights divided by the real
    part of its nearest cell of ``griddata`` when every polarisation's cell is
    non-zero.  Updates ``vis`` in place and returns it."""
    precision = _precision_of(vis, precision)
    device = dv.require_cuda()
    gd = dv.grid_desc(griddata.grid_wcs, griddata.data.shape)
    cd = dv.cf_desc(cf.grid_wcs, cf.data.shape, 0, 0, None)
    g = griddata.data
    if isinstance(g, torch.Tensor):
        wgrid = (g.real if g.is_complex() else g).to(device=device, dtype=torch.float64).contiguous()
    else:
        wgrid = dv.to_device(numpy.real(g), torch.float64, device)
    uvw, f, w = _weight_rows(vis, precision, device)
    _reweight(vis, uvw, f, w, wgrid, gd, cd, precision)
    return vis


def _reweight(vis, uvw, f, w, wgrid, gd, cd, precision):
    wc = w if w.is_contiguous() else w.contiguous()
    nat.call('arlgpu_reweight', nat.ptr(uvw), nat.ptr(f), nat.ptr(wc), uvw.shape[0], nat.PRECISIONS[precision],
             ctypes.byref(cd), nat.ptr(wgrid), ctypes.byref(gd), nat.stream_ptr())
    if isinstance(vis, DeviceVisibility):
        if wc is not w:
            w.copy_(wc)
    else:
        vis.data['imaging_weight'][...] = wc.to(torch.float64).cpu().numpy()


def weight_visibility(vis, model, gcfcf=None, weighting='uniform', precision=None, **kwargs):
    """``imaging/weighting.py:19-40``: uniform weighting.  The weights are gridded
    onto the model's grid (nearest cell) and each row's imaging weight is divided
    by its cell's sum, in place.  As in the reference, ``weighting`` is not
    consulted.  Returns ``vis``."""
    if gcfcf is None:
        gcfcf = create_pswf_convolutionfunction(model)
    from .kernels import _grid_wcs
    precision = _precision_of(vis, precision)
    device = dv.require_cuda()
    nchan, npol, ny, nx = model.shape
    gd = dv.grid_desc(_grid_wcs(model, 1, 1e15), (nchan, npol, 1, ny, nx))
    cf = gcfcf[1]
    cd = dv.cf_desc(cf.grid_wcs, cf.data.shape, 0, 0, None)
    uvw, f, w = _weight_rows(vis, precision, device)
    wgrid, _ = _grid_weights(uvw, f, w, gd, cd, precision, device)
    _reweight(vis, uvw, f, w, wgrid, gd, cd, precision)
    return vis
