"""Point-component (DFT) predict on the GB300 kernels.

Reference behaviour:
  predict_skycomponent_visibility   processing_components/imaging/base.py:192-244
  simulate_point                    processing_library/util/coordinate_support.py:192-212
  get_frequency_map (im=None)       processing_library/imaging/imaging_params.py:18-48

Each component adds flux[chan(row), pol] * exp(-2 pi i uvw . s) to every row,
s = (l, m, sqrt(1 - l^2 - m^2) - 1) with (l, m) the component's direction
cosines relative to the visibility phase centre.  The phase is formed in FP64
on the GPU (``csrc/dft.cu``).
"""
import collections.abc

import numpy
import torch

from . import _native as nat
from . import device as dv
from .data_models import BlockVisibility, Skycomponent, Visibility
from .gridding import DeviceVisibility

C_M_S = 299792458.0


def _components(sc, phasecentre):
    if not isinstance(sc, collections.abc.Iterable):
        sc = [sc]
    sc = list(sc)
    lmn = numpy.empty((len(sc), 3))
    for i, comp in enumerate(sc):
        assert isinstance(comp, Skycomponent), comp
        l, m, _ = comp.direction.lmn(phasecentre)
        lmn[i] = (l, m, numpy.sqrt(1 - l ** 2 - m ** 2) - 1.0)
    flux = numpy.stack([c.flux for c in sc]) if sc else numpy.zeros((0, 1, 1))
    return lmn, flux


def _row_channels(frequency):
    """Channel of each row: its frequency's rank among the unique frequencies
    (``get_frequency_map`` with no image)."""
    uf, inv = numpy.unique(numpy.asarray(frequency), return_inverse=True)
    return inv.astype(numpy.int32), uf.size


def dft_predict(uvw, row_chan, lmn, flux, vis, precision):
    """vis (device tensor [nvis, npol]) += DFT of the components; all device tensors."""
    npol = vis.shape[1]
    ncomp, nchan = flux.shape[0], flux.shape[1]
    rc = None if row_chan is None else row_chan
    nat.call('arlgpu_dft_predict', nat.ptr(uvw), nat.ptr(rc), uvw.shape[0], nat.ptr(lmn), nat.ptr(flux), ncomp,
             nchan, npol, nat.PRECISIONS[precision], nat.ptr(vis), nat.stream_ptr())
    return vis


def dft_adjoint(uvw, lmn, x, precision, image=None):
    """image[k, p] (+)= Re sum_r conj(exp(-2 pi i uvw_r . s_k)) x[r, p] on the device."""
    ncomp = lmn.shape[0]
    npol = x.shape[1]
    if image is None:
        image = torch.zeros((ncomp, npol), dtype=torch.float64, device=x.device)
    xc = x.contiguous()
    nat.call('arlgpu_dft_adjoint', nat.ptr(uvw), uvw.shape[0], nat.ptr(lmn), ncomp, npol, nat.PRECISIONS[precision],
             nat.ptr(xc), nat.ptr(image), nat.stream_ptr())
    return image


def predict_skycomponent_visibility(vis, sc, precision=None):
    """``imaging/base.py:192-244``: add the components' visibilities to ``vis``
    (Visibility, DeviceVisibility or BlockVisibility) in place; returns it."""
    if sc is None:
        return vis
    device = dv.require_cuda()
    lmn, flux = _components(sc, vis.phasecentre)
    if lmn.shape[0] == 0:
        return vis
    lmn_t = torch.as_tensor(lmn, device=device)
    if isinstance(vis, DeviceVisibility):
        prec = vis.precision
        freq = vis.frequency.cpu().numpy()
        rc, nchan = _row_channels(freq)
        assert flux.shape[1] >= nchan and flux.shape[2] == vis.npol, "component and visibility channels / pols"
        rc_t = torch.as_tensor(rc, device=device)
        flux_t = torch.as_tensor(numpy.ascontiguousarray(flux), device=device)
        dft_predict(vis.uvw, rc_t, lmn_t, flux_t, vis.vis, prec)
        return vis
    prec = dv.resolve_precision(precision) if precision is not None else 'fp64'
    if isinstance(vis, Visibility):
        rc, nchan = _row_channels(vis.frequency)
        assert flux.shape[1] >= nchan and flux.shape[2] == vis.npol, "component and visibility channels / pols"
        uvw = dv.to_device(vis.uvw, torch.float64, device)
        v = dv.to_device(vis.vis, torch.complex128, device).to(dv.CDTYPE[prec])
        rc_t = torch.as_tensor(rc, device=device)
        flux_t = torch.as_tensor(numpy.ascontiguousarray(flux), device=device)
        dft_predict(uvw, rc_t, lmn_t, flux_t, v, prec)
        vis.data['vis'][...] = v.to(torch.complex128).cpu().numpy()
        return vis
    assert isinstance(vis, BlockVisibility), vis
    # Every block cell, [t, i, j, chan], with uvw (metres) * f / c per channel.
    ntimes, nant, _, nchan, npol = vis.vis.shape
    k = torch.as_tensor(vis.frequency / C_M_S, device=device)
    buvw = dv.to_device(vis.uvw, torch.float64, device)                      # [t, i, j, 3]
    uvw = (buvw[..., None, :] * k[:, None]).reshape(-1, 3).contiguous()     # [t, i, j, c, 3]
    rc_t = torch.arange(nchan, dtype=torch.int32, device=device).repeat(ntimes * nant * nant)
    v = dv.to_device(vis.vis, torch.complex128, device).to(dv.CDTYPE[prec]).reshape(-1, npol).contiguous()
    flux_t = torch.as_tensor(numpy.ascontiguousarray(flux), device=device)
    dft_predict(uvw, rc_t, lmn_t, flux_t, v, prec)
    vis.data['vis'][...] = v.to(torch.complex128).cpu().numpy().reshape(vis.vis.shape)
    return vis
