"""BlockVisibility <-> Visibility on the GB300 kernels.

Reference behaviour:
  convert_blockvisibility_to_visibility   processing_components/visibility/coalesce.py:85-109
  convert_blocks                          processing_components/visibility/coalesce.py:331-443
  convert_visibility_to_blockvisibility   processing_components/visibility/coalesce.py:446-454
  decoalesce_visibility                   processing_components/visibility/coalesce.py:112-143

``DeviceVisibility.from_blockvisibility`` (below, ``device_rows_from_blocks``)
turns an uploaded block straight into the gridder's row layout in HBM, so no
host reshaping sits between a BlockVisibility and the gridder.
"""
import ctypes

import numpy
import torch

from . import _native as nat
from . import device as dv
from .data_models import BlockVisibility, Visibility, copy_blockvisibility
from .gridding import DeviceVisibility


def _block_columns(bvis, precision, device):
    cdt, rdt = dv.CDTYPE[precision], dv.RDTYPE[precision]
    d = bvis.data
    return (dv.to_device(d['vis'], torch.complex128, device).to(cdt),
            dv.to_device(d['uvw'], torch.float64, device),
            dv.to_device(d['weight'], torch.float64, device).to(rdt),
            dv.to_device(d['imaging_weight'], torch.float64, device).to(rdt),
            dv.to_device(bvis.frequency, torch.float64, device))


def _convert(bvis, precision, device, want_index=True):
    ntimes, nant, _, nchan, npol = bvis.data['vis'].shape
    nrows = ntimes * nant * (nant - 1) // 2 * nchan
    bv, buvw, bw, biw, freq = _block_columns(bvis, precision, device)
    cdt, rdt = dv.CDTYPE[precision], dv.RDTYPE[precision]
    out = dict(vis=torch.empty((nrows, npol), dtype=cdt, device=device),
               uvw=torch.empty((nrows, 3), dtype=torch.float64, device=device),
               weight=torch.empty((nrows, npol), dtype=rdt, device=device),
               imaging_weight=torch.empty((nrows, npol), dtype=rdt, device=device),
               frequency=torch.empty(nrows, dtype=torch.float64, device=device),
               antenna1=torch.empty(nrows, dtype=torch.int32, device=device),
               antenna2=torch.empty(nrows, dtype=torch.int32, device=device),
               time_index=torch.empty(nrows, dtype=torch.int32, device=device),
               cindex=torch.empty(ntimes * nant * nant * nchan, dtype=torch.int64, device=device)
               if want_index else None)
    nat.call('arlgpu_convert_blocks', nat.ptr(bv), nat.ptr(buvw), nat.ptr(bw), nat.ptr(biw), nat.ptr(freq),
             ntimes, nant, nchan, npol, nat.PRECISIONS[precision], nat.ptr(out['vis']), nat.ptr(out['uvw']),
             nat.ptr(out['weight']), nat.ptr(out['imaging_weight']), nat.ptr(out['frequency']),
             nat.ptr(out['antenna1']), nat.ptr(out['antenna2']), nat.ptr(out['time_index']),
             nat.ptr(out['cindex']), nat.stream_ptr())
    return out


def convert_blockvisibility_to_visibility(vis, precision='fp64'):
    """``coalesce.py:85-109``: rows (time, a2, a1, channel) over the baselines
    a2 > a1, uvw in wavelengths, with ``cindex`` and ``blockvis`` filled in."""
    assert isinstance(vis, BlockVisibility), "vis is not a BlockVisibility: %r" % vis
    device = dv.require_cuda()
    o = _convert(vis, precision, device)
    ntimes, nant, _, nchan, npol = vis.data['vis'].shape
    nbl = nant * (nant - 1) // 2
    tix = o['time_index'].cpu().numpy()
    chan = numpy.tile(numpy.arange(nchan), ntimes * nbl)
    return Visibility(uvw=o['uvw'].cpu().numpy(), time=vis.time[tix], frequency=o['frequency'].cpu().numpy(),
                      channel_bandwidth=vis.channel_bandwidth[chan], phasecentre=vis.phasecentre,
                      antenna1=o['antenna1'].cpu().numpy().astype(int),
                      antenna2=o['antenna2'].cpu().numpy().astype(int),
                      vis=o['vis'].to(torch.complex128).cpu().numpy(),
                      weight=o['weight'].to(torch.float64).cpu().numpy(),
                      imaging_weight=o['imaging_weight'].to(torch.float64).cpu().numpy(),
                      configuration=vis.configuration, integration_time=vis.integration_time[tix],
                      polarisation_frame=vis.polarisation_frame, cindex=o['cindex'].cpu().numpy(), blockvis=vis,
                      meta=vis.meta)


def device_rows_from_blocks(bvis, precision=None):
    """A DeviceVisibility straight from a BlockVisibility: one upload of the
    block, rows formed on the device.  The returned object also carries
    antenna1, antenna2, time_index and cindex tensors."""
    precision = dv.resolve_precision(precision)
    device = dv.require_cuda()
    o = _convert(bvis, precision, device)
    dvis = DeviceVisibility(o['uvw'], o['frequency'], o['vis'], o['imaging_weight'], bvis.polarisation_frame,
                            bvis.phasecentre)
    for k in ('antenna1', 'antenna2', 'time_index', 'cindex', 'weight'):
        setattr(dvis, k, o[k])
    return dvis


def _decoalesce_column(rows, cindex, block, device):
    """Rows [nrows, npol] back into a copy of block [..., npol] (reference loop semantics)."""
    ntimes, nant, _, nchan, npol = block.shape
    is_c = numpy.iscomplexobj(block)
    r = torch.as_tensor(numpy.ascontiguousarray(rows, dtype=numpy.complex128 if is_c else numpy.float64)).to(device)
    b = torch.as_tensor(numpy.ascontiguousarray(block, dtype=numpy.complex128 if is_c else numpy.float64)).to(device)
    ci = torch.as_tensor(numpy.ascontiguousarray(cindex, dtype=numpy.int64)).to(device)
    n_bad = torch.zeros(1, dtype=torch.int64, device=device)
    nat.call('arlgpu_decoalesce', nat.ptr(r), r.shape[0], nat.ptr(ci), ntimes, nant, nchan, npol,
             16 if is_c else 8, nat.ptr(b), nat.ptr(n_bad), nat.stream_ptr())
    nb = int(n_bad.item())
    assert nb == 0, "Incorrect template used in decoalescing"
    return b.cpu().numpy()


def decoalesce_visibility(vis, **kwargs):
    """``coalesce.py:112-143``: a copy of ``vis.blockvis`` with its vis, weight and
    imaging_weight overwritten from the rows through ``vis.cindex``."""
    assert isinstance(vis, Visibility), "vis is not a Visibility: %r" % vis
    assert isinstance(vis.blockvis, BlockVisibility), "No blockvisibility in vis %r" % vis
    assert vis.cindex is not None, "No reverse index in Visibility %r" % vis
    device = dv.require_cuda()
    out = copy_blockvisibility(vis.blockvis)
    assert numpy.max(vis.cindex) < vis.vis.shape[0], "Incorrect template used in decoalescing"
    for col in ('vis', 'weight', 'imaging_weight'):
        out.data[col] = _decoalesce_column(vis.data[col], vis.cindex, vis.blockvis.data[col], device)
    return out


def convert_visibility_to_blockvisibility(vis):
    """``coalesce.py:446-454``."""
    if isinstance(vis, BlockVisibility):
        return vis
    return decoalesce_visibility(vis)
