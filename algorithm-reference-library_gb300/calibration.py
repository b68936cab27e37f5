"""Gain application on the GB300 kernels.

Reference behaviour:
  apply_gaintable      processing_components/calibration/operations.py:79-164
  vis_timeslice_iter   processing_components/visibility/iterators.py:35-58
  vis_timeslices       processing_components/visibility/iterators.py:61-76

The host walks ARL's time slices and looks up each slice's gain-table rows
(a few comparisons per slice); the block itself is updated on the GPU
(``arlgpu_apply_gaintable``), one launch per group of slices that do not share
a block time.
"""
import numpy
import torch

from . import _native as nat
from . import device as dv
from .data_models import BlockVisibility, GainTable


def vis_timeslices(vis, timeslice='auto'):
    """Number of time slices: the count of distinct times, or the span over
    ``timeslice`` seconds (``iterators.py:61-76``)."""
    if timeslice == 'auto':
        return len(numpy.unique(vis.time))
    return numpy.ceil(numpy.max(vis.time) - numpy.min(vis.time)) / timeslice


def vis_timeslice_iter(vis, vis_slices=None):
    """Boolean masks over the block times, one per slice: the times within
    half a slice of each of ``vis_slices`` equally spaced centres
    (``iterators.py:35-58``)."""
    tmin, tmax = numpy.min(vis.time), numpy.max(vis.time)
    if vis_slices is None:
        vis_slices = vis_timeslices(vis, 'auto')
    boxes = numpy.linspace(tmin, tmax, vis_slices)
    timeslice = boxes[1] - boxes[0] if vis_slices > 1 else tmax - tmin
    for box in boxes:
        yield numpy.abs(vis.time - box) <= 0.5 * timeslice


def gain_rows_per_pass(vis_time, gt_time, gt_interval, vis_slices=None):
    """The gain-table row of each block time, in passes: ARL's loop takes the
    time slices in order and gives a slice's k-th time the k-th gain-table row
    whose time lies within half an interval of the slice's mean time
    (``operations.py:108-119``).  Slices are merged into one pass (one launch)
    until one of them shares a block time with the pass, which starts the next
    pass: a time on a slice boundary is then updated twice, as the reference's
    loop does.  Returns a list of int32 arrays [ntimes] (-1: time untouched)."""
    vis_time = numpy.asarray(vis_time)
    passes = []
    pending = numpy.full(vis_time.shape[0], -1, dtype=numpy.int32)
    for rows in vis_timeslice_iter(_Times(vis_time), vis_slices=vis_slices):
        if numpy.sum(rows) == 0:
            continue
        vistime = numpy.average(vis_time[rows])
        grows = numpy.nonzero(numpy.abs(gt_time - vistime) < gt_interval / 2.0)[0]
        times = numpy.nonzero(rows)[0]
        if grows.size > times.size:
            raise IndexError('apply_gaintable: %d gain-table rows for a slice of %d times' % (grows.size, times.size))
        times = times[:grows.size]
        if numpy.any(pending[times] >= 0):
            passes.append(pending)
            pending = numpy.full(vis_time.shape[0], -1, dtype=numpy.int32)
        pending[times] = grows
    if numpy.any(pending >= 0):
        passes.append(pending)
    return passes


class _Times:
    def __init__(self, time):
        self.time = time


def apply_gaintable(vis, gt, inverse=False, vis_slices=None, precision=None, **kwargs):
    """``calibration/operations.py:79-164`` for scalar gains: every block cell
    of a slice's k-th time is multiplied by g_i g_j^* of the k-th gain-table row
    whose time lies within half an interval of the slice's mean time (1/g for
    the inverse; cells whose antennas' gain weights multiply to 0 are zeroed).
    Updates ``vis`` in place and returns it.  Polarised (2 x 2) gains raise
    NotImplementedError."""
    assert isinstance(vis, BlockVisibility), 'vis is not a BlockVisibility: %r' % vis
    assert isinstance(gt, GainTable), 'gt is not a GainTable: %r' % gt
    assert vis.nchan == gt.nchan
    assert vis.npol == gt.nrec * gt.nrec
    if gt.gain.shape[-2:] != (1, 1):
        raise NotImplementedError('apply_gaintable: only scalar gains run on the GB300 path')
    ntimes, nant, _, nchan, _ = vis.vis.shape
    assert gt.nants == nant
    device = dv.require_cuda()
    prec = dv.resolve_precision(precision) if precision is not None else 'fp64'
    v = dv.to_device(numpy.ascontiguousarray(vis.vis[..., 0]), torch.complex128, device).to(dv.CDTYPE[prec])
    gain = dv.to_device(numpy.ascontiguousarray(gt.gain[..., 0, 0]), torch.complex128, device)
    gwt = dv.to_device(numpy.ascontiguousarray(gt.weight[..., 0, 0]), torch.float64, device)
    for trow in gain_rows_per_pass(vis.time, gt.time, gt.interval, vis_slices):
        t = torch.as_tensor(trow, device=device)
        nat.call('arlgpu_apply_gaintable', nat.ptr(v), ntimes, nant, nchan, nat.PRECISIONS[prec], nat.ptr(t),
                 nat.ptr(gain), nat.ptr(gwt), int(bool(inverse)), nat.stream_ptr())
    vis.data['vis'][..., 0] = v.to(torch.complex128).cpu().numpy()
    return vis
