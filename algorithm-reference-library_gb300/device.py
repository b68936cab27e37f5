"""Device-resident layer: torch CUDA tensors in, libarlgpu calls out.

The ARL-compatible functions (``gridding``, ``imaging``, ``kernels``) convert
their data models to the tensors and descriptors used here.  Everything in
this module works on tensors already in HBM; host copies happen only in the
callers that were handed NumPy arrays.
"""
import ctypes

import numpy
import torch

from . import _native as nat

CDTYPE = {'fp32c': torch.complex64, 'fp64': torch.complex128}
RDTYPE = {'fp32c': torch.float32, 'fp64': torch.float64}

_default_precision = 'fp32c'


def set_default_precision(p):
    """'fp32c' (complex64 storage, compensated FP32 accumulation) or 'fp64'."""
    global _default_precision
    if p not in nat.PRECISIONS:
        raise ValueError(p)
    _default_precision = p


def default_precision():
    return _default_precision


def resolve_precision(p):
    p = _default_precision if p is None else p
    if p not in nat.PRECISIONS:
        raise ValueError("precision must be 'fp32c' or 'fp64', got %r" % (p,))
    return p


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError('arl_gb300 needs a CUDA device: there is no CPU fallback')
    nat.load()
    return torch.device('cuda', torch.cuda.current_device())


# ---------------------------------------------------------------------------
# Descriptors
# ---------------------------------------------------------------------------
def _axis(wcs, i):
    a = nat.Axis()
    a.crval, a.crpix, a.cdelt = wcs.axis(i)
    return a


def grid_desc(grid_wcs, shape):
    """GridDesc from a GridData WCS (axes UU, VV, WW, STOKES, FREQ) and shape
    [nchan, npol, nw, ny, nx]."""
    d = nat.GridDesc()
    d.nchan, d.npol, d.nw, d.ny, d.nx = (int(s) for s in shape)
    d.u, d.v, d.w, d.f = _axis(grid_wcs, 0), _axis(grid_wcs, 1), _axis(grid_wcs, 2), _axis(grid_wcs, 4)
    return d


def cf_desc(cf_wcs, shape, chan_stride, pol_stride, plane_support=None, table=None):
    """CfDesc from a ConvolutionFunction WCS (UU, VV, DUU, DVV, WW, ...) and shape
    [nchan, npol, nz, O, O, S, S]; strides in elements.  With the device
    ``table`` (from device_cf) the descriptor carries the table's largest tap
    component, which lets the FP32C gridder sum tiles in fixed point."""
    d = nat.CfDesc()
    d.nchan, d.npol, d.nz, d.oversampling, _, d.support, _ = (int(s) for s in shape)
    d.chan_stride, d.pol_stride = int(chan_stride), int(pol_stride)
    d.du, d.dv, d.z = _axis(cf_wcs, 2), _axis(cf_wcs, 3), _axis(cf_wcs, 4)
    d.plane_support = None if plane_support is None else plane_support.data_ptr()
    d.tap_absmax = 0.0 if table is None else tap_absmax(table)
    return d


_ABSMAX = {}


def tap_absmax(table):
    """max(|Re|, |Im|) over a device cf table, remembered per (tensor, version)."""
    key = (table.data_ptr(), table.numel(), table._version)
    hit = _ABSMAX.get(id(table))
    if hit is not None and hit[0] == key:
        return hit[1]
    v = float(torch.view_as_real(table).abs().max().item()) if table.numel() else 0.0
    _ABSMAX[id(table)] = (key, v)
    return v


# ---------------------------------------------------------------------------
# Scratch
# ---------------------------------------------------------------------------
class Workspace:
    """Grow-only scratch buffer per device (stream-ordered reuse)."""

    def __init__(self):
        self._buf = {}

    def get(self, nbytes, device):
        key = (device.type, device.index)
        b = self._buf.get(key)
        if b is None or b.numel() < nbytes:
            b = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)
            self._buf[key] = b
        return b


WORKSPACE = Workspace()


def plan_bytes(nvis, gd, cd):
    out = ctypes.c_size_t()
    nat.call('arlgpu_plan_workspace_bytes', int(nvis), ctypes.byref(gd), ctypes.byref(cd), ctypes.byref(out))
    return out.value


# ---------------------------------------------------------------------------
# Convolution function upload
# ---------------------------------------------------------------------------
def device_cf(cf, precision, device):
    """(table tensor, chan_stride, pol_stride, plane_support tensor|None) for a
    ConvolutionFunction; cached on the object until its ``data`` is replaced.
    Channel / polarisation blocks that are identical to block [0, 0] are stored
    once (stride 0)."""
    key = (precision, device.type, device.index)
    hit = cf._device_cache.get(key)
    if hit is not None:
        return hit
    data = cf.data
    nchan, npol, nz, O, _, S, _ = data.shape
    block = nz * O * O * S * S
    if isinstance(data, torch.Tensor):
        t = data.to(device=device, dtype=CDTYPE[precision]).contiguous()
        cs, ps = npol * block, block
    else:
        same = all(numpy.array_equal(data[c, p], data[0, 0]) for c in range(nchan) for p in range(npol))
        if same:
            t = torch.from_numpy(numpy.ascontiguousarray(data[0, 0])).to(device=device, dtype=CDTYPE[precision])
            cs, ps = 0, 0
        else:
            t = torch.from_numpy(numpy.ascontiguousarray(data)).to(device=device, dtype=CDTYPE[precision])
            cs, ps = npol * block, block
    psup = None
    if cf.plane_support is not None:
        psup = torch.as_tensor(numpy.asarray(cf.plane_support, dtype=numpy.int32), device=device)
    out = (t, cs, ps, psup)
    cf._device_cache[key] = out
    return out


# ---------------------------------------------------------------------------
# Hot path on device tensors
# ---------------------------------------------------------------------------
def _check_rows(uvw, freq, nvis):
    assert uvw.is_cuda and uvw.dtype == torch.float64 and uvw.shape == (nvis, 3) and uvw.is_contiguous()
    assert freq.is_cuda and freq.dtype == torch.float64 and freq.shape == (nvis,) and freq.is_contiguous()


def grid(uvw, freq, vis, wt, cf_t, cd, gd, precision, out=None, sumwt=None, n_bad=None, stream=None):
    """Grid rows into ``out`` [nchan, npol, nw, ny, nx] (zeroed first); returns
    (grid, sumwt, n_bad) with n_bad a 1-element int64 device tensor."""
    nvis = vis.shape[0]
    _check_rows(uvw, freq, nvis)
    dev = uvw.device
    assert vis.dtype == CDTYPE[precision] and wt.dtype == RDTYPE[precision]
    assert vis.shape == (nvis, gd.npol) and wt.shape == (nvis, gd.npol) and vis.is_contiguous() and wt.is_contiguous()
    assert cf_t.dtype == CDTYPE[precision]
    if out is None:
        out = torch.empty((gd.nchan, gd.npol, gd.nw, gd.ny, gd.nx), dtype=CDTYPE[precision], device=dev)
    if sumwt is None:
        sumwt = torch.empty((gd.nchan, gd.npol), dtype=torch.float64, device=dev)
    if n_bad is None:
        n_bad = torch.zeros(1, dtype=torch.int64, device=dev)
    nbytes = plan_bytes(nvis, gd, cd)
    ws = WORKSPACE.get(nbytes, dev)
    nat.call('arlgpu_grid', nat.ptr(uvw), nat.ptr(freq), nat.ptr(vis), nat.ptr(wt), nvis, nat.PRECISIONS[precision],
             nat.ptr(cf_t), ctypes.byref(cd), nat.ptr(out), ctypes.byref(gd), nat.ptr(sumwt), nat.ptr(n_bad),
             nat.ptr(ws), ws.numel(), nat.stream_ptr(stream))
    return out, sumwt, n_bad


def degrid(uvw, freq, grid_t, cf_t, cd, gd, precision, out=None, n_bad=None, stream=None):
    """Predict rows from a device grid; returns (vis [nvis, npol], n_bad)."""
    nvis = uvw.shape[0]
    _check_rows(uvw, freq, nvis)
    dev = uvw.device
    assert grid_t.dtype == CDTYPE[precision] and grid_t.is_contiguous()
    assert tuple(grid_t.shape) == (gd.nchan, gd.npol, gd.nw, gd.ny, gd.nx)
    if out is None:
        out = torch.empty((nvis, gd.npol), dtype=CDTYPE[precision], device=dev)
    if n_bad is None:
        n_bad = torch.zeros(1, dtype=torch.int64, device=dev)
    nbytes = plan_bytes(nvis, gd, cd)
    ws = WORKSPACE.get(nbytes, dev)
    nat.call('arlgpu_degrid', nat.ptr(uvw), nat.ptr(freq), nvis, nat.PRECISIONS[precision], nat.ptr(cf_t),
             ctypes.byref(cd), nat.ptr(grid_t), ctypes.byref(gd), nat.ptr(out), nat.ptr(n_bad), nat.ptr(ws),
             ws.numel(), nat.stream_ptr(stream))
    return out, n_bad


def fft_grid_to_image(grid_t, gd, gcf_t, precision, sumwt=None, imaginary=False, buf=None, stream=None):
    """Image (and imaginary part) [nchan, npol, ny, nx] float64 from a device grid.
    ``buf`` is complex128 FFT scratch (a complex128 grid with nw == 1 may be reused)."""
    dev = grid_t.device
    shape = (gd.nchan, gd.npol, gd.ny, gd.nx)
    re = torch.empty(shape, dtype=torch.float64, device=dev)
    im = torch.empty(shape, dtype=torch.float64, device=dev) if imaginary else None
    if buf is None or buf.dtype != torch.complex128:
        buf = torch.empty(shape, dtype=torch.complex128, device=dev)
    nat.call('arlgpu_fft_grid_to_image', nat.ptr(grid_t), ctypes.byref(gd), nat.PRECISIONS[precision],
             nat.ptr(gcf_t), nat.ptr(sumwt), nat.ptr(re), nat.ptr(im), nat.ptr(buf), nat.stream_ptr(stream))
    return re, im


def fft_image_to_grid(image_t, gcf_t, gd, precision, out=None, stream=None):
    """Device grid [nchan, npol, nw, ny, nx] = centred FFT of image * gcf."""
    dev = image_t.device
    if out is None:
        out = torch.empty((gd.nchan, gd.npol, gd.nw, gd.ny, gd.nx), dtype=CDTYPE[precision], device=dev)
    image_t = image_t.contiguous()
    gcf_t = gcf_t.contiguous()
    nat.call('arlgpu_fft_image_to_grid', nat.ptr(image_t), nat.ptr(gcf_t),
             ctypes.byref(gd), nat.PRECISIONS[precision], nat.ptr(out), nat.stream_ptr(stream))
    return out


def to_device(a, dtype, device, non_blocking=True):
    """Host NumPy array -> device tensor through pinned memory."""
    t = torch.from_numpy(numpy.ascontiguousarray(a)).to(dtype)
    if device.type == 'cuda':
        t = t.pin_memory().to(device, non_blocking=non_blocking)
    return t
