"""Batched w-stacking over one set of rows, with the whole pipeline resident in
HBM and optionally recorded as a CUDA graph.

Reference behaviour:
  vis_wslice_iter                   processing_components/visibility/iterators.py:91-109
  invert_wstack_single / predict_wstack_single
                                    processing_components/imaging/wstack_single.py:26-96
  sum of the slices (sumwt-weighted images, normalised by the total sumwt)
                                    workflows/serial/imaging/imaging_serial.py:186-197
  predicted rows of every slice     workflows/serial/imaging/imaging_serial.py:41-122

ARL loops over K w-slices in Python: copy the slice's rows, shift w by the
slice's mean, invert_2d or predict_2d, multiply by the w-beam, sum.  Here every
slice is one plane of a [nchan, npol, K, ny, nx] grid:

  invert   plan (FP64 map + bin rows by channel, slice and uv-tile) -> one
           gridder launch over all channels, polarisations and slices ->
           inverse transforms of the planes (double-single on FP32C,
           complex128 on FP64), the last pass applying each slice's w-beam
           and summing the slices into the image.
  predict  one pass writing conj(w-beam_s) * model * gcf into every plane ->
           forward transforms -> one degridder launch over all rows (each row
           reads its own slice's plane).

``capture()`` records either pipeline, plan build included, into a CUDA
graph; ``load_rows()`` copies new rows of the same count into the resident
buffers, so a replay images the new rows.
"""
import ctypes

import numpy
import torch

from . import _native as nat
from . import device as dv
from .data_models import GridData
from .gridding import DeviceVisibility, _gcf_t, _rows
from .kernels import _grid_wcs, create_pswf_convolutionfunction


def slice_axis(w_t, vis_slices):
    """WW grid axis (crval, crpix, cdelt) whose round-to-nearest plane index is
    the ``vis_wslice_iter`` slice: boxes linspace(-wmax, wmax, K), a row in slice
    s when |w - box_s| < step/2 (``visibility/iterators.py:91-109``)."""
    wmax = float(w_t.abs().max().item()) if w_t.numel() else 0.0
    if vis_slices > 1:
        step = (2.0 * wmax) / (vis_slices - 1)
    else:
        step = 2.0 * wmax
    if step == 0.0:
        step = 1e15
    return -wmax, 1.0, step


class WStackImager:
    """W-stack invert / predict of one set of rows onto one image geometry.

    vis: Visibility or DeviceVisibility; im: template Image [nchan, npol, ny, nx];
    gcfcf: (gcf, cf) with a 2-D kernel (nz == 1), default PSWF.  The plan (row
    mapping and binning), the grid, the FFT scratch and the outputs stay on the
    device for the imager's lifetime."""

    def __init__(self, vis, im, vis_slices, gcfcf=None, precision=None):
        self.precision = dv.resolve_precision(precision)
        self.device = dv.require_cuda()
        gcf, cf = gcfcf if gcfcf is not None else create_pswf_convolutionfunction(im)
        if cf.shape[2] != 1:
            raise NotImplementedError('batched w-stacking grids with a 2-D kernel (nz == 1); use '
                                      'invert_wstack_single per slice for w-stacking with w-projection kernels')
        self.gcf, self.cf, self.im = gcf, cf, im
        self.vis_slices = vis_slices
        self.uvw, self.f, self.v, self.w = _rows(vis, self.precision, self.device)
        self.n = self.uvw.shape[0]
        nchan, npol, ny, nx = im.shape
        self.shape = (nchan, npol, ny, nx)
        self.gwcs = _grid_wcs(im, vis_slices, 1e15)
        self.w_axis = slice_axis(self.uvw[:, 2], vis_slices)
        self.gwcs.wcs.crval[2], self.gwcs.wcs.crpix[2], self.gwcs.wcs.cdelt[2] = self.w_axis
        self.gd = dv.grid_desc(self.gwcs, (nchan, npol, vis_slices, ny, nx))
        self.cf_t, cs, ps, self._psup = dv.device_cf(cf, self.precision, self.device)
        self.cd = dv.cf_desc(cf.grid_wcs, cf.data.shape, cs, ps, self._psup, table=self.cf_t)
        self.ws = torch.empty(dv.plan_bytes(self.n, self.gd, self.cd), dtype=torch.uint8, device=self.device)
        self.n_bad = torch.zeros(1, dtype=torch.int64, device=self.device)
        self.wmean = torch.empty(vis_slices, dtype=torch.float64, device=self.device)
        self.gcf_t = _gcf_t(gcf, self.device)
        self.cellsize = abs(float(im.wcs.wcs.cdelt[0])) * numpy.pi / 180.0
        cdt = dv.CDTYPE[self.precision]
        self.grid_t = torch.empty((nchan, npol, vis_slices, ny, nx), dtype=cdt, device=self.device)
        self.sumwt = torch.empty((nchan, npol), dtype=torch.float64, device=self.device)
        self.ones = torch.ones((nchan, npol), dtype=torch.float64, device=self.device)
        self.image = torch.empty((nchan, npol, ny, nx), dtype=torch.float64, device=self.device)
        self.model = torch.zeros((nchan, npol, ny, nx), dtype=torch.float64, device=self.device)
        self.out = torch.empty((self.n, npol), dtype=cdt, device=self.device)
        if self.precision == 'fp64':
            self.fftbuf = self.grid_t
        else:
            nbytes = ctypes.c_size_t(0)
            nat.call('arlgpu_wstack_fftbuf_bytes', ctypes.byref(self.gd), ctypes.byref(nbytes))
            self.fftbuf = torch.empty(nbytes.value // 16, dtype=torch.complex128, device=self.device)
        self.psf_v = None
        self.graphs = {}
        self._owned = False
        self.plan()
        self.check_rows()

    # -- stages -------------------------------------------------------------
    def plan(self):
        """FP64 mapping + binning of the rows, and each slice's mean w."""
        nat.call('arlgpu_plan_build', nat.ptr(self.uvw), nat.ptr(self.f), self.n, ctypes.byref(self.gd),
                 ctypes.byref(self.cd), nat.ptr(self.ws), self.ws.numel(), nat.ptr(self.n_bad), nat.stream_ptr())
        nat.call('arlgpu_plan_plane_mean_w', nat.ptr(self.uvw), self.n, ctypes.byref(self.gd), ctypes.byref(self.cd),
                 nat.ptr(self.ws), self.ws.numel(), nat.ptr(self.wmean), nat.stream_ptr())

    def check_rows(self):
        """Raise as ARL's asserts do if a row falls outside the grid.  Rows
        outside every slice (possible only with one slice) are dropped as
        vis_wslice_iter drops them."""
        crval, crpix, cdelt = self.w_axis
        pw = torch.round((self.uvw[:, 2] - crval) / cdelt + crpix - 1.0)
        n_outside = int(((pw < 0) | (pw >= self.vis_slices)).sum().item())
        nb = int(self.n_bad.item())
        assert nb == n_outside, "%d visibilities fall outside the grid or convolution function" % (nb - n_outside)

    def grid(self, dopsf=False):
        """All rows onto the slice planes (zeroed first); sumwt [nchan, npol]."""
        if dopsf:
            if self.psf_v is None:
                self.psf_v = torch.ones_like(self.v)
            v = self.psf_v
        else:
            v = self.v
        nat.call('arlgpu_grid_planned', nat.ptr(v), nat.ptr(self.w), self.n, nat.PRECISIONS[self.precision],
                 nat.ptr(self.cf_t), ctypes.byref(self.cd), nat.ptr(self.grid_t), ctypes.byref(self.gd),
                 nat.ptr(self.sumwt), nat.ptr(self.ws), self.ws.numel(), nat.stream_ptr())

    def grid_to_image(self, normalize=True):
        """Slice planes -> image (w-beams applied, slices summed, / sumwt)."""
        norm = self.sumwt if normalize else self.ones
        nat.call('arlgpu_wstack_grid_to_image', nat.ptr(self.grid_t), ctypes.byref(self.gd),
                 nat.PRECISIONS[self.precision], nat.ptr(self.gcf_t), nat.ptr(self.wmean), self.cellsize,
                 nat.ptr(norm), nat.ptr(self.image), nat.ptr(self.fftbuf), nat.stream_ptr())

    def invert(self, dopsf=False, normalize=True, replan=False):
        """(image tensor [nchan, npol, ny, nx], sumwt tensor); the tensors are the
        imager's own buffers, overwritten by the next call."""
        if replan:
            self.plan()
        self.grid(dopsf)
        self.grid_to_image(normalize)
        return self.image, self.sumwt

    def predict(self, model=None, replan=False):
        """Predicted rows [n, npol] of ``model`` (tensor or array [nchan, npol, ny,
        nx]; default the imager's ``model`` buffer)."""
        if model is not None:
            self.set_model(model)
        if replan:
            self.plan()
        nat.call('arlgpu_wstack_image_to_grid', nat.ptr(self.model), nat.ptr(self.gcf_t), nat.ptr(self.wmean),
                 self.cellsize, ctypes.byref(self.gd), nat.PRECISIONS[self.precision], nat.ptr(self.grid_t),
                 nat.stream_ptr())
        nat.call('arlgpu_degrid_planned', self.n, nat.PRECISIONS[self.precision], nat.ptr(self.cf_t),
                 ctypes.byref(self.cd), nat.ptr(self.grid_t), ctypes.byref(self.gd), nat.ptr(self.out),
                 nat.ptr(self.ws), self.ws.numel(), nat.stream_ptr())
        return self.out

    def set_model(self, model):
        m = model if isinstance(model, torch.Tensor) else torch.as_tensor(numpy.asarray(model, numpy.float64))
        self.model.copy_(m.to(device=self.device, dtype=torch.float64).reshape(self.model.shape))

    @property
    def griddata(self):
        """The slice planes as a GridData (UU, VV, WW = slice axis, STOKES, FREQ)."""
        return GridData(self.grid_t, self.gwcs, self.im.wcs.deepcopy(), self.im.polarisation_frame)

    # -- resident rows and CUDA graphs ---------------------------------------
    def _own_rows(self):
        if not self._owned:
            self.uvw, self.f = self.uvw.clone(), self.f.clone()
            self.v, self.w = self.v.clone(), self.w.clone()
            self._owned = True

    def load_rows(self, uvw=None, frequency=None, vis=None, weight=None):
        """Copy new rows (same count) into the imager's own buffers.  The WW
        slice axis stays as built; rows beyond it are reported in n_bad."""
        self._own_rows()
        for dst, src in ((self.uvw, uvw), (self.f, frequency), (self.v, vis), (self.w, weight)):
            if src is not None:
                t = src if isinstance(src, torch.Tensor) else torch.as_tensor(numpy.asarray(src))
                dst.copy_(t.reshape(dst.shape), non_blocking=True)

    def capture(self, which='invert', dopsf=False, normalize=True):
        """Record 'invert' (plan + grid + transforms + combine) or 'predict'
        (plan + model transforms + degrid) as one CUDA graph; returns it.
        Replaying reads the imager's resident rows and model buffer."""
        self._own_rows()
        if which == 'invert':
            def fn():
                self.invert(dopsf, normalize, replan=True)
        elif which == 'predict':
            def fn():
                self.predict(replan=True)
        else:
            raise ValueError(which)
        side = torch.cuda.Stream(device=self.device)
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            fn()  # creates the cuFFT plans and kernel attributes before capture
        torch.cuda.current_stream().wait_stream(side)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            fn()
        self.graphs[which] = g
        return g

    def replay(self, which='invert'):
        self.graphs[which].replay()
        return (self.image, self.sumwt) if which == 'invert' else self.out


def invert_to_host(imager, vis, dopsf, normalize):
    image, sumwt = imager.invert(dopsf, normalize)
    if isinstance(vis, DeviceVisibility):
        return image.clone(), sumwt.clone()
    return image.cpu().numpy(), sumwt.cpu().numpy()
