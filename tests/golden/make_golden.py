"""Generate golden fixtures by running the reference's own Python code.

Run in a container that has the ARL sources; their location is required,
given with ``--reference`` or the ``ARL_REFERENCE`` environment variable:

    python tests/golden/make_golden.py --reference PATH [--out DIR] [case ...]

With no case names every case runs; ``--out`` (default: this folder) is where
the ``ref_*.npz`` files go.

The reference cannot be imported unchanged here (no astropy; numpy 2 rejects
the scalar assignment at ``processing_components/griddata/kernels.py:72``;
Python 3.12 lacks ``collections.Iterable``).  Three environment shims make it
importable without touching its sources:

* ``astropy_standin.install()`` supplies a linear-axis WCS (all axes on this
  path are linear), celestial directions with the sky-offset transform of
  ``skycoord_to_lmn``, and inert placeholders for the rest;
* ``kernels.grdsf`` is wrapped so a length-1 input returns scalars (the value
  is the reference's own ``grdsf``);
* ``collections.Iterable`` is aliased to ``collections.abc.Iterable``.

Everything else -- mapping, gridding and degridding loops, FFT stages, PSWF
and w-kernel builders, invert_2d / predict_2d, the w-stack workflow, phase
rotation, component predict, gain application -- is the reference's code.
"""
import collections
import collections.abc
import os
import sys

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))


def _args(argv):
    ref, out, cases = os.environ.get('ARL_REFERENCE'), HERE, []
    it = iter(argv)
    for a in it:
        if a == '--reference':
            ref = next(it)
        elif a == '--out':
            out = next(it)
        else:
            cases.append(a)
    if not ref or not os.path.isdir(ref):
        sys.exit('make_golden.py: give the ARL source tree with --reference PATH or ARL_REFERENCE')
    return ref, out, cases


REF, OUT, CASES = _args(sys.argv[1:]) if __name__ == '__main__' else (os.environ.get('ARL_REFERENCE'), HERE, [])

sys.path.insert(0, HERE)
import astropy_standin  # noqa: E402

astropy_standin.install()
sys.path.insert(0, REF)
collections.Iterable = collections.abc.Iterable

from data_models.memory_data_models import Visibility  # noqa: E402
from data_models.polarisation import PolarisationFrame  # noqa: E402
from processing_library.image.operations import create_image_from_array  # noqa: E402
import processing_components.griddata.kernels as kernels  # noqa: E402
from processing_components.griddata import gridding  # noqa: E402
from processing_components.griddata.operations import create_griddata_from_image  # noqa: E402
from processing_components.imaging.base import invert_2d, predict_2d  # noqa: E402

_ref_grdsf = kernels.grdsf


def _grdsf_scalar(nu):
    a, b = _ref_grdsf(nu)
    if numpy.ndim(nu) == 1 and len(nu) == 1:
        return a[0], b[0]
    return a, b


kernels.grdsf = _grdsf_scalar

WCS = astropy_standin.WCS
SkyCoord = astropy_standin.SkyCoord


def make_image(npixel, cellsize, frequency, channel_bandwidth, polframe):
    """Template image with the WCS numbers ``create_image`` writes
    (``processing_library/image/operations.py:31-69``)."""
    pf = PolarisationFrame(polframe)
    nchan = len(frequency)
    w = WCS(naxis=4)
    w.wcs.cdelt = [-cellsize * 180.0 / numpy.pi, cellsize * 180.0 / numpy.pi, 1.0, channel_bandwidth]
    w.wcs.crpix = [npixel // 2 + 1, npixel // 2 + 1, 1.0, 1.0]
    w.wcs.ctype = ["RA---SIN", "DEC--SIN", 'STOKES', 'FREQ']
    w.wcs.crval = [0.0, -45.0, 1.0, frequency[0]]
    w.naxis = 4
    im = create_image_from_array(numpy.zeros([nchan, pf.npol, npixel, npixel]), w, polarisation_frame=pf)
    return im


def make_vis(rng, nvis, npol, umax, wmax, freqs, polframe):
    uvw = numpy.zeros([nvis, 3])
    uvw[:, 0] = rng.uniform(-umax, umax, nvis)
    uvw[:, 1] = rng.uniform(-umax, umax, nvis)
    uvw[:, 2] = rng.uniform(-wmax, wmax, nvis)
    f = rng.choice(freqs, nvis)
    vis = rng.normal(size=(nvis, npol)) + 1j * rng.normal(size=(nvis, npol))
    wt = rng.uniform(0.5, 2.0, size=(nvis, npol))
    z = numpy.zeros(nvis)
    v = Visibility(uvw=uvw, time=z, frequency=f, channel_bandwidth=z + 1e6, vis=vis, weight=wt,
                   imaging_weight=wt, integration_time=z + 1.0, antenna1=z.astype(int),
                   antenna2=z.astype(int), polarisation_frame=PolarisationFrame(polframe))
    v.phasecentre = SkyCoord(0.0, -45.0)
    return v


def case_2d_pswf(out):
    rng = numpy.random.default_rng(4242)
    N, cell, O, S = 128, 4e-3, 8, 8
    im = make_image(N, cell, numpy.array([1e8]), 1e6, 'stokesI')
    du = abs(1.0 / (N * cell))
    vis = make_vis(rng, 3000, 1, (N // 2 - S // 2 - 2) * du, 50.0, numpy.array([1e8]), 'stokesI')
    gcf, cf = kernels.create_pswf_convolutionfunction(im, oversampling=O, support=S)
    gd = create_griddata_from_image(im)
    maps = gridding.convolution_mapping(vis, gd, cf)
    gd, sumwt = gridding.grid_visibility_to_griddata(vis, gd, cf)
    grid = gd.data.copy()
    img_re, img_im = gridding.fft_griddata_to_image(gd, gcf, imaginary=True)
    model = numpy.zeros([1, 1, N, N])
    for _ in range(6):
        model[0, 0, rng.integers(N // 4, 3 * N // 4), rng.integers(N // 4, 3 * N // 4)] = rng.uniform(0.5, 3)
    mim = create_image_from_array(model, im.wcs, im.polarisation_frame)
    gd2 = gridding.fft_image_to_griddata(mim, create_griddata_from_image(im), gcf)
    grid2 = gd2.data.copy()
    newvis = gridding.degrid_visibility_from_griddata(vis, gd2, cf)
    dirty, sumwt2 = invert_2d(vis, im, gcfcf=(gcf, cf))
    psf, _ = invert_2d(vis, im, dopsf=True, gcfcf=(gcf, cf))
    pvis = predict_2d(vis, mim, gcfcf=(gcf, cf))
    numpy.savez_compressed(
        out, N=N, cell=cell, O=O, S=S, freq0=1e8, dfreq=1e6,
        uvw=vis.uvw, frequency=vis.frequency, vis=vis.vis, wt=vis.imaging_weight,
        maps=numpy.stack([numpy.asarray(m) for m in (maps[0], maps[1], maps[2], maps[3], maps[4], maps[6], maps[8])]),
        cf=cf.data, gcf=gcf.data, grid=grid, sumwt=sumwt, img_re=img_re.data, img_im=img_im.data,
        model=model, grid_model=grid2, degrid=newvis.vis, dirty=dirty.data, sumwt_dirty=sumwt2,
        psf=psf.data, predict=pvis.vis)


def case_wproj_2chan_2pol(out):
    rng = numpy.random.default_rng(4343)
    N, cell, O, S, nw, wstep = 64, 8e-3, 4, 8, 5, 20.0
    freqs = numpy.array([1.0e8, 1.1e8])
    im = make_image(N, cell, freqs, 1e7, 'stokesIQ')
    du = abs(1.0 / (N * cell))
    vis = make_vis(rng, 1500, 2, (N // 2 - S // 2 - 2) * du, 2.4 * wstep, freqs, 'stokesIQ')
    gcf, cf = kernels.create_awterm_convolutionfunction(im, nw=nw, wstep=wstep, oversampling=O, support=S,
                                                        use_aaf=True, maxsupport=64)
    gd = create_griddata_from_image(im)
    maps = gridding.convolution_mapping(vis, gd, cf)
    gd, sumwt = gridding.grid_visibility_to_griddata(vis, gd, cf)
    grid = gd.data.copy()
    img_re, img_im = gridding.fft_griddata_to_image(gd, gcf, imaginary=True)
    rgrid = rng.normal(size=grid.shape) + 1j * rng.normal(size=grid.shape)
    gd.data[...] = rgrid
    newvis = gridding.degrid_visibility_from_griddata(vis, gd, cf)
    numpy.savez_compressed(
        out, N=N, cell=cell, O=O, S=S, nw=nw, wstep=wstep, freqs=freqs, dfreq=1e7,
        uvw=vis.uvw, frequency=vis.frequency, vis=vis.vis, wt=vis.imaging_weight,
        maps=numpy.stack([numpy.asarray(m) for m in (maps[0], maps[1], maps[2], maps[3], maps[4], maps[6], maps[8])]),
        cf=cf.data, gcf=gcf.data, grid=grid, sumwt=sumwt, img_re=img_re.data, img_im=img_im.data,
        rgrid=rgrid, degrid=newvis.vis)


def case_wstack(out):
    from workflows.serial.imaging.imaging_serial import invert_list_serial_workflow, \
        predict_list_serial_workflow
    rng = numpy.random.default_rng(4444)
    N, cell, O, S, K = 64, 8e-3, 8, 6, 5
    im = make_image(N, cell, numpy.array([1e8]), 1e6, 'stokesI')
    du = abs(1.0 / (N * cell))
    vis = make_vis(rng, 1200, 1, (N // 2 - S // 2 - 2) * du, 60.0, numpy.array([1e8]), 'stokesI')
    gcfcf = kernels.create_pswf_convolutionfunction(im, oversampling=O, support=S)
    (dirty, sumwt), = invert_list_serial_workflow([vis], [im], context='wstack', vis_slices=K,
                                                  gcfcf=[gcfcf])
    model = numpy.zeros([1, 1, N, N])
    for _ in range(4):
        model[0, 0, rng.integers(N // 4, 3 * N // 4), rng.integers(N // 4, 3 * N // 4)] = rng.uniform(0.5, 3)
    mim = create_image_from_array(model, im.wcs, im.polarisation_frame)
    (pvis,) = predict_list_serial_workflow([vis], [mim], context='wstack', vis_slices=K, gcfcf=[gcfcf])
    # normalize=False: each slice's unnormalised image, weighted by the
    # slice's sumwt, summed and divided by the total (imaging_serial.py:186-197)
    (dirty_nn, sumwt_nn), = invert_list_serial_workflow([vis], [im], context='wstack', vis_slices=K,
                                                        normalize=False, gcfcf=[gcfcf])
    numpy.savez_compressed(out, N=N, cell=cell, O=O, S=S, K=K, freq0=1e8, dfreq=1e6,
                           uvw=vis.uvw, frequency=vis.frequency, vis=vis.vis, wt=vis.imaging_weight,
                           cf=gcfcf[1].data, gcf=gcfcf[0].data, dirty=dirty.data, sumwt=sumwt,
                           model=model, predict=pvis.vis, dirty_nonorm=dirty_nn.data, sumwt_nonorm=sumwt_nn)


def case_workflow_trace(out):
    """The reference's serial workflows (``workflows/serial/imaging/imaging_serial.py:
    41-216``) with context 'wstack' on the ``ref_wstack`` rows, their imaging
    context (``workflows/shared/imaging/imaging_shared.py:21-94``) wrapped so
    that every call the workflow makes is recorded: the row masks its
    vis_iterator yields, each invert's keyword arguments and (image, sumwt),
    each predict's rows.  A test replays the same calls through the package's
    own context functions."""
    from workflows.serial.imaging import imaging_serial
    d = numpy.load(os.path.join(OUT, 'ref_wstack.npz'))
    N, K = int(d['N']), int(d['K'])
    im = make_image(N, float(d['cell']), numpy.array([float(d['freq0'])]), float(d['dfreq']), 'stokesI')
    gcfcf = kernels.create_pswf_convolutionfunction(im, oversampling=int(d['O']), support=int(d['S']))
    n = d['uvw'].shape[0]
    z = numpy.zeros(n)
    vis = Visibility(uvw=d['uvw'], time=z, frequency=d['frequency'], channel_bandwidth=z + float(d['dfreq']),
                     vis=d['vis'].copy(), weight=d['wt'], imaging_weight=d['wt'], integration_time=z + 1.0,
                     antenna1=z.astype(int), antenna2=z.astype(int), polarisation_frame=PolarisationFrame('stokesI'))
    vis.phasecentre = im.phasecentre
    model = create_image_from_array(d['model'], im.wcs, im.polarisation_frame)
    calls = {'masks': [], 'inv_img': [], 'inv_sw': [], 'inv_kw': [], 'pred': []}
    original = imaging_serial.imaging_context

    def traced(context):
        c = dict(original(context))
        inv, pred, it = c['invert'], c['predict'], c['vis_iterator']

        def vis_iterator(v, vis_slices=1):
            for rows in it(v, vis_slices):
                calls['masks'].append(numpy.array(rows, dtype=bool))
                yield rows

        def invert(v, model_im, dopsf=False, normalize=True, **kw):
            r = inv(v, model_im, dopsf=dopsf, normalize=normalize, **kw)
            calls['inv_img'].append(r[0].data.copy())
            calls['inv_sw'].append(numpy.array(r[1]))
            calls['inv_kw'].append([int(dopsf), int(normalize)])
            return r

        def predict(v, model_im, **kw):
            r = pred(v, model_im, **kw)
            calls['pred'].append(r.vis.copy())
            return r
        c.update(invert=invert, predict=predict, vis_iterator=vis_iterator)
        return c
    imaging_serial.imaging_context = traced
    try:
        (dirty, sumwt), = imaging_serial.invert_list_serial_workflow([vis], [im], context='wstack', vis_slices=K,
                                                                     gcfcf=[gcfcf])
        (psf, _), = imaging_serial.invert_list_serial_workflow([vis], [im], context='wstack', vis_slices=K,
                                                               dopsf=True, normalize=False, gcfcf=[gcfcf])
        (pv,) = imaging_serial.predict_list_serial_workflow([vis], [model], context='wstack', vis_slices=K,
                                                            gcfcf=[gcfcf])
    finally:
        imaging_serial.imaging_context = original
    numpy.savez_compressed(out, masks=numpy.array(calls['masks']), inv_img=numpy.array(calls['inv_img']),
                           inv_sw=numpy.array(calls['inv_sw']), inv_kw=numpy.array(calls['inv_kw']),
                           pred=numpy.concatenate(calls['pred']), pred_len=numpy.array([len(p) for p in calls['pred']]),
                           dirty=dirty.data, sumwt=sumwt, psf=psf.data, predict=pv.vis)


def case_kernels(out):
    """Kernel values of the reference's kernel tests
    (``tests/processing_components/test_griddata_kernels.py:33-139``) plus a small
    w-kernel stack with its bounding boxes."""
    im = make_image(512, 0.0005, numpy.array([1e8]), 1e6, 'stokesI')
    _, cf8 = kernels.create_pswf_convolutionfunction(im, oversampling=8, support=6)
    _, cf1 = kernels.create_pswf_convolutionfunction(im, oversampling=1, support=6)
    gcf, cfw = kernels.create_awterm_convolutionfunction(im, nw=9, wstep=8.0, oversampling=8, support=16,
                                                         use_aaf=True)
    from processing_components.griddata.convolution_functions import \
        calculate_bounding_box_convolutionfunction
    bb = calculate_bounding_box_convolutionfunction(cfw, 1e-3)
    numpy.savez_compressed(out, pswf8=cf8.data[0, 0, 0], pswf1=cf1.data[0, 0, 0], gcf=gcf.data[0, 0],
                           wker=cfw.data[0, 0], bbox=numpy.array([[b[0], *b[1], *b[2]] for b in bb]))


def case_wkernels_noaaf(out):
    """``create_awterm_convolutionfunction(use_aaf=False)`` (``processing_components/
    griddata/kernels.py:100-200``): w-screens not divided by the anti-aliasing
    function, and an all-ones grid correction."""
    im = make_image(256, 0.001, numpy.array([1e8]), 1e6, 'stokesI')
    gcf, cfw = kernels.create_awterm_convolutionfunction(im, nw=5, wstep=20.0, oversampling=4, support=8,
                                                         use_aaf=False, maxsupport=128)
    numpy.savez_compressed(out, gcf=gcf.data[0, 0], wker=cfw.data[0, 0])


def case_weighting(out):
    """grid_weight_to_griddata and weight_visibility (uniform weighting,
    ``processing_components/griddata/gridding.py:161-230``,
    ``processing_components/imaging/weighting.py:19-40``), 2 channels x 2 pols,
    with half of the rows sharing a cell with another row."""
    from processing_components.imaging.weighting import weight_visibility
    rng = numpy.random.default_rng(4545)
    N, cell, O, S = 64, 8e-3, 8, 8
    freqs = numpy.array([1.0e8, 1.1e8])
    im = make_image(N, cell, freqs, 1e7, 'stokesIQ')
    du = abs(1.0 / (N * cell))
    vis = make_vis(rng, 2000, 2, (N // 2 - 2) * du, 30.0, freqs, 'stokesIQ')
    vis.data['uvw'][1000:] = vis.data['uvw'][:1000] + rng.uniform(-0.01, 0.01, (1000, 3)) * du
    vis.data['frequency'][1000:] = vis.data['frequency'][:1000]
    gcf, cf = kernels.create_pswf_convolutionfunction(im, oversampling=O, support=S)
    wt_before = vis.imaging_weight.copy()
    gd, sumwt = gridding.grid_weight_to_griddata(vis, create_griddata_from_image(im), cf)
    wgrid = gd.data.copy()
    vis2 = weight_visibility(vis, im, gcfcf=(gcf, cf))
    numpy.savez_compressed(out, N=N, cell=cell, O=O, S=S, freqs=freqs, dfreq=1e7, uvw=vis.uvw,
                           frequency=vis.frequency, wt_before=wt_before, wgrid=wgrid, sumwt=sumwt,
                           wt_after=vis2.imaging_weight.copy())


def case_blocks(out):
    """convert_blockvisibility_to_visibility and its inverse
    (``processing_components/visibility/coalesce.py:85-109,331-443,446-474``) on
    seeded blocks, one and two polarisations."""
    from data_models.memory_data_models import BlockVisibility
    from processing_components.visibility.coalesce import convert_blockvisibility_to_visibility, \
        convert_visibility_to_blockvisibility
    rng = numpy.random.default_rng(4646)
    res = {}
    for npol, frame in ((1, 'stokesI'), (2, 'linearnp')):
        ntimes, nant, nchan = 3, 5, 4
        freqs = numpy.linspace(1.0e8, 1.3e8, nchan)
        shape = (ntimes, nant, nant, nchan, npol)
        uvw = rng.uniform(-500.0, 500.0, (ntimes, nant, nant, 3))
        bvis = rng.normal(size=shape) + 1j * rng.normal(size=shape)
        wt = rng.uniform(0.5, 2.0, shape)
        iwt = rng.uniform(0.5, 2.0, shape)
        times = numpy.arange(ntimes) * 30.0 + 4.5e9
        bv = BlockVisibility(frequency=freqs, channel_bandwidth=numpy.full(nchan, 1e7),
                             phasecentre=SkyCoord(0.0, -45.0), configuration=None, uvw=uvw, time=times,
                             vis=bvis, weight=wt, integration_time=numpy.full(ntimes, 30.0),
                             polarisation_frame=PolarisationFrame(frame), imaging_weight=iwt)
        v = convert_blockvisibility_to_visibility(bv)
        rows = dict(uvw=v.uvw.copy(), vis=v.vis.copy(), weight=v.weight.copy(),
                    imaging_weight=v.imaging_weight.copy(), time=v.time.copy(), frequency=v.frequency.copy(),
                    antenna1=numpy.asarray(v.antenna1).copy(), antenna2=numpy.asarray(v.antenna2).copy(),
                    cindex=numpy.asarray(v.cindex).copy())
        v.data['vis'] *= (2.0 + 1.0j)
        v.data['weight'] *= 3.0
        back = convert_visibility_to_blockvisibility(v)
        for k, a in rows.items():
            res['p%d_%s' % (npol, k)] = a
        res['p%d_block_uvw' % npol] = uvw
        res['p%d_block_vis' % npol] = bvis
        res['p%d_block_weight' % npol] = wt
        res['p%d_block_imaging_weight' % npol] = iwt
        res['p%d_freqs' % npol] = freqs
        res['p%d_times' % npol] = times
        res['p%d_back_vis' % npol] = back.data['vis'].copy()
        res['p%d_back_weight' % npol] = back.data['weight'].copy()
        res['p%d_back_imaging_weight' % npol] = back.data['imaging_weight'].copy()
    numpy.savez_compressed(out, **res)


def case_hogbom(out):
    """Hogbom CLEAN (``processing_library/arrays/cleaners.py:12-69``) and
    ``deconvolve_cube(algorithm='hogbom')`` (``processing_components/image/
    deconvolution.py:43-300``) on a dirty image made from a sampled-uv PSF."""
    from processing_library.arrays.cleaners import hogbom
    from processing_components.image.deconvolution import deconvolve_cube
    rng = numpy.random.default_rng(4747)
    N = 128
    # PSF: the transform of a random uv sampling (sidelobes like a real beam)
    samp = numpy.zeros((N, N))
    samp[rng.integers(N // 2 - 30, N // 2 + 30, 3000), rng.integers(N // 2 - 30, N // 2 + 30, 3000)] = 1.0
    samp = samp + samp[::-1, ::-1]
    psf = numpy.real(numpy.fft.fftshift(numpy.fft.ifft2(numpy.fft.ifftshift(samp))))
    psf /= psf.max()
    sky = numpy.zeros((N, N))
    sky[rng.integers(N // 4, 3 * N // 4, 12), rng.integers(N // 4, 3 * N // 4, 12)] = rng.uniform(0.5, 4.0, 12)
    dirty = numpy.real(numpy.fft.fftshift(numpy.fft.ifft2(numpy.fft.fft2(numpy.fft.ifftshift(sky)) *
                                                          numpy.fft.fft2(numpy.fft.ifftshift(psf)))))
    dirty += 0.01 * rng.normal(size=(N, N))
    window = numpy.zeros((N, N))
    window[N // 8:7 * N // 8, N // 8:7 * N // 8] = 1.0
    c1, r1 = hogbom(dirty, psf, None, 0.1, 0.0, 400, 0.01)
    c2, r2 = hogbom(dirty, psf, window, 0.7, 0.05, 300, 0.001)
    im = make_image(N, 0.001, numpy.array([1e8, 1.1e8]), 1e7, 'stokesI')
    d2 = numpy.stack([dirty, 0.5 * dirty])[:, None]
    p2 = numpy.stack([psf, psf])[:, None]
    dim = create_image_from_array(d2, im.wcs, im.polarisation_frame)
    pim = create_image_from_array(p2.copy(), im.wcs, im.polarisation_frame)
    comp, resid = deconvolve_cube(dim, pim, algorithm='hogbom', niter=200, gain=0.2, threshold=0.0,
                                  fractional_threshold=0.05, window_shape='quarter', psf_support=40)
    numpy.savez_compressed(out, dirty=dirty, psf=psf, window=window, c1=c1, r1=r1, c2=c2, r2=r2, d2=d2, p2=p2,
                           cube_comp=comp.data, cube_resid=resid.data)


def case_hogbom_complex(out):
    """Complex Hogbom CLEAN of Q + iU (``processing_library/arrays/cleaners.py:72-131``)
    and ``deconvolve_cube(algorithm='hogbom-complex')`` on a four-polarisation
    cube (``processing_components/image/deconvolution.py:244-292``: I and V
    by Hogbom, Q and U together)."""
    from processing_library.arrays.cleaners import hogbom_complex
    from processing_components.image.deconvolution import deconvolve_cube
    rng = numpy.random.default_rng(5151)
    N = 96
    samp = numpy.zeros((N, N))
    samp[rng.integers(N // 2 - 24, N // 2 + 24, 2500), rng.integers(N // 2 - 24, N // 2 + 24, 2500)] = 1.0
    samp = samp + samp[::-1, ::-1]
    psf = numpy.real(numpy.fft.fftshift(numpy.fft.ifft2(numpy.fft.ifftshift(samp))))
    psf /= psf.max()

    def dirty_of(sky):
        return numpy.real(numpy.fft.fftshift(numpy.fft.ifft2(numpy.fft.fft2(numpy.fft.ifftshift(sky)) *
                                                             numpy.fft.fft2(numpy.fft.ifftshift(psf)))))
    pos = (rng.integers(N // 4, 3 * N // 4, 10), rng.integers(N // 4, 3 * N // 4, 10))
    sky_i, sky_q, sky_u, sky_v = (numpy.zeros((N, N)) for _ in range(4))
    sky_i[pos] = rng.uniform(1.0, 4.0, 10)
    sky_q[pos] = rng.uniform(-1.0, 1.0, 10)
    sky_u[pos] = rng.uniform(-1.0, 1.0, 10)
    sky_v[pos] = rng.uniform(-0.2, 0.2, 10)
    dq = dirty_of(sky_q) + 0.01 * rng.normal(size=(N, N))
    du = dirty_of(sky_u) + 0.01 * rng.normal(size=(N, N))
    window = numpy.zeros((N, N))
    window[N // 8:7 * N // 8, N // 8:7 * N // 8] = 1.0
    cq1, cu1, rq1, ru1 = hogbom_complex(dq, du, psf, psf, None, 0.1, 0.0, 300, 0.01)
    cq2, cu2, rq2, ru2 = hogbom_complex(dq, du, psf, psf, window, 0.5, 0.02, 200, 0.001)
    im = make_image(N, 0.001, numpy.array([1e8]), 1e7, 'stokesIQUV')
    d4 = numpy.stack([dirty_of(sky_i) + 0.01 * rng.normal(size=(N, N)), dq, du,
                      dirty_of(sky_v) + 0.01 * rng.normal(size=(N, N))])[None]
    p4 = numpy.stack([psf] * 4)[None]
    dim = create_image_from_array(d4, im.wcs, im.polarisation_frame)
    pim = create_image_from_array(p4.copy(), im.wcs, im.polarisation_frame)
    comp, resid = deconvolve_cube(dim, pim, algorithm='hogbom-complex', niter=150, gain=0.2, threshold=0.0,
                                  fractional_threshold=0.05, window_shape='quarter', psf_support=30)
    numpy.savez_compressed(out, dq=dq, du=du, psf=psf, window=window, cq1=cq1, cu1=cu1, rq1=rq1, ru1=ru1,
                           cq2=cq2, cu2=cu2, rq2=rq2, ru2=ru2, di=d4[0, 0], dv=d4[0, 3], cube_comp=comp.data,
                           cube_resid=resid.data)


def case_msclean(out):
    """Multiscale CLEAN (``processing_library/arrays/cleaners.py:165-280``) and
    ``deconvolve_cube(algorithm='msclean')`` on the Hogbom case's dirty image."""
    from processing_library.arrays.cleaners import msclean
    from processing_components.image.deconvolution import deconvolve_cube
    d = numpy.load(os.path.join(OUT, 'ref_hogbom.npz'))
    dirty, psf, window = d['dirty'], d['psf'], d['window']
    c1, r1 = msclean(dirty, psf, None, 0.3, 0.0, 150, [0, 3, 10], 0.01)
    c2, r2 = msclean(dirty, psf[32:96, 32:96], window, 0.7, 0.02, 100, [0, 3], 0.001)
    im = make_image(128, 0.001, numpy.array([1e8, 1.1e8]), 1e7, 'stokesI')
    dim = create_image_from_array(d['d2'], im.wcs, im.polarisation_frame)
    pim = create_image_from_array(d['p2'].copy(), im.wcs, im.polarisation_frame)
    comp, resid = deconvolve_cube(dim, pim, algorithm='msclean', niter=60, gain=0.5, threshold=0.0,
                                  fractional_threshold=0.05, scales=[0, 4, 8], psf_support=32)
    numpy.savez_compressed(out, c1=c1, r1=r1, c2=c2, r2=r2, cube_comp=comp.data, cube_resid=resid.data)


def case_msmfsclean(out):
    """Multi-scale multi-frequency CLEAN (``processing_library/arrays/cleaners.py:469-760``,
    each findpeak), the image frequency moments (``processing_components/image/
    operations.py:239-330``) and ``deconvolve_cube(algorithm='msmfsclean')`` on a
    five-channel cube whose PSF scales with frequency."""
    from processing_library.arrays.cleaners import msmfsclean
    from processing_components.image.deconvolution import deconvolve_cube
    from processing_components.image.operations import calculate_image_frequency_moments
    rng = numpy.random.default_rng(6262)
    N, nchan = 64, 5
    freqs = numpy.linspace(0.9e8, 1.1e8, nchan)
    u = rng.normal(0.0, 7.0, 1500)
    v = rng.normal(0.0, 7.0, 1500)

    def psf_at(f):
        samp = numpy.zeros((N, N))
        iu = numpy.round(u * f / 1e8).astype(int) + N // 2
        iv = numpy.round(v * f / 1e8).astype(int) + N // 2
        ok = (iu > 0) & (iu < N) & (iv > 0) & (iv < N)
        numpy.add.at(samp, (iu[ok], iv[ok]), 1.0)
        samp = samp + samp[::-1, ::-1]
        p = numpy.real(numpy.fft.fftshift(numpy.fft.ifft2(numpy.fft.ifftshift(samp))))
        return p / p.max()

    psfs = numpy.stack([psf_at(f) for f in freqs])
    pos = (rng.integers(N // 4, 3 * N // 4, 6), rng.integers(N // 4, 3 * N // 4, 6))
    flux, alpha = rng.uniform(1.0, 3.0, 6), rng.uniform(-1.0, 0.5, 6)
    cube = numpy.zeros((nchan, 1, N, N))
    for c, f in enumerate(freqs):
        sky = numpy.zeros((N, N))
        sky[pos] = flux * (f / 1e8) ** alpha
        cube[c, 0] = numpy.real(numpy.fft.fftshift(numpy.fft.ifft2(numpy.fft.fft2(numpy.fft.ifftshift(sky)) *
                                                                   numpy.fft.fft2(numpy.fft.ifftshift(psfs[c])))))
    cube += 0.005 * rng.normal(size=cube.shape)
    im = make_image(N, 0.001, freqs, freqs[1] - freqs[0], 'stokesI')
    dim = create_image_from_array(cube, im.wcs, im.polarisation_frame)
    pim = create_image_from_array(psfs[:, None].copy(), im.wcs, im.polarisation_frame)
    dmom = calculate_image_frequency_moments(dim, nmoment=2).data[:, 0]
    pmom = calculate_image_frequency_moments(pim, nmoment=4).data[:, 0]
    res = dict(cube=cube, psfs=psfs, freqs=freqs, dmom=dmom, pmom=pmom)
    window = numpy.zeros((N, N))
    window[8:56, 8:56] = 1.0
    res['window'] = window
    for tag, fp, win in (('arl', 'ARL', None), ('casa', 'CASA', None), ('alg1', 'Algorithm1', None),
                         ('arlw', 'ARL', window)):
        c, r = msmfsclean(dmom.copy(), pmom.copy(), win, 0.3, 0.0, 80, [0, 3, 8], 0.02, fp)
        res['c_' + tag], res['r_' + tag] = c, r
    comp, resid = deconvolve_cube(dim, create_image_from_array(psfs[:, None].copy(), im.wcs, im.polarisation_frame),
                                  algorithm='msmfsclean', nmoment=2, niter=60, gain=0.3, threshold=0.0,
                                  fractional_threshold=0.05, scales=[0, 3, 8])
    res['cube_comp'], res['cube_resid'] = comp.data, resid.data
    numpy.savez_compressed(out, **res)


def case_rotate_uvw(out):
    """``phaserotate_visibility(tangent=False)`` (``processing_components/visibility/
    base.py:295-343``) forward and inverse on the phase-rotation rows of
    ``ref_rowops``: the phases as on the tangent plane, then uvw re-projected
    through earth coordinates (``uvw_to_xyz`` / ``xyz_to_uvw``,
    ``processing_library/util/coordinate_support.py:59-113``) and the phase
    centre moved."""
    from processing_components.visibility.base import phaserotate_visibility
    d = numpy.load(os.path.join(OUT, 'ref_rowops.npz'))
    uvw, vis = d['rot_uvw'], d['rot_vis']
    n = uvw.shape[0]
    z = numpy.zeros(n)
    res = {}
    for tag, inverse in (('fwd', False), ('inv', True)):
        v = Visibility(uvw=uvw.copy(), time=z, frequency=z + 1e8, channel_bandwidth=z + 1e6, vis=vis.copy(),
                       weight=z[:, None] + 1.0, imaging_weight=z[:, None] + 1.0, integration_time=z + 1.0,
                       antenna1=z.astype(int), antenna2=z.astype(int), polarisation_frame=PolarisationFrame('stokesIQ'))
        v.phasecentre = SkyCoord(*d['rot_vis_pc'])
        r = phaserotate_visibility(v, SkyCoord(*d['rot_far_pc']), tangent=False, inverse=inverse)
        res['vis_' + tag] = r.vis.copy()
        res['uvw_' + tag] = r.uvw.copy()
        res['pc_' + tag] = numpy.array([r.phasecentre.ra.deg, r.phasecentre.dec.deg])
    numpy.savez_compressed(out, **res)


def case_rowops(out):
    """Row operations on the path's edges, from the reference's own code:

    * ``skycoord_to_lmn`` (``processing_library/util/coordinate_support.py:150-169``)
      on the stand-in's directions, first checked against every expectation of
      the reference's ``test_skycoord_to_lmn``, then on offsets of the kind
      the imaging path meets;
    * ``shift_vis_to_image`` / ``phaserotate_visibility`` (tangent, both
      directions; ``processing_components/imaging/base.py:50-81``,
      ``processing_components/visibility/base.py:295-334``) on a Visibility
      whose phase centre differs from the image's;
    * ``predict_skycomponent_visibility`` (``imaging/base.py:192-244``) on a
      Visibility (3 channels, 2 polarisations) and a BlockVisibility;
    * ``apply_gaintable`` with scalar gains, forward and inverse
      (``processing_components/calibration/operations.py:79-164``), with
      zero gain weights and one zero gain."""
    from numpy.testing import assert_allclose
    from data_models.memory_data_models import BlockVisibility, GainTable, Skycomponent
    from data_models.polarisation import ReceptorFrame
    from processing_library.util.coordinate_support import skycoord_to_lmn
    from processing_components.imaging.base import shift_vis_to_image, predict_skycomponent_visibility
    from processing_components.visibility.base import phaserotate_visibility
    from processing_components.calibration.operations import apply_gaintable
    res = {}
    # (1) the stand-in against the reference's own skycoord_to_lmn test
    center, north, south = SkyCoord(0, 0), SkyCoord(0, 90), SkyCoord(0, -90)
    east, west = SkyCoord(90, 0), SkyCoord(-90, 0)
    kat = [(center, center, (0, 0, 0), 0), (north, center, (0, 1, -1), 0), (south, center, (0, -1, -1), 0),
           (south, north, (0, 0, -2), 1e-14), (east, center, (1, 0, -1), 0), (west, center, (-1, 0, -1), 0),
           (center, west, (1, 0, -1), 0), (north, west, (0, 1, -1), 1e-14), (south, west, (0, -1, -1), 1e-14),
           (north, east, (0, 1, -1), 1e-14), (south, east, (0, -1, -1), 1e-14)]
    for a, b, want, atol in kat:
        assert_allclose(skycoord_to_lmn(a, b), want, atol=atol)
    rng = numpy.random.default_rng(4848)
    pcs = numpy.column_stack([rng.uniform(-180, 180, 16), rng.uniform(-85, 85, 16)])
    offs = numpy.column_stack([pcs[:, 0] + rng.uniform(-6, 6, 16), numpy.clip(pcs[:, 1] + rng.uniform(-6, 6, 16),
                                                                                -89, 89)])
    res['lmn_pc'] = pcs
    res['lmn_dir'] = offs
    res['lmn'] = numpy.array([skycoord_to_lmn(SkyCoord(*o), SkyCoord(*p)) for o, p in zip(offs, pcs)])

    # (2) phase rotation to the image's phase centre
    n = 3000
    uvw = rng.normal(size=(n, 3)) * numpy.array([800.0, 800.0, 80.0])
    z = numpy.zeros(n)
    vis = rng.normal(size=(n, 2)) + 1j * rng.normal(size=(n, 2))
    v = Visibility(uvw=uvw, time=z, frequency=z + 1e8, channel_bandwidth=z + 1e6, vis=vis, weight=z[:, None] + 1.0,
                   imaging_weight=z[:, None] + 1.0, integration_time=z + 1.0, antenna1=z.astype(int),
                   antenna2=z.astype(int), polarisation_frame=PolarisationFrame('stokesIQ'))
    v.phasecentre = SkyCoord(10.0, -45.0)
    im = make_image(64, 1e-3, numpy.array([1e8]), 1e6, 'stokesIQ')
    im.wcs.wcs.crval[0], im.wcs.wcs.crval[1] = 10.3, -44.8
    fwd = shift_vis_to_image(v, im, tangent=True, inverse=False)
    inv = shift_vis_to_image(v, im, tangent=True, inverse=True)
    far = phaserotate_visibility(v, SkyCoord(25.0, -30.0), tangent=True, inverse=False)
    res.update(rot_uvw=uvw, rot_vis=vis, rot_vis_pc=numpy.array([10.0, -45.0]), rot_im_pc=numpy.array([10.3, -44.8]),
               rot_fwd=fwd.vis.copy(), rot_inv=inv.vis.copy(), rot_far_pc=numpy.array([25.0, -30.0]),
               rot_far=far.vis.copy(),
               rot_lmn=numpy.array(skycoord_to_lmn(im.phasecentre, v.phasecentre)))

    # (3) point components onto rows (3 channels, 2 pols) and onto blocks
    freqs = numpy.array([1.0e8, 1.1e8, 1.2e8])
    n = 4000
    f = rng.choice(freqs, n)
    uvw = rng.uniform(-3000, 3000, (n, 3)) * numpy.array([1.0, 1.0, 0.1])
    z = numpy.zeros(n)
    base = rng.normal(size=(n, 2)) + 1j * rng.normal(size=(n, 2))
    v = Visibility(uvw=uvw, time=z, frequency=f, channel_bandwidth=z + 1e7, vis=base.copy(), weight=z[:, None] + 1.0,
                   imaging_weight=z[:, None] + 1.0, integration_time=z + 1.0, antenna1=z.astype(int),
                   antenna2=z.astype(int), polarisation_frame=PolarisationFrame('linearnp'))
    v.phasecentre = SkyCoord(0.0, -45.0)
    cdir = numpy.column_stack([rng.uniform(-4, 4, 10), -45.0 + rng.uniform(-4, 4, 10)])
    cflux = rng.uniform(0.1, 5.0, (10, 3, 2))
    comps = [Skycomponent(direction=SkyCoord(*d), frequency=freqs, flux=fl,
                          polarisation_frame=PolarisationFrame('linearnp')) for d, fl in zip(cdir, cflux)]
    predict_skycomponent_visibility(v, comps)
    res.update(dft_uvw=uvw, dft_freq=f, dft_base=base, dft_dir=cdir, dft_flux=cflux, dft_pc=numpy.array([0.0, -45.0]),
               dft_vis=v.vis.copy())
    ntimes, nant = 3, 6
    buvw = rng.uniform(-2000.0, 2000.0, (ntimes, nant, nant, 3))
    bbase = rng.normal(size=(ntimes, nant, nant, 3, 2)) + 1j * rng.normal(size=(ntimes, nant, nant, 3, 2))
    bv = BlockVisibility(frequency=freqs, channel_bandwidth=numpy.full(3, 1e7), phasecentre=SkyCoord(0.0, -45.0),
                         configuration=None, uvw=buvw, time=numpy.arange(ntimes) * 30.0, vis=bbase.copy(),
                         weight=numpy.ones(bbase.shape), integration_time=numpy.full(ntimes, 30.0),
                         polarisation_frame=PolarisationFrame('linearnp'), imaging_weight=numpy.ones(bbase.shape))
    predict_skycomponent_visibility(bv, comps)
    res.update(dftb_uvw=buvw, dftb_base=bbase, dftb_vis=bv.vis.copy())

    # (4) scalar gains on a BlockVisibility, forward and inverse
    ntimes, nant, nchan = 4, 7, 3
    times = 4.5e9 + numpy.arange(ntimes) * 30.0
    gshape = (ntimes, nant, nant, nchan, 1)
    gvis = rng.normal(size=gshape) + 1j * rng.normal(size=gshape)
    gain = (rng.normal(1.0, 0.1, (ntimes, nant, nchan, 1, 1)) *
            numpy.exp(1j * rng.uniform(-numpy.pi, numpy.pi, (ntimes, nant, nchan, 1, 1))))
    gain[2, 3, 1] = 0.0
    gwt = numpy.ones((ntimes, nant, nchan, 1, 1))
    gwt[1, 2, 0] = 0.0
    gwt[3, 5, 2] = 0.0
    gt = GainTable(gain=gain, time=times, interval=numpy.full(ntimes, 30.0), weight=gwt,
                   residual=numpy.zeros((ntimes, nchan, 1, 1)), frequency=freqs,
                   receptor_frame=ReceptorFrame('stokesI'))

    def block():
        return BlockVisibility(frequency=freqs, channel_bandwidth=numpy.full(nchan, 1e7),
                               phasecentre=SkyCoord(0.0, -45.0), configuration=None,
                               uvw=numpy.zeros((ntimes, nant, nant, 3)), time=times, vis=gvis.copy(),
                               weight=numpy.ones(gshape), integration_time=numpy.full(ntimes, 30.0),
                               polarisation_frame=PolarisationFrame('stokesI'), imaging_weight=numpy.ones(gshape))
    fwd = apply_gaintable(block(), gt)
    inv = apply_gaintable(block(), gt, inverse=True)
    res.update(gt_vis=gvis, gt_time=times, gt_interval=numpy.full(ntimes, 30.0), gt_gain=gain, gt_weight=gwt,
               gt_freqs=freqs, gt_fwd=fwd.vis.copy(), gt_inv=inv.vis.copy())
    numpy.savez_compressed(out, **res)


# Public functions of the path: (reference module, name).  Their signatures
# are recorded so the package's functions can be checked against them.
API = [
    ('processing_components.griddata.gridding', n) for n in (
        'convolution_mapping', 'grid_visibility_to_griddata', 'degrid_visibility_from_griddata',
        'fft_griddata_to_image', 'fft_image_to_griddata', 'grid_weight_to_griddata', 'griddata_merge_weights',
        'griddata_reweight')] + [
    ('processing_components.griddata.kernels', 'create_pswf_convolutionfunction'),
    ('processing_components.griddata.kernels', 'create_awterm_convolutionfunction'),
    ('processing_components.griddata.convolution_functions', 'calculate_bounding_box_convolutionfunction'),
    ('processing_components.griddata.convolution_functions', 'apply_bounding_box_convolutionfunction'),
    ('processing_components.griddata.operations', 'create_griddata_from_image'),
    ('processing_components.imaging.base', 'invert_2d'),
    ('processing_components.imaging.base', 'predict_2d'),
    ('processing_components.imaging.base', 'shift_vis_to_image'),
    ('processing_components.imaging.base', 'normalize_sumwt'),
    ('processing_components.imaging.base', 'predict_skycomponent_visibility'),
    ('processing_components.imaging.wstack_single', 'invert_wstack_single'),
    ('processing_components.imaging.wstack_single', 'predict_wstack_single'),
    ('processing_components.visibility.base', 'phaserotate_visibility'),
    ('processing_components.visibility.iterators', 'vis_wslice_iter'),
    ('processing_components.visibility.iterators', 'vis_null_iter'),
    ('processing_components.calibration.operations', 'apply_gaintable'),
    ('processing_components.visibility.coalesce', 'convert_blockvisibility_to_visibility'),
    ('processing_components.visibility.coalesce', 'convert_visibility_to_blockvisibility'),
    ('processing_components.image.deconvolution', 'deconvolve_cube'),
    ('processing_library.arrays.cleaners', 'hogbom'),
    ('processing_library.arrays.cleaners', 'hogbom_complex'),
    ('processing_library.arrays.cleaners', 'msclean'),
    ('processing_library.arrays.cleaners', 'msmfsclean'),
    ('processing_components.image.operations', 'calculate_image_frequency_moments'),
    ('processing_components.image.operations', 'calculate_image_from_frequency_moments'),
    ('workflows.shared.imaging.imaging_shared', 'imaging_contexts'),
    ('workflows.shared.imaging.imaging_shared', 'imaging_context'),
    ('workflows.serial.imaging.imaging_serial', 'invert_list_serial_workflow'),
    ('workflows.serial.imaging.imaging_serial', 'predict_list_serial_workflow'),
]


def case_api(out):
    """Signatures of the path's public functions: parameter names, kinds and
    defaults (literal defaults as values, anything else as its type name)."""
    import importlib
    import inspect
    import json
    rec = []
    for mod, name in API:
        fn = getattr(importlib.import_module(mod), name)
        params = []
        for p in inspect.signature(fn).parameters.values():
            d = p.default
            if d is inspect.Parameter.empty:
                dv = None
                has = False
            else:
                has = True
                dv = d if isinstance(d, (int, float, str, bool, type(None))) else '<%s>' % type(d).__name__
            params.append({'name': p.name, 'kind': p.kind.name, 'has_default': has, 'default': dv})
        rec.append({'module': mod, 'name': name, 'params': params})
    with open(out[:-4] + '.json', 'w') as f:
        json.dump(rec, f, indent=1)


ALL_CASES = {
    'ref_2d_pswf': case_2d_pswf,
    'ref_wproj_2chan_2pol': case_wproj_2chan_2pol,
    'ref_wstack': case_wstack,
    'ref_workflow_trace': case_workflow_trace,
    'ref_kernels': case_kernels,
    'ref_wkernels_noaaf': case_wkernels_noaaf,
    'ref_weighting': case_weighting,
    'ref_blocks': case_blocks,
    'ref_hogbom': case_hogbom,
    'ref_hogbom_complex': case_hogbom_complex,
    'ref_msclean': case_msclean,
    'ref_msmfsclean': case_msmfsclean,
    'ref_rowops': case_rowops,
    'ref_rotate_uvw': case_rotate_uvw,
    'ref_api': case_api,
}

if __name__ == '__main__':
    os.makedirs(OUT, exist_ok=True)
    for name, fn in ALL_CASES.items():
        if not CASES or name in CASES:
            fn(os.path.join(OUT, name + '.npz'))
            made = [f for f in (name + '.npz', name + '.json') if os.path.exists(os.path.join(OUT, f))]
            print(name, [(f, os.path.getsize(os.path.join(OUT, f))) for f in made])
