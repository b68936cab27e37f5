"""W-stacking on the GPU against the reference's serial w-stack workflow
(golden fixture) and the oracle."""
import numpy
import pytest
import torch

from helpers import assert_image

pytestmark = pytest.mark.gpu
TOL = {'fp64': 1e-10, 'fp32c': 1e-5}  # outputs pass through an FFT


def rel(a, b):
    return float(numpy.max(numpy.abs(numpy.asarray(a) - b)) / numpy.max(numpy.abs(b)))


@pytest.fixture(scope='module', autouse=True)
def need_cuda(arl):
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')


def _case(arl, d):
    im = arl.create_image(npixel=int(d['N']), cellsize=float(d['cell']), frequency=numpy.array([1e8]),
                          channel_bandwidth=numpy.array([1e6]), phasecentre=arl.PhaseCentre(0.0, -45.0))
    gcf, cf = arl.create_pswf_convolutionfunction(im, oversampling=int(d['O']), support=int(d['S']))
    vis = arl.Visibility(uvw=d['uvw'], frequency=d['frequency'], vis=d['vis'], weight=d['wt'], imaging_weight=d['wt'])
    vis.phasecentre = arl.PhaseCentre(0.0, -45.0)
    return im, gcf, cf, vis


@pytest.mark.parametrize('precision', ['fp64', 'fp32c'])
def test_wstack_workflow_matches_reference(arl, golden, precision):
    d = golden('ref_wstack.npz')
    im, gcf, cf, vis = _case(arl, d)
    K = int(d['K'])
    (dirty, sumwt), = arl.imaging.invert_list_serial_workflow([vis], [im], context='wstack', vis_slices=K,
                                                               gcfcf=[(gcf, cf)], precision=precision)
    assert_image(dirty.data, d['dirty'], d['gcf'], precision)
    assert numpy.allclose(sumwt, d['sumwt'], rtol=1e-12 if precision == 'fp64' else 1e-6)
    model = arl.create_image_from_array(d['model'], im.wcs, im.polarisation_frame)
    (pv,) = arl.imaging.predict_list_serial_workflow([vis], [model], context='wstack', vis_slices=K,
                                                      gcfcf=[(gcf, cf)], precision=precision)
    assert rel(pv.vis, d['predict']) < TOL[precision]


@pytest.mark.parametrize('precision', ['fp64', 'fp32c'])
def test_wstack_workflow_unnormalised_matches_reference(arl, golden, precision):
    """invert_list_serial_workflow(context='wstack', normalize=False): the
    reference's own result (slice images unnormalised, weighted by each
    slice's sumwt, divided by the total)."""
    d = golden('ref_wstack.npz')
    im, gcf, cf, vis = _case(arl, d)
    K = int(d['K'])
    (dirty, sumwt), = arl.imaging.invert_list_serial_workflow([vis], [im], context='wstack', vis_slices=K,
                                                               normalize=False, gcfcf=[(gcf, cf)],
                                                               precision=precision)
    assert_image(dirty.data, d['dirty_nonorm'], d['gcf'], precision)
    assert numpy.allclose(sumwt, d['sumwt_nonorm'], rtol=1e-12 if precision == 'fp64' else 1e-6)


@pytest.mark.parametrize('precision', ['fp64', 'fp32c'])
def test_reference_workflow_calls_replayed(arl, golden, precision):
    """The reference's serial 'wstack' workflows (invert normalised, invert of the
    PSF unnormalised, predict) had every call into their imaging context
    recorded (tests/golden/ref_workflow_trace.npz).  Replayed through this
    package's own imaging_contexts()['wstack']: its vis_iterator yields the
    same row masks, and each invert / predict called with the workflow's
    arguments on those rows returns the reference's (image, sumwt) and rows;
    the workflow's assembly of those results gives the reference's dirty
    image and predicted visibilities."""
    d = golden('ref_wstack.npz')
    t = golden('ref_workflow_trace.npz')
    im, gcf, cf, vis = _case(arl, d)
    K = int(d['K'])
    ctx = arl.imaging_contexts()['wstack']
    masks = [numpy.asarray(m) for m in ctx['vis_iterator'](vis, K)]
    assert all(numpy.array_equal(m, t['masks'][k]) for k, m in enumerate(masks))
    assert numpy.array_equal(t['masks'][:K], t['masks'][K:2 * K])
    acc = numpy.zeros_like(t['dirty'])
    total = numpy.zeros_like(t['sumwt'])
    for k in range(2 * K):
        row_vis = arl.data_models.create_visibility_from_rows(vis, t['masks'][k])
        dopsf, normalize = (bool(x) for x in t['inv_kw'][k])
        img, sw = ctx['invert'](row_vis, im, dopsf=dopsf, normalize=normalize, context='wstack', gcfcf=(gcf, cf),
                                precision=precision)
        assert_image(img.data, t['inv_img'][k], d['gcf'], precision)
        assert numpy.allclose(sw, t['inv_sw'][k], rtol=1e-12 if precision == 'fp64' else 1e-6)
        if k < K:
            acc += sw[:, :, None, None] * img.data
            total += sw
    dirty = arl.normalize_sumwt(arl.create_image_from_array(acc, im.wcs, im.polarisation_frame), total)
    assert_image(dirty.data, t['dirty'], d['gcf'], precision)
    model = arl.create_image_from_array(d['model'], im.wcs, im.polarisation_frame)
    pv = numpy.zeros_like(t['predict'])
    start = numpy.concatenate([[0], numpy.cumsum(t['pred_len'])])
    for j in range(K):
        mask = t['masks'][2 * K + j]
        row_vis = arl.data_models.create_visibility_from_rows(vis, mask)
        out = ctx['predict'](row_vis, model, context='wstack', gcfcf=(gcf, cf), precision=precision)
        assert rel(out.vis, t['pred'][start[j]:start[j + 1]]) < TOL[precision]
        pv[mask] = out.vis
    assert rel(pv, t['predict']) < TOL[precision]


@pytest.mark.parametrize('precision', ['fp64', 'fp32c'])
def test_wstack_single_matches_oracle(arl, oracle, golden, precision):
    d = golden('ref_wstack.npz')
    im, gcf, cf, vis = _case(arl, d)
    N, cell = int(d['N']), float(d['cell'])
    img = oracle.image_geometry(N, cell)
    cax = oracle.cf_axes(img, int(d['O']), int(d['S']))
    ocf = oracle.create_pswf_cf(1, 1, N, N, int(d['O']), int(d['S']))[1]
    ogcf = oracle.pswf_gcf(N)[None, None]
    # one slice: all rows, w-beam of their mean w
    uvw = d['uvw'].copy()
    wav = numpy.average(uvw[:, 2])
    uvw[:, 2] -= wav
    ref, sw = oracle.invert_2d(uvw, d['frequency'], d['vis'], d['wt'], img, ogcf, ocf, cax)
    wb = oracle.w_term_image(N, cell, wav)
    want = wb.real * ref.real - wb.imag * ref.imag
    got, gsw = arl.imaging.invert_wstack_single(vis, im, False, gcfcf=(gcf, cf), precision=precision)
    assert_image(got.data, want, ogcf, precision)
    model = arl.create_image_from_array(d['model'], im.wcs, im.polarisation_frame)
    vr = oracle.predict_2d(uvw, d['frequency'], wb.real * d['model'], img, ogcf, ocf, cax)
    vi = oracle.predict_2d(uvw, d['frequency'], wb.imag * d['model'], img, ogcf, ocf, cax)
    pv = arl.imaging.predict_wstack_single(vis, model, gcfcf=(gcf, cf), precision=precision)
    assert rel(pv.vis, vr - 1j * vi) < TOL[precision]


@pytest.mark.parametrize('N', [96, 128])
def test_wstack_many_slices_vs_oracle(arl, oracle, N):
    """12 slices, 2 channels imaged together (MFS through one wide image channel).
    N = 96 takes the complex128 cuFFT transforms on both precisions, N = 128 the
    double-single transform on FP32C."""
    rng = numpy.random.default_rng(8)
    cell, O, S, K, n = 6e-3 * 96 / N, 8, 8, 12, 4000
    im = arl.create_image(npixel=N, cellsize=cell, frequency=numpy.array([1.05e8]), channel_bandwidth=numpy.array([1e8]),
                          phasecentre=arl.PhaseCentre(0.0, -45.0))
    gcf, cf = arl.create_pswf_convolutionfunction(im, oversampling=O, support=S)
    lim = (N // 2 - S // 2 - 2) / (N * cell)
    uvw = numpy.stack([rng.uniform(-lim, lim, n), rng.uniform(-lim, lim, n), rng.uniform(-300, 300, n)], axis=1)
    freq = rng.choice([1.0e8, 1.1e8], n)
    v = rng.normal(size=(n, 1)) + 1j * rng.normal(size=(n, 1))
    wt = numpy.ones((n, 1))
    vis = arl.Visibility(uvw=uvw, frequency=freq, vis=v, weight=wt, imaging_weight=wt)
    vis.phasecentre = arl.PhaseCentre(0.0, -45.0)
    img = oracle.image_geometry(N, cell, 1, 1, 1.05e8, 1e8)
    cax = oracle.cf_axes(img, O, S)
    ocf = oracle.create_pswf_cf(1, 1, N, N, O, S)[1]
    want, wsw = oracle.invert_wstack(uvw, freq, v, wt, img, oracle.pswf_gcf(N)[None, None], ocf, cax, K, cell)
    for p in ('fp64', 'fp32c'):
        got, sw = arl.imaging.invert_wstack(vis, im, K, gcfcf=(gcf, cf), precision=p)
        assert_image(got.data, want, oracle.pswf_gcf(N), p)
        assert numpy.allclose(sw, wsw, rtol=1e-12 if p == 'fp64' else 1e-6)


@pytest.mark.parametrize('precision', ['fp64', 'fp32c'])
def test_wstack_plan_at_slice_ties_vs_oracle(arl, oracle, precision):
    """Rows on the half-way points between w slices, and one ulp either side:
    w = 0 with an even slice count (every row of a coplanar array at transit
    sits there) and the other slice boundaries.  The planned gridder must put
    each row in the slice NumPy's round-half-even of world2pix0 picks; the grid
    is compared cell by cell with the oracle's."""
    rng = numpy.random.default_rng(21)
    N, cell, O, S, K, wmax = 128, 4.5e-3, 8, 8, 8, 250.0
    im = arl.create_image(npixel=N, cellsize=cell, frequency=numpy.array([1e8]), channel_bandwidth=numpy.array([1e6]),
                          phasecentre=arl.PhaseCentre(0.0, -45.0))
    gcf, cf = arl.create_pswf_convolutionfunction(im, oversampling=O, support=S)
    step = 2.0 * wmax / (K - 1)
    ties = numpy.concatenate([[0.0, 1e-13, -1e-13, 5e-324, -5e-324], -wmax + (numpy.arange(K - 1) + 0.5) * step])
    ties = numpy.concatenate([ties, numpy.nextafter(ties, numpy.inf), numpy.nextafter(ties, -numpy.inf)])
    w = numpy.concatenate([[wmax, -wmax], numpy.repeat(ties, 60), rng.uniform(-wmax, wmax, 1000)])
    n = w.size
    lim = (N // 2 - S // 2 - 2) / (N * cell)
    uvw = numpy.stack([rng.uniform(-lim, lim, n), rng.uniform(-lim, lim, n), w], axis=1)
    freq = numpy.full(n, 1e8)
    v = rng.normal(size=(n, 1)) + 1j * rng.normal(size=(n, 1))
    wt = numpy.ones((n, 1))
    dev = torch.device('cuda')
    dvis = arl.DeviceVisibility(torch.as_tensor(uvw, device=dev), torch.as_tensor(freq, device=dev),
                                torch.as_tensor(v, device=dev).to(arl.device.CDTYPE[precision]),
                                torch.ones((n, 1), dtype=arl.device.RDTYPE[precision], device=dev))
    imager = arl.WStackImager(dvis, im, K, gcfcf=(gcf, cf), precision=precision)
    assert imager.w_axis == (-wmax, 1.0, step)
    imager.grid()
    img = oracle.image_geometry(N, cell)
    gax = oracle.grid_axes(img, nw=K)
    gax['w'] = imager.w_axis
    cax = oracle.cf_axes(img, O, S)
    _, ocf = oracle.create_pswf_cf(1, 1, 8, 8, O, S)
    maps = oracle.convolution_mapping(uvw, freq, gax, cax)
    assert numpy.all((maps[4] >= 0) & (maps[4] < K))
    cells, vals, sw = oracle.grid_sparse(v, wt, maps, ocf, gax['shape'])
    flat = imager.grid_t.reshape(-1)
    got = flat[torch.as_tensor(cells, device=dev)].to(torch.complex128).cpu().numpy()
    assert rel(got, vals) < TOL[precision]
    total = float((flat.to(torch.complex128).abs() ** 2).sum())
    assert abs(total - float(numpy.sum(numpy.abs(got) ** 2))) <= 1e-9 * total
