"""The benchmark workloads other than the bench's own (C2) as parity cases.

C1  plain 2-D invert_2d / predict_2d at full size against the oracle.
C3  batched w-stacking (4 polarisations, 64 flagged channels summed, 20
    slices, 4096^2) at full size: FP32C against the FP64 GPU path, exact weight
    sums, bit-exact row mapping against the oracle over every row, the CUDA
    graph of the whole pipeline against eager execution, and the gridder and
    degridder against the oracle on a seeded row subsample.
C5  ~1e8 rows onto 8192^2 with 32 w-stack slices: the invert / predict round
    trip in FP32C against FP64, exact weight sums, bit-exact mapping over every
    row, and the FP64 oracle on a seeded 1e6-row subsample.
(C4, the gain solve, is covered in test_gpu_gainsolve.py.)

Tolerances are the parity tests' (helpers.py): FP32C 1e-5, FP64 1e-12 on
grids and visibilities, the image rule for grid-corrected images.
"""
import ctypes

import numpy
import pytest
import torch

from helpers import assert_image, rel

pytestmark = pytest.mark.gpu

TOL = {'fp64': 1e-12, 'fp32c': 1e-5}


@pytest.fixture(scope='module', autouse=True)
def need_cuda(arl):
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    arl._native.load()


def _free():
    torch.cuda.synchronize()
    torch.cuda.empty_cache()


def oracle_geometry(oracle, w):
    return oracle.image_geometry(w['npixel'], w['cellsize'], len(w['image_frequency']), w['npol'],
                                 w['image_frequency'][0], w['image_bandwidth'])


def device_rows(arl, w, precision, sel=None):
    dev = torch.device('cuda')
    uvw, f = w['uvw'], w['frequency']
    vis = w['vis']
    if sel is not None:
        uvw, f = uvw[sel], f[sel]
        vis = vis[torch.as_tensor(sel, device=vis.device)]
    n = uvw.shape[0]
    return arl.DeviceVisibility(torch.as_tensor(uvw, device=dev), torch.as_tensor(f, device=dev),
                                vis.to(device=dev, dtype=arl.device.CDTYPE[precision]),
                                torch.ones((n, w['npol']), dtype=arl.device.RDTYPE[precision], device=dev))


def gpu_mapping(arl, imager):
    """The library's row mapping (C ABI) for the imager's rows and grid."""
    nat = arl._native
    n = imager.n
    outs = [torch.empty(n, dtype=torch.int32, device=imager.device) for _ in range(7)]
    nbad = ctypes.c_int64()
    nat.call('arlgpu_convolution_mapping', nat.ptr(imager.uvw), nat.ptr(imager.f), n, ctypes.byref(imager.gd),
             ctypes.byref(imager.cd), *[nat.ptr(o) for o in outs], ctypes.byref(nbad), nat.stream_ptr())
    return outs, nbad.value


def assert_mapping_bit_exact(arl, oracle, imager, w, img, chunk=10_000_000):
    """Every row's (pu, pu_off, pv, pv_off, pwg, pwc, pfreq) equals the oracle's."""
    outs, nbad = gpu_mapping(arl, imager)
    assert nbad == 0
    gax = oracle.grid_axes(img, nw=imager.vis_slices)
    gax['w'] = imager.w_axis
    cax = oracle.cf_axes(img, w['oversampling'], w['support'])
    for s in range(0, imager.n, chunk):
        e = min(s + chunk, imager.n)
        ref = oracle.convolution_mapping(w['uvw'][s:e], w['frequency'][s:e], gax, cax)
        for k, (g, r) in enumerate(zip(outs, ref)):
            assert numpy.array_equal(g[s:e].cpu().numpy().astype(numpy.int64), r), (k, s)
    del outs


def subsample_oracle(arl, oracle, w, im, gcfcf, nsub, seed, model):
    """Grid and degrid of a seeded row subsample through the w-stack imager (both
    precisions) against the oracle: the grid over the cells the rows touch (and
    nothing anywhere else), the degridded rows from the same grid windows."""
    gcf, cf = gcfcf
    rng = numpy.random.default_rng(seed)
    n = w['uvw'].shape[0]
    sel = numpy.sort(rng.choice(n, min(nsub, n), replace=False))
    img = oracle_geometry(oracle, w)
    _, ocf = oracle.create_pswf_cf(1, w['npol'], 8, 8, w['oversampling'], w['support'])
    assert rel(cf.data[0:1], ocf) < 1e-14
    vis64 = w['vis'][torch.as_tensor(sel, device=w['vis'].device)].cpu().numpy()
    wt = numpy.ones(vis64.shape)
    for precision in ('fp64', 'fp32c'):
        dvis = device_rows(arl, w, precision, sel)
        imager = arl.WStackImager(dvis, im, w['vis_slices'], gcfcf=gcfcf, precision=precision)
        imager.grid()
        gax = oracle.grid_axes(img, nw=imager.vis_slices)
        gax['w'] = imager.w_axis
        cax = oracle.cf_axes(img, w['oversampling'], w['support'])
        maps = oracle.convolution_mapping(w['uvw'][sel], w['frequency'][sel], gax, cax)
        assert numpy.all(oracle.rows_in_grid(maps, gax['shape'], ocf.shape))
        cells, vals, sw = oracle.grid_sparse(vis64, wt, maps, ocf, gax['shape'])
        flat = imager.grid_t.reshape(-1)
        got = flat[torch.as_tensor(cells, device=flat.device)].to(torch.complex128).cpu().numpy()
        assert rel(got, vals) < TOL[precision], precision
        total = float((flat.to(torch.complex128).abs() ** 2).sum())
        assert abs(total - float(numpy.sum(numpy.abs(got) ** 2))) <= 1e-9 * total
        assert numpy.array_equal(imager.sumwt.cpu().numpy(), sw)
        out = imager.predict(model)
        idx = torch.as_tensor(oracle.window_index(maps, gax['shape'], w['support']), device=flat.device)
        win = imager.grid_t.reshape(-1)[idx].to(torch.complex128).cpu().numpy()
        ref = oracle.degrid_windows(win, maps, ocf)
        assert rel(out.to(torch.complex128).cpu().numpy(), ref) < TOL[precision], precision
        del imager, dvis, idx, flat
        _free()


# ---------------------------------------------------------------------------
# C1: plain 2-D imaging, full size, against the oracle
# ---------------------------------------------------------------------------
@pytest.mark.parametrize('precision', ['fp64', 'fp32c'])
def test_c1_invert_predict_vs_oracle(arl, oracle, precision):
    sim = arl.simulation
    w = sim.make_workload('C1')
    im = sim.workload_image(arl, w)
    gcf, cf = arl.create_pswf_convolutionfunction(im, oversampling=w['oversampling'], support=w['support'])
    n = w['uvw'].shape[0]
    vis64 = w['vis'].cpu().numpy()
    wt = numpy.ones((n, 1))
    vis = arl.Visibility(uvw=w['uvw'], frequency=w['frequency'], vis=vis64, weight=wt, imaging_weight=wt,
                         polarisation_frame=arl.PolarisationFrame('stokesI'))
    vis.phasecentre = arl.PhaseCentre(0.0, -45.0)
    img = oracle_geometry(oracle, w)
    ogcf, ocf = oracle.create_pswf_cf(1, 1, w['npixel'], w['npixel'], w['oversampling'], w['support'])
    cax = oracle.cf_axes(img, w['oversampling'], w['support'])
    dirty, sw = arl.invert_2d(vis, im, gcfcf=(gcf, cf), precision=precision)
    ref, rsw = oracle.invert_2d(w['uvw'], w['frequency'], vis64, wt, img, ogcf, ocf, cax)
    assert_image(dirty.data, ref.real, ogcf, precision)
    assert numpy.array_equal(sw, rsw)
    model = numpy.zeros((1, 1, w['npixel'], w['npixel']))
    rng = numpy.random.default_rng(5)
    c = w['npixel'] // 2
    model[0, 0, rng.integers(c - 100, c + 100, 20), rng.integers(c - 100, c + 100, 20)] = rng.uniform(0.1, 5, 20)
    mim = arl.create_image_from_array(model, im.wcs, im.polarisation_frame)
    pv = arl.predict_2d(vis, mim, gcfcf=(gcf, cf), precision=precision)
    rv = oracle.predict_2d(w['uvw'], w['frequency'], model, img, ogcf, ocf, cax)
    assert rel(pv.vis, rv) < (1e-10 if precision == 'fp64' else 1e-5)


# ---------------------------------------------------------------------------
# C3: batched w-stacking with 4 polarisations and flagged channels
# ---------------------------------------------------------------------------
@pytest.fixture(scope='module')
def c3(arl):
    w = arl.simulation.make_workload('C3', device=torch.device('cuda'))
    im = arl.simulation.workload_image(arl, w)
    gcfcf = arl.create_pswf_convolutionfunction(im, oversampling=w['oversampling'], support=w['support'])
    yield w, im, gcfcf
    del w
    _free()


def _model(w, seed):
    rng = numpy.random.default_rng(seed)
    N = w['npixel']
    m = numpy.zeros((1, w['npol'], N, N))
    k = 40
    ys = rng.integers(N // 2 - N // 8, N // 2 + N // 8, k)
    xs = rng.integers(N // 2 - N // 8, N // 2 + N // 8, k)
    for p in range(w['npol']):
        m[0, p, ys, xs] = rng.uniform(0.1, 5.0, k) * (1.0 if p in (0, w['npol'] - 1) else 0.1)
    return m


def test_c3_full_size(arl, oracle, c3):
    w, im, gcfcf = c3
    n = w['uvw'].shape[0]
    model = _model(w, 31)
    res = {}
    for precision in ('fp64', 'fp32c'):
        dvis = device_rows(arl, w, precision)
        imager = arl.WStackImager(dvis, im, w['vis_slices'], gcfcf=gcfcf, precision=precision)
        if precision == 'fp64':
            assert_mapping_bit_exact(arl, oracle, imager, w, oracle_geometry(oracle, w))
        image, sumwt = imager.invert()
        image, sumwt = image.cpu().numpy(), sumwt.cpu().numpy()
        out = imager.predict(model).to(torch.complex128).cpu().numpy()
        if precision == 'fp32c':
            # The whole invert (plan + grid + transforms + combine) as one CUDA
            # graph, replayed on the same rows, and then on new rows.
            imager.capture('invert')
            g_image, g_sumwt = imager.replay('invert')
            assert_image(g_image.cpu().numpy(), image, gcfcf[0].data, 'fp32c')
            assert numpy.array_equal(g_sumwt.cpu().numpy(), sumwt)
            imager.load_rows(vis=(2.0 * dvis.vis))
            g2, _ = imager.replay('invert')
            assert_image(g2.cpu().numpy(), 2.0 * image, gcfcf[0].data, 'fp32c')
            imager.load_rows(weight=2.0 * dvis.imaging_weight)
            g3, sw2 = imager.replay('invert')
            assert numpy.array_equal(sw2.cpu().numpy(), 2.0 * sumwt)
            assert_image(g3.cpu().numpy(), 2.0 * image, gcfcf[0].data, 'fp32c')
        res[precision] = (image, sumwt, out)
        del imager, dvis
        _free()
    assert numpy.array_equal(res['fp64'][1], numpy.full((1, 4), float(n)))
    assert numpy.array_equal(res['fp32c'][1], res['fp64'][1])
    assert_image(res['fp32c'][0], res['fp64'][0], gcfcf[0].data, 'fp32c')
    assert rel(res['fp32c'][2], res['fp64'][2]) < 1e-5


def test_c3_subsample_vs_oracle(arl, oracle, c3):
    w, im, gcfcf = c3
    subsample_oracle(arl, oracle, w, im, gcfcf, 200_000, 33, _model(w, 32))


# ---------------------------------------------------------------------------
# C5: ~1e8 rows, 8192^2 grid, 32 w-stack slices
# ---------------------------------------------------------------------------
def test_c5_round_trip_and_subsample(arl, oracle):
    sim = arl.simulation
    w = sim.make_workload('C5', device=torch.device('cuda'))
    n = w['uvw'].shape[0]
    assert n > 9e7
    im = sim.workload_image(arl, w)
    gcfcf = arl.create_pswf_convolutionfunction(im, oversampling=w['oversampling'], support=w['support'])
    model = _model(w, 56)
    res = {}
    for precision in ('fp64', 'fp32c'):
        dvis = device_rows(arl, w, precision)
        imager = arl.WStackImager(dvis, im, w['vis_slices'], gcfcf=gcfcf, precision=precision)
        if precision == 'fp64':
            assert_mapping_bit_exact(arl, oracle, imager, w, oracle_geometry(oracle, w))
        image, sumwt = imager.invert()
        r = [image.cpu().numpy(), sumwt.cpu().numpy()]
        # round trip: predict the model onto the rows, then image those rows
        out = imager.predict(model)
        r.append(out.to(torch.complex128).cpu().numpy())
        imager.load_rows(vis=out)
        image2, _ = imager.invert()
        r.append(image2.cpu().numpy())
        res[precision] = r
        del imager, dvis, out, image2
        _free()
    assert numpy.array_equal(res['fp64'][1], numpy.full((1, 1), float(n)))
    assert numpy.array_equal(res['fp32c'][1], res['fp64'][1])
    assert_image(res['fp32c'][0], res['fp64'][0], gcfcf[0].data, 'fp32c')
    assert rel(res['fp32c'][2], res['fp64'][2]) < 1e-5
    assert_image(res['fp32c'][3], res['fp64'][3], gcfcf[0].data, 'fp32c')
    del res
    _free()
    subsample_oracle(arl, oracle, w, im, gcfcf, 1_000_000, 55, model)
