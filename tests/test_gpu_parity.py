"""Parity of the CUDA path with the oracle and with the reference's golden
outputs.  Every call goes through libarlgpu.so (C ABI) via the package.

Tolerances (max-norm error / max-norm of the reference result):
  FP64 path   1e-12 (grid, degrid, kernels); 1e-10 for outputs that pass
              through an FFT (cuFFT and NumPy's pocketfft sum in different
              orders; measured differences are ~2e-12)
  FP32C path  1e-5  (the ≤1e-5 relative-error target for complex64 storage
              with compensated FP32 accumulation)
Integer index work (convolution_mapping) must be bit-identical.
"""
import numpy
import pytest
import torch

from helpers import assert_image

pytestmark = pytest.mark.gpu

TOL = {'fp64': 1e-12, 'fp32c': 1e-5}
TOLF = {'fp64': 1e-10, 'fp32c': 1e-5}
# sumwt is summed in FP64 on both paths, but FP32C weights are float32 copies
TOLW = {'fp64': 1e-12, 'fp32c': 1e-6}


def rel(a, b):
    a = numpy.asarray(a)
    b = numpy.asarray(b)
    return float(numpy.max(numpy.abs(a - b)) / max(numpy.max(numpy.abs(b)), 1e-300))


@pytest.fixture(scope='module', autouse=True)
def need_cuda(arl):
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    arl._native.load()


def make_image(arl, N, cell, freqs, dfreq, polframe='stokesI'):
    return arl.create_image(npixel=N, cellsize=cell, frequency=numpy.asarray(freqs, float),
                            channel_bandwidth=numpy.array([dfreq]), polarisation_frame=arl.PolarisationFrame(polframe),
                            phasecentre=arl.PhaseCentre(0.0, -45.0))


def make_vis(arl, uvw, freq, vis, wt, polframe='stokesI'):
    v = arl.Visibility(uvw=uvw, frequency=freq, vis=vis, weight=wt, imaging_weight=wt,
                       polarisation_frame=arl.PolarisationFrame(polframe))
    v.phasecentre = arl.PhaseCentre(0.0, -45.0)
    return v


# ---------------------------------------------------------------------------
# Mapping: bit-exact indices
# ---------------------------------------------------------------------------
def test_mapping_matches_golden(arl, golden):
    d = golden('ref_2d_pswf.npz')
    im = make_image(arl, int(d['N']), float(d['cell']), [1e8], 1e6)
    gd = arl.create_griddata_from_image(im)
    _, cf = arl.create_pswf_convolutionfunction(im, oversampling=int(d['O']), support=int(d['S']))
    vis = make_vis(arl, d['uvw'], d['frequency'], d['vis'], d['wt'])
    m = arl.convolution_mapping(vis, gd, cf)
    for got, want in zip((m[0], m[1], m[2], m[3], m[4], m[6], m[8]), d['maps']):
        assert numpy.array_equal(got, want)


@pytest.mark.parametrize('N,cell,O', [(512, 1e-3, 8), (1024, 3e-4, 16), (256, 2e-3, 6)])
def test_mapping_bit_exact_at_rounding_boundaries(arl, oracle, N, cell, O):
    """Rows placed exactly on (and one ulp either side of) the half-pixel and
    sub-pixel boundaries where round-half-even / floor decide the index (power
    of two oversampling takes the X = P * O path, 6 the one-FMA path)."""
    S = 8
    im = make_image(arl, N, cell, [1e8], 1e6)
    gd = arl.create_griddata_from_image(im)
    cf = arl.create_convolutionfunction_from_image(im, oversampling=O, support=S)
    du = gd.grid_wcs.wcs.cdelt[0]
    rng = numpy.random.default_rng(5)
    k = rng.integers(-N // 3, N // 3, 4000).astype(float)
    base = numpy.concatenate([(k + 0.5) * du, (k + 0.5 + rng.integers(0, O, 4000) / O) * du,
                              rng.uniform(-N // 3, N // 3, 4000) * du])
    u = numpy.concatenate([base, numpy.nextafter(base, numpy.inf), numpy.nextafter(base, -numpy.inf)])
    n = u.size
    uvw = numpy.stack([u, u[::-1], rng.uniform(-100, 100, n)], axis=1)
    freq = numpy.full(n, 1e8)
    vis = make_vis(arl, uvw, freq, numpy.zeros((n, 1)), numpy.ones((n, 1)))
    img = oracle.image_geometry(N, cell)
    gax, cax = oracle.grid_axes(img), oracle.cf_axes(img, O, S)
    # As built (the one-FMA fast path applies), then with the cf's sub-pixel
    # cdelt nudged by one ulp (the library must take the exact path).
    for nudge in (False, True):
        if nudge:
            for ax, key in ((2, 'du'), (3, 'dv')):
                cf.grid_wcs.wcs.cdelt[ax] = numpy.nextafter(cf.grid_wcs.wcs.cdelt[ax], numpy.inf)
                cax[key] = (cax[key][0], cax[key][1], float(cf.grid_wcs.wcs.cdelt[ax]))
        got = arl.convolution_mapping(vis, gd, cf)
        want = oracle.convolution_mapping(uvw, freq, gax, cax)
        for g, w in zip((got[0], got[1], got[2], got[3], got[4], got[6], got[8]), want):
            assert numpy.array_equal(g, w)


# ---------------------------------------------------------------------------
# Grid / degrid / FFT against the reference's golden outputs
# ---------------------------------------------------------------------------
@pytest.mark.parametrize('precision', ['fp64', 'fp32c'])
def test_golden_2d_pswf(arl, golden, precision):
    d = golden('ref_2d_pswf.npz')
    tol = TOL[precision]
    im = make_image(arl, int(d['N']), float(d['cell']), [1e8], 1e6)
    gcf, cf = arl.create_pswf_convolutionfunction(im, oversampling=int(d['O']), support=int(d['S']))
    assert rel(cf.data, d['cf']) < 1e-14 and rel(gcf.data, d['gcf']) < 1e-14
    vis = make_vis(arl, d['uvw'], d['frequency'], d['vis'], d['wt'])
    gd = arl.create_griddata_from_image(im)
    gd, sumwt = arl.grid_visibility_to_griddata(vis, gd, cf, precision=precision)
    assert rel(gd.data, d['grid']) < tol
    assert rel(sumwt, d['sumwt']) < TOLW[precision]
    re, imag = arl.fft_griddata_to_image(gd, gcf, imaginary=True, precision=precision)
    tolf = TOLF[precision]
    assert_image(re.data, d['img_re'], d['gcf'], precision)
    assert_image(imag.data + 1j * d['img_re'], d['img_im'] + 1j * d['img_re'], d['gcf'], precision)
    mim = arl.create_image_from_array(d['model'], im.wcs, im.polarisation_frame)
    gd2 = arl.fft_image_to_griddata(mim, arl.create_griddata_from_image(im), gcf, precision=precision)
    assert rel(gd2.data, d['grid_model']) < tolf
    gm = arl.create_griddata_from_image(im)
    gm.data[...] = d['grid_model']
    newvis = arl.degrid_visibility_from_griddata(vis, gm, cf, precision=precision)
    assert rel(newvis.vis, d['degrid']) < tol
    dirty, sw = arl.invert_2d(vis, im, gcfcf=(gcf, cf), precision=precision)
    assert_image(dirty.data, d['dirty'], d['gcf'], precision)
    assert rel(sw, d['sumwt_dirty']) < TOLW[precision]
    psf, _ = arl.invert_2d(vis, im, dopsf=True, gcfcf=(gcf, cf), precision=precision)
    assert_image(psf.data, d['psf'], d['gcf'], precision)
    pv = arl.predict_2d(vis, mim, gcfcf=(gcf, cf), precision=precision)
    assert rel(pv.vis, d['predict']) < tolf


def test_fp32c_edge_error_is_storage_rounding(arl, golden):
    """Where the whole-image FP32C error comes from, on the golden 2-D PSWF
    case (128^2, grid correction up to 6.2e4 at the corners): the FP64 path
    given the same taps rounded to complex64, or its own grid rounded to
    complex64 before the transform, shows the same edge error as the FP32C
    path (each ~2e-4 of the image peak), while rounding the visibilities and
    weights to FP32 costs ~4e-8.  So the edge error is the FP32 storage of the
    kernel table and of the grid cells, amplified by the grid correction; the
    gridder's arithmetic and the double-single transform add nothing
    visible, and no FP32-storage path meets 1e-5 over the whole field."""
    from helpers import image_errors
    d = golden('ref_2d_pswf.npz')
    im = make_image(arl, int(d['N']), float(d['cell']), [1e8], 1e6)
    gcf, cf = arl.create_pswf_convolutionfunction(im, oversampling=int(d['O']), support=int(d['S']))

    def image(vis, wt, cfx, grid_prec, round_grid=False):
        gd = arl.create_griddata_from_image(im)
        gd, _ = arl.grid_visibility_to_griddata(make_vis(arl, d['uvw'], d['frequency'], vis, wt), gd, cfx,
                                                precision=grid_prec)
        g = numpy.asarray(gd.data)
        gd.data = (g.astype(numpy.complex64) if round_grid else g).astype(numpy.complex128)
        re = arl.fft_griddata_to_image(gd, gcf, precision='fp64' if grid_prec == 'fp64' else 'fp32c')
        return image_errors(re.data, d['img_re'], d['gcf'])

    e32, i32 = image(d['vis'], d['wt'], cf, 'fp32c')
    cf32 = arl.create_pswf_convolutionfunction(im, oversampling=int(d['O']), support=int(d['S']))[1]
    cf32.data = cf.data.astype(numpy.complex64).astype(numpy.complex128)
    e_taps, _ = image(d['vis'], d['wt'], cf32, 'fp64')
    e_grid, _ = image(d['vis'], d['wt'], cf, 'fp64', round_grid=True)
    e_vis, _ = image(d['vis'].astype(numpy.complex64).astype(numpy.complex128),
                     d['wt'].astype(numpy.float32).astype(numpy.float64), cf, 'fp64')
    assert i32 < 1e-5
    assert e_vis < 1e-6
    assert min(e_taps, e_grid) > 1e-5
    assert e32 < 3.0 * max(e_taps, e_grid), (e32, e_taps, e_grid)


@pytest.mark.parametrize('precision', ['fp64', 'fp32c'])
def test_golden_wproj_2chan_2pol(arl, golden, precision):
    d = golden('ref_wproj_2chan_2pol.npz')
    tol = TOL[precision]
    im = make_image(arl, int(d['N']), float(d['cell']), d['freqs'], float(d['dfreq']), 'stokesIQ')
    gcf, cf = arl.create_awterm_convolutionfunction(im, nw=int(d['nw']), wstep=float(d['wstep']),
                                                    oversampling=int(d['O']), support=int(d['S']), maxsupport=64)
    assert rel(cf.data, d['cf']) < 1e-12 and rel(gcf.data, d['gcf']) < 1e-14
    vis = make_vis(arl, d['uvw'], d['frequency'], d['vis'], d['wt'], 'stokesIQ')
    gd = arl.create_griddata_from_image(im)
    gd, sumwt = arl.grid_visibility_to_griddata(vis, gd, cf, precision=precision)
    assert rel(gd.data, d['grid']) < tol and rel(sumwt, d['sumwt']) < TOLW[precision]
    re = arl.fft_griddata_to_image(gd, gcf, precision=precision)
    assert_image(re.data, d['img_re'], d['gcf'], precision)
    gd.data[...] = d['rgrid']
    newvis = arl.degrid_visibility_from_griddata(vis, gd, cf, precision=precision)
    assert rel(newvis.vis, d['degrid']) < tol


def test_kernels_match_reference(arl, golden):
    d = golden('ref_kernels.npz')
    im = make_image(arl, 512, 0.0005, [1e8], 1e6)
    _, cf8 = arl.create_pswf_convolutionfunction(im, oversampling=8, support=6)
    _, cf1 = arl.create_pswf_convolutionfunction(im, oversampling=1, support=6)
    assert rel(cf8.data[0, 0, 0], d['pswf8']) < 1e-14 and rel(cf1.data[0, 0, 0], d['pswf1']) < 1e-14
    gcf, cfw = arl.create_awterm_convolutionfunction(im, nw=9, wstep=8.0, oversampling=8, support=16)
    assert rel(cfw.data[0, 0], d['wker']) < 1e-12 and rel(gcf.data[0, 0], d['gcf']) < 1e-14
    bb = arl.calculate_bounding_box_convolutionfunction(cfw, 1e-3)
    assert numpy.array_equal(numpy.array([[b[0], *b[1], *b[2]] for b in bb]), d['bbox'])


def test_wkernels_without_aaf_match_reference(arl, golden):
    """create_awterm_convolutionfunction(use_aaf=False): the w-screens without
    the anti-aliasing function's inverse, and an all-ones gcf."""
    d = golden('ref_wkernels_noaaf.npz')
    im = make_image(arl, 256, 0.001, [1e8], 1e6)
    gcf, cfw = arl.create_awterm_convolutionfunction(im, nw=5, wstep=20.0, oversampling=4, support=8, use_aaf=False,
                                                     maxsupport=128)
    assert rel(cfw.data[0, 0], d['wker']) < 1e-12
    assert numpy.array_equal(gcf.data[0, 0], d['gcf'])


# ---------------------------------------------------------------------------
# Oracle parity on cases the fixtures do not cover
# ---------------------------------------------------------------------------
def _random_case(arl, oracle, rng, N, cell, O, S, nvis, nchan=1, npol=1, nz=1, zstep=1e15, distinct_chan=False,
                 lim_px=None):
    """Random rows, weights and cf taps; uv uniform over the grid, or within
    +/- lim_px pixels of its centre."""
    freqs = 1e8 + 1e7 * numpy.arange(nchan)
    pf = {1: 'stokesI', 2: 'stokesIQ', 4: 'stokesIQUV'}[npol]
    im = make_image(arl, N, cell, freqs, 1e7, pf)
    du = abs(1.0 / (N * cell))
    lim = ((N // 2 - S // 2 - 2) if lim_px is None else lim_px) * du
    uvw = numpy.stack([rng.uniform(-lim, lim, nvis), rng.uniform(-lim, lim, nvis),
                       rng.uniform(-0.45 * nz * zstep, 0.45 * nz * zstep, nvis) if nz > 1 else
                       rng.uniform(-50, 50, nvis)], axis=1)
    freq = rng.choice(freqs, nvis)
    visd = rng.normal(size=(nvis, npol)) + 1j * rng.normal(size=(nvis, npol))
    wt = rng.uniform(0.5, 2.0, size=(nvis, npol))
    if nz == 1:
        zstep = 1e15
    cf = arl.create_convolutionfunction_from_image(im, nz=nz, zstep=zstep, oversampling=O, support=S)
    base = rng.normal(size=(nz, O, O, S, S)) + 1j * rng.normal(size=(nz, O, O, S, S))
    data = numpy.broadcast_to(base[None, None], cf.data.shape).copy()
    if distinct_chan:
        for c in range(nchan):
            for p in range(npol):
                data[c, p] *= (1.0 + 0.25 * c) * (1.0 - 0.1 * p)
    cf.data = data
    vis = make_vis(arl, uvw, freq, visd, wt, pf)
    img = oracle.image_geometry(N, cell, nchan, npol, 1e8, 1e7)
    gax = oracle.grid_axes(img)
    cax = oracle.cf_axes(img, O, S, nz=nz, zstep=zstep)
    maps = oracle.convolution_mapping(uvw, freq, gax, cax)
    return im, cf, vis, maps, gax


@pytest.mark.parametrize('precision', ['fp64', 'fp32c'])
@pytest.mark.parametrize('N,O,S,npol,nchan,nz,distinct', [
    (128, 8, 6, 1, 1, 1, False),      # ARL's default support 6
    (128, 128, 6, 1, 1, 1, False),    # ARL invert_2d's default oversampling 128
    (96, 4, 10, 4, 3, 1, True),       # 4 pols, per-channel / per-pol kernels
    (128, 8, 32, 1, 2, 7, False),     # large w-kernels, several planes
    (160, 2, 64, 2, 1, 3, False),     # support 64
])
def test_grid_degrid_vs_oracle(arl, oracle, precision, N, O, S, npol, nchan, nz, distinct):
    rng = numpy.random.default_rng(N + O + S + npol)
    im, cf, vis, maps, gax = _random_case(arl, oracle, rng, N, 4e-3, O, S, 2500, nchan, npol, nz, 20.0, distinct)
    gd = arl.create_griddata_from_image(im)
    gd, sumwt = arl.grid_visibility_to_griddata(vis, gd, cf, precision=precision)
    g_ref, sw_ref = oracle.grid_vec(vis.vis, vis.imaging_weight, maps, cf.data, gax['shape'])
    assert rel(gd.data, g_ref) < TOL[precision]
    assert rel(sumwt, sw_ref) < TOLW[precision]
    rg = rng.normal(size=gax['shape']) + 1j * rng.normal(size=gax['shape'])
    gd.data[...] = rg
    out = arl.degrid_visibility_from_griddata(vis, gd, cf, precision=precision)
    assert rel(out.vis, oracle.degrid_vec(rg, maps, cf.data)) < TOL[precision]


@pytest.mark.parametrize('precision', ['fp64', 'fp32c'])
def test_plane_support(arl, oracle, precision):
    """Plane-dependent support (8 -> 32 with |w|): the GPU skips the cropped taps,
    the oracle grids with them zeroed."""
    rng = numpy.random.default_rng(77)
    N, cell, O, S, nz, zstep = 192, 3e-3, 4, 32, 9, 15.0
    im = make_image(arl, N, cell, [1e8], 1e7)
    gcf, cf = arl.create_awterm_convolutionfunction(im, nw=nz, wstep=zstep, oversampling=O, support=S,
                                                    maxsupport=256)
    wpl = (numpy.arange(nz) - nz // 2) * zstep
    arl.set_plane_support(cf, arl.support_schedule(wpl, 8, 32))
    du = abs(1.0 / (N * cell))
    lim = (N // 2 - S // 2 - 2) * du
    n = 3000
    uvw = numpy.stack([rng.uniform(-lim, lim, n), rng.uniform(-lim, lim, n), rng.uniform(-60, 60, n)], axis=1)
    freq = numpy.full(n, 1e8)
    vis = make_vis(arl, uvw, freq, rng.normal(size=(n, 1)) + 1j * rng.normal(size=(n, 1)), numpy.ones((n, 1)))
    img = oracle.image_geometry(N, cell)
    gax, cax = oracle.grid_axes(img), oracle.cf_axes(img, O, S, nz=nz, zstep=zstep)
    maps = oracle.convolution_mapping(uvw, freq, gax, cax)
    gd, _ = arl.grid_visibility_to_griddata(vis, arl.create_griddata_from_image(im), cf, precision=precision)
    g_ref, _ = oracle.grid_vec(vis.vis, vis.imaging_weight, maps, cf.data, gax['shape'])
    assert rel(gd.data, g_ref) < TOL[precision]
    out = arl.degrid_visibility_from_griddata(vis, gd, cf, precision=precision)
    assert rel(out.vis, oracle.degrid_vec(g_ref, maps, cf.data)) < TOL[precision]


# ---------------------------------------------------------------------------
# Edge cases and properties
# ---------------------------------------------------------------------------
def test_empty_rows(arl):
    im = make_image(arl, 64, 8e-3, [1e8], 1e6)
    gcf, cf = arl.create_pswf_convolutionfunction(im, oversampling=4, support=6)
    vis = make_vis(arl, numpy.zeros((0, 3)), numpy.zeros(0), numpy.zeros((0, 1)), numpy.zeros((0, 1)))
    for p in ('fp64', 'fp32c'):
        gd, sw = arl.grid_visibility_to_griddata(vis, arl.create_griddata_from_image(im), cf, precision=p)
        assert numpy.all(gd.data == 0) and numpy.all(sw == 0)
        out = arl.degrid_visibility_from_griddata(vis, gd, cf, precision=p)
        assert out.vis.shape == (0, 1)


def test_rows_outside_grid_raise(arl):
    im = make_image(arl, 64, 8e-3, [1e8], 1e6)
    gcf, cf = arl.create_pswf_convolutionfunction(im, oversampling=4, support=8)
    du = abs(1.0 / (64 * 8e-3))
    uvw = numpy.array([[0.0, 0.0, 0.0], [31.5 * du, 0.0, 0.0], [0.0, -29.0 * du, 0.0], [0.0, 10 * du, 0.0]])
    vis = make_vis(arl, uvw, numpy.full(4, 1e8), numpy.ones((4, 1)), numpy.ones((4, 1)))
    with pytest.raises(AssertionError):
        arl.grid_visibility_to_griddata(vis, arl.create_griddata_from_image(im), cf)
    gd, _ = arl.grid_visibility_to_griddata(vis, arl.create_griddata_from_image(im), cf, check=False)
    out = arl.degrid_visibility_from_griddata(vis, gd, cf, check=False)
    assert out.vis[1, 0] == 0 and out.vis[2, 0] == 0 and out.vis[0, 0] != 0


def test_adjointness(arl):
    """<grid(v), g> = <v * wt, degrid(g)>: the gridder is the degridder's adjoint."""
    rng = numpy.random.default_rng(11)
    N, O, S, n = 128, 8, 8, 5000
    im = make_image(arl, N, 4e-3, [1e8], 1e6)
    _, cf = arl.create_pswf_convolutionfunction(im, oversampling=O, support=S)
    du = abs(1.0 / (N * 4e-3))
    lim = (N // 2 - S // 2 - 2) * du
    uvw = numpy.stack([rng.uniform(-lim, lim, n), rng.uniform(-lim, lim, n), numpy.zeros(n)], axis=1)
    v = rng.normal(size=(n, 1)) + 1j * rng.normal(size=(n, 1))
    wt = rng.uniform(0.5, 2, (n, 1))
    vis = make_vis(arl, uvw, numpy.full(n, 1e8), v, wt)
    g = rng.normal(size=(1, 1, 1, N, N)) + 1j * rng.normal(size=(1, 1, 1, N, N))
    for p, tol in (('fp64', 1e-12), ('fp32c', 1e-5)):
        gd, _ = arl.grid_visibility_to_griddata(vis, arl.create_griddata_from_image(im), cf, precision=p)
        lhs = numpy.vdot(gd.data, g)
        gg = arl.create_griddata_from_image(im)
        gg.data[...] = g
        out = arl.degrid_visibility_from_griddata(vis, gg, cf, precision=p)
        rhs = numpy.vdot(v * wt, out.vis)
        assert abs(lhs - rhs) / abs(lhs) < tol


def test_device_resident_path_matches_host(arl):
    rng = numpy.random.default_rng(21)
    N, O, S, n = 128, 8, 8, 4000
    im = make_image(arl, N, 4e-3, [1e8], 1e6)
    gcf, cf = arl.create_pswf_convolutionfunction(im, oversampling=O, support=S)
    du = abs(1.0 / (N * 4e-3))
    lim = (N // 2 - S // 2 - 2) * du
    uvw = numpy.stack([rng.uniform(-lim, lim, n), rng.uniform(-lim, lim, n), numpy.zeros(n)], axis=1)
    vis = make_vis(arl, uvw, numpy.full(n, 1e8), rng.normal(size=(n, 1)) + 0j, numpy.ones((n, 1)))
    dvis = arl.DeviceVisibility.from_visibility(vis, 'fp32c')
    host_img, host_sw = arl.invert_2d(vis, im, gcfcf=(gcf, cf), precision='fp32c')
    dev_img, dev_sw = arl.invert_2d(dvis, im, gcfcf=(gcf, cf), precision='fp32c')
    assert isinstance(dev_img.data, torch.Tensor) and dev_img.data.is_cuda
    # Two FP32C runs differ only by atomic ordering, which the grid correction
    # amplifies at the field edge.
    assert_image(dev_img.data.cpu().numpy(), host_img.data, gcf.data, 'fp32c')
    gdev = arl.create_griddata_on_device(im, precision='fp32c')
    gdev, _ = arl.grid_visibility_to_griddata(dvis, gdev, cf, precision='fp32c')
    assert gdev.data.is_cuda


def test_c2_full_size_properties(arl):
    """Full C2 workload (W-projection, 64 planes, support 8 -> 32, 4 channels):
    FP32C against the FP64 GPU path, exact weight sums, exact linearity."""
    sim = __import__('importlib').import_module('algorithm-reference-library_gb300.simulation')
    w = sim.make_workload('C2', device=torch.device('cuda'))
    n = w['uvw'].shape[0]
    im = make_image(arl, w['npixel'], w['cellsize'], w['freqs'], w['channel_bandwidth'])
    gcf, cf = arl.create_awterm_convolutionfunction(im, nw=w['nwplanes'], wstep=w['wstep'],
                                                    oversampling=w['oversampling'], support=w['support'],
                                                    plane_support=w['plane_support'])
    dev = torch.device('cuda')
    uvw = torch.as_tensor(w['uvw'], device=dev)
    f = torch.as_tensor(w['frequency'], device=dev)
    v64 = w['vis'].to(dev)
    res = {}
    for p in ('fp64', 'fp32c'):
        dvis = arl.DeviceVisibility(uvw, f, v64.to(arl.device.CDTYPE[p]),
                                    torch.ones((n, 1), dtype=arl.device.RDTYPE[p], device=dev))
        gd = arl.create_griddata_on_device(im, precision=p)
        gd, sw = arl.grid_visibility_to_griddata(dvis, gd, cf, precision=p)
        out = arl.degrid_visibility_from_griddata(dvis, gd, cf, precision=p)
        res[p] = (gd.data.to(torch.complex128).cpu().numpy(), sw.cpu().numpy(),
                  out.vis.to(torch.complex128).cpu().numpy())
    assert rel(res['fp32c'][0], res['fp64'][0]) < 1e-5
    assert rel(res['fp32c'][2], res['fp64'][2]) < 1e-5
    counts = numpy.bincount(numpy.round((w['frequency'] - w['freqs'][0]) / w['channel_bandwidth']).astype(int),
                            minlength=len(w['freqs']))
    assert numpy.array_equal(res['fp64'][1][:, 0], counts.astype(float))
    # Linearity: doubling the visibilities doubles the grid bit for bit.
    dvis2 = arl.DeviceVisibility(uvw, f, (2 * v64).to(torch.complex64),
                                 torch.ones((n, 1), dtype=torch.float32, device=dev))
    g2, _ = arl.grid_visibility_to_griddata(dvis2, arl.create_griddata_on_device(im, precision='fp32c'), cf,
                                            precision='fp32c')
    g1 = res['fp32c'][0]
    assert numpy.max(numpy.abs(g2.data.to(torch.complex128).cpu().numpy() - 2 * g1)) <= 1e-6 * numpy.abs(g1).max()


def _oracle_by_support(oracle, vis, wt, maps, ocf, gshape, supports, grid=None):
    """The oracle's grid_vec / degrid_vec with each row's window cropped to its
    plane's support: rows are grouped by the support of their cf plane and
    each group runs on the centrally cropped table (the same taps and window
    positions as the full S x S window, whose outer taps are zero).  Returns
    (grid, sumwt) when grid is None, else the degridded rows of grid."""
    pwc = maps[5]
    S = ocf.shape[-1]
    out = None
    if grid is None:
        out = numpy.zeros(gshape, dtype=numpy.complex128)
        sumwt = numpy.zeros(gshape[:2])
    else:
        res = numpy.zeros((pwc.size, gshape[1]), dtype=numpy.complex128)
    for sz in numpy.unique(supports):
        rows = numpy.nonzero(supports[pwc] == sz)[0]
        if rows.size == 0:
            continue
        lo = S // 2 - sz // 2
        cfz = ocf[..., lo:lo + sz, lo:lo + sz]
        m = tuple(a[rows] for a in maps)
        if grid is None:
            g, sw = oracle.grid_vec(vis[rows], wt[rows], m, cfz, gshape)
            out += g
            sumwt += sw
        else:
            res[rows] = oracle.degrid_vec(grid, m, cfz)
    return (out, sumwt) if grid is None else res


def test_c2_subsample_vs_oracle(arl, oracle):
    """The bench workload's own geometry (C2: 4 channels onto 4 x 1024^2, 64
    w-kernel planes with support 8 -> 32, O = 8) on a seeded 1,000,000-row
    subsample: GPU grid and degrid, both precisions, against the oracle's
    complex128 gridder and degridder with the oracle's own w-kernels."""
    sim = __import__('importlib').import_module('algorithm-reference-library_gb300.simulation')
    w = sim.make_workload('C2')
    rng = numpy.random.default_rng(22)
    n = w['uvw'].shape[0]
    sel = numpy.sort(rng.choice(n, 1_000_000, replace=False))
    img = oracle.image_geometry(w['npixel'], w['cellsize'], len(w['freqs']), w['npol'], w['freqs'][0],
                                w['channel_bandwidth'])
    _, ocf = oracle.create_awterm_cf(img, nw=w['nwplanes'], wstep=w['wstep'], oversampling=w['oversampling'],
                                     support=w['support'])
    ocf = oracle.crop_cf_planes(ocf, w['plane_support'])
    gax = oracle.grid_axes(img)
    cax = oracle.cf_axes(img, w['oversampling'], w['support'], nz=w['nwplanes'], zstep=w['wstep'])
    uvw, f = w['uvw'][sel], w['frequency'][sel]
    maps = oracle.convolution_mapping(uvw, f, gax, cax)
    assert numpy.all(oracle.rows_in_grid(maps, gax['shape'], ocf.shape))
    vis = w['vis'].numpy()[sel]
    wt = numpy.ones(vis.shape)
    supports = numpy.asarray(w['plane_support'])
    g_ref, sw_ref = _oracle_by_support(oracle, vis, wt, maps, ocf, gax['shape'], supports)
    d_ref = _oracle_by_support(oracle, vis, wt, maps, ocf, gax['shape'], supports, grid=g_ref)

    im = make_image(arl, w['npixel'], w['cellsize'], w['freqs'], w['channel_bandwidth'])
    _, cf = arl.create_awterm_convolutionfunction(im, nw=w['nwplanes'], wstep=w['wstep'],
                                                  oversampling=w['oversampling'], support=w['support'],
                                                  plane_support=w['plane_support'])
    assert rel(cf.data, ocf) < 1e-12
    dv = arl.device
    dev = torch.device('cuda')
    gd = dv.grid_desc(arl.kernels._grid_wcs(im, 1, 1e15), gax['shape'])
    for p in ('fp64', 'fp32c'):
        cf_t, cs, ps, psup = dv.device_cf(cf, p, dev)
        cd = dv.cf_desc(cf.grid_wcs, cf.data.shape, cs, ps, psup, table=cf_t)
        t_uvw = torch.as_tensor(uvw, device=dev)
        t_f = torch.as_tensor(f, device=dev)
        g, sw, nbad = dv.grid(t_uvw, t_f, torch.as_tensor(vis, device=dev).to(dv.CDTYPE[p]),
                              torch.as_tensor(wt, device=dev).to(dv.RDTYPE[p]), cf_t, cd, gd, p)
        assert int(nbad.item()) == 0
        assert rel(g.to(torch.complex128).cpu().numpy(), g_ref) < TOL[p], p
        assert numpy.allclose(sw.cpu().numpy(), sw_ref, rtol=1e-12)
        d, _ = dv.degrid(t_uvw, t_f, torch.as_tensor(g_ref, device=dev).to(dv.CDTYPE[p]), cf_t, cd, gd, p)
        assert rel(d.to(torch.complex128).cpu().numpy(), d_ref) < TOL[p], p
        del g, d, cf_t
        torch.cuda.empty_cache()


@pytest.mark.parametrize('grid_kernel,degrid_kernel,subgrid,chunk', [
    (0, 0, 48, 512), (1, 1, 0, 512), (2, 2, 32, 2048), (2, 2, 0, 512), (3, 0, 0, 512), (4, 2, 0, 512),
    (4, 2, 32, 2048), (5, 2, 0, 512), (4, 3, 0, 512), (2, 3, 0, 2048)])
@pytest.mark.parametrize('npol', [1, 2, 4])
def test_kernel_variants_vs_oracle(arl, oracle, grid_kernel, degrid_kernel, subgrid, chunk, npol):
    """Every gridder / degridder variant, against the oracle (grid_kernels 3 and
    5 are the uncompensated measurement variants, held to the same 1e-5 bound
    here; 4 and 5 are the fixed-point gridders, FP32C only: FP64 runs 2)."""
    before = arl.tune.get_tuning()
    try:
        arl.tune.set_tuning(grid_kernel=grid_kernel, degrid_kernel=degrid_kernel, subgrid=subgrid, chunk=chunk)
        for precision in ('fp64', 'fp32c'):
            rng = numpy.random.default_rng(7 + npol)
            im, cf, vis, maps, gax = _random_case(arl, oracle, rng, 128, 4e-3, 8, 12, 4000, 2, npol, 3, 20.0, True)
            arl.set_plane_support(cf, [8, 12, 10])
            gd, sumwt = arl.grid_visibility_to_griddata(vis, arl.create_griddata_from_image(im), cf,
                                                        precision=precision)
            g_ref, sw_ref = oracle.grid_vec(vis.vis, vis.imaging_weight, maps, cf.data, gax['shape'])
            assert rel(gd.data, g_ref) < TOL[precision]
            assert rel(sumwt, sw_ref) < TOLW[precision]
            out = arl.degrid_visibility_from_griddata(vis, gd, cf, precision=precision)
            assert rel(out.vis, oracle.degrid_vec(g_ref, maps, cf.data)) < TOL[precision]
    finally:
        arl.tune.set_tuning(**before)


@pytest.mark.parametrize('persistent,lanes_per_row,chunk', [(1, 0, 256), (2, 0, 256), (2, 8, 64), (2, 16, 512),
                                                          (2, 32, 128), (0, 8, 512), (0, 32, 512)])
@pytest.mark.parametrize('npol', [1, 4])
def test_work_queue_and_lanes_per_row_vs_oracle(arl, oracle, persistent, lanes_per_row, chunk, npol):
    """The resident grid with static (1) or work-queue (2) chunk assignment,
    and every fixed lanes-per-row choice, against the oracle.  Small chunks
    make many more chunks than resident CTAs, so the queue hands out most of
    them; supports 12, 8 and 4 mix rows of different supports in one bin."""
    before = arl.tune.get_tuning()
    try:
        arl.tune.set_tuning(persistent=persistent, lanes_per_row=lanes_per_row, chunk=chunk)
        for precision in ('fp64', 'fp32c'):
            rng = numpy.random.default_rng(27 + npol)
            im, cf, vis, maps, gax = _random_case(arl, oracle, rng, 128, 4e-3, 8, 12, 30000, 2, npol, 3, 20.0, True)
            arl.set_plane_support(cf, [12, 8, 4])
            gd, sumwt = arl.grid_visibility_to_griddata(vis, arl.create_griddata_from_image(im), cf,
                                                        precision=precision)
            g_ref, sw_ref = oracle.grid_vec(vis.vis, vis.imaging_weight, maps, cf.data, gax['shape'])
            assert rel(gd.data, g_ref) < TOL[precision]
            assert rel(sumwt, sw_ref) < TOLW[precision]
            out = arl.degrid_visibility_from_griddata(vis, gd, cf, precision=precision)
            assert rel(out.vis, oracle.degrid_vec(g_ref, maps, cf.data)) < TOL[precision]
    finally:
        arl.tune.set_tuning(**before)


@pytest.mark.parametrize('gather_rows,persistent,stash_rows,chunk',
                         [(0, 0, 0, 512), (1, 0, 0, 512), (1, 0, 1, 512), (1, 2, 1, 128), (0, 2, 1, 256),
                          (1, 0, 1, 2048)])
def test_bin_order_rows_vs_oracle(arl, oracle, gather_rows, persistent, stash_rows, chunk):
    """The FP32C gridder with one polarisation reading vis and weight from a
    bin-order copy in the plan workspace (gather_rows 1, the default) or
    through the sort index (0), and the gridder and packed degridder taking
    each row's set-up from the footprint pass (stash_rows 1, the default for
    supports above 8 with chunks of at most 512 rows; chunk 2048 falls back),
    against the oracle; a plan gridded twice and then degridded, so the copy
    in the plan's mapping scratch must leave the plan itself intact."""
    import ctypes
    before = arl.tune.get_tuning()
    try:
        arl.tune.set_tuning(gather_rows=gather_rows, persistent=persistent, stash_rows=stash_rows, chunk=chunk)
        rng = numpy.random.default_rng(63)
        im, cf, vis, maps, gax = _random_case(arl, oracle, rng, 128, 4e-3, 8, 12, 40000, 2, 1, 3, 20.0, True)
        arl.set_plane_support(cf, [12, 8, 4])
        g_ref, sw_ref = oracle.grid_vec(vis.vis, vis.imaging_weight, maps, cf.data, gax['shape'])
        nat, dv = arl._native, arl.device
        dev = torch.device('cuda')
        cf_t, cs, ps, psup = dv.device_cf(cf, 'fp32c', dev)
        cd = dv.cf_desc(cf.grid_wcs, cf.data.shape, cs, ps, psup, table=cf_t)
        gd = dv.grid_desc(arl.create_griddata_from_image(im).grid_wcs, g_ref.shape)
        n = vis.nvis
        uvw = torch.as_tensor(vis.uvw, device=dev)
        f = torch.as_tensor(vis.frequency, device=dev)
        v = torch.as_tensor(vis.vis, device=dev).to(torch.complex64)
        w = torch.as_tensor(vis.imaging_weight, device=dev).to(torch.float32)
        ws = torch.empty(dv.plan_bytes(n, gd, cd), dtype=torch.uint8, device=dev)
        grid = torch.empty(g_ref.shape, dtype=torch.complex64, device=dev)
        sumwt = torch.empty(sw_ref.shape, dtype=torch.float64, device=dev)
        sp = nat.stream_ptr()
        nat.call('arlgpu_plan_build', nat.ptr(uvw), nat.ptr(f), n, ctypes.byref(gd), ctypes.byref(cd), nat.ptr(ws),
                 ws.numel(), None, sp)
        for _ in range(2):
            nat.call('arlgpu_grid_planned', nat.ptr(v), nat.ptr(w), n, nat.FP32C, nat.ptr(cf_t), ctypes.byref(cd),
                     nat.ptr(grid), ctypes.byref(gd), nat.ptr(sumwt), nat.ptr(ws), ws.numel(), sp)
            assert rel(grid.to(torch.complex128).cpu().numpy(), g_ref) < TOL['fp32c']
            assert rel(sumwt.cpu().numpy(), sw_ref) < TOLW['fp32c']
        out = torch.empty((n, 1), dtype=torch.complex64, device=dev)
        nat.call('arlgpu_degrid_planned', n, nat.FP32C, nat.ptr(cf_t), ctypes.byref(cd), nat.ptr(grid),
                 ctypes.byref(gd), nat.ptr(out), nat.ptr(ws), ws.numel(), sp)
        assert rel(out.to(torch.complex128).cpu().numpy(), oracle.degrid_vec(g_ref, maps, cf.data)) < TOL['fp32c']
    finally:
        arl.tune.set_tuning(**before)


@pytest.mark.parametrize('S,npol', [(8, 1), (12, 1), (8, 4)])
def test_dense_cells_vs_oracle(arl, oracle, S, npol):
    """30,000 rows within 1.5 pixels of the grid centre: every segment is a
    full chunk of 512 rows and the cells under it take up to 512 taps each,
    the most the fixed-point gridder's biased cell sums carry (the tap count
    comes back from the residual plane's high bits).  Held to 1e-6, ten times
    tighter than the other FP32C grid checks."""
    rng = numpy.random.default_rng(71 + S + npol)
    im, cf, vis, maps, gax = _random_case(arl, oracle, rng, 64, 4e-3, 8, S, 30000, 1, npol, lim_px=1.5)
    g_ref, sw_ref = oracle.grid_vec(vis.vis, vis.imaging_weight, maps, cf.data, gax['shape'])
    gd = arl.create_griddata_from_image(im)
    gd, sw = arl.grid_visibility_to_griddata(vis, gd, cf, precision='fp32c')
    assert rel(gd.data, g_ref) < 1e-6
    assert rel(sw, sw_ref) < TOLW['fp32c']


def _degrid_planned_with_flags(arl, vis, gd_h, cf, precision='fp32c'):
    """Degrid through the C ABI (plan_build + degrid_planned on this test's own
    workspace) and read the plan's status flags afterwards."""
    import ctypes
    nat = arl._native
    dv = arl.device
    dev = torch.device('cuda')
    cf_t, cs, ps, psup = dv.device_cf(cf, precision, dev)
    cd = dv.cf_desc(cf.grid_wcs, cf.data.shape, cs, ps, psup, table=cf_t)
    gd = dv.grid_desc(gd_h.grid_wcs, gd_h.data.shape)
    n = vis.nvis
    uvw = torch.as_tensor(vis.uvw, device=dev)
    f = torch.as_tensor(vis.frequency, device=dev)
    g = torch.as_tensor(gd_h.data, device=dev).to(dv.CDTYPE[precision]).contiguous()
    ws = torch.empty(dv.plan_bytes(n, gd, cd), dtype=torch.uint8, device=dev)
    out = torch.empty((n, gd.npol), dtype=dv.CDTYPE[precision], device=dev)
    sp = nat.stream_ptr()
    nat.call('arlgpu_plan_build', nat.ptr(uvw), nat.ptr(f), n, ctypes.byref(gd), ctypes.byref(cd), nat.ptr(ws),
             ws.numel(), None, sp)
    nat.call('arlgpu_degrid_planned', n, nat.PRECISIONS[precision], nat.ptr(cf_t), ctypes.byref(cd), nat.ptr(g),
             ctypes.byref(gd), nat.ptr(out), nat.ptr(ws), ws.numel(), sp)
    flags = ctypes.c_uint32(99)
    nat.call('arlgpu_plan_flags', n, ctypes.byref(gd), ctypes.byref(cd), nat.ptr(ws), ws.numel(),
             ctypes.byref(flags), sp)
    return out.to(torch.complex128).cpu().numpy(), flags.value


@pytest.mark.parametrize('persistent,chunk,nvis', [(0, 512, 60000), (2, 128, 60000), (0, 512, 300), (1, 2048, 60000)])
def test_tma_degridder_vs_oracle(arl, oracle, persistent, chunk, nvis):
    """degrid_kernel 4 (grid tile and kernel taps staged by TMA tensor copies)
    against the oracle: supports 2 .. 32 whose windows start on even and odd
    columns (so both box widths sz and sz + 2 occur), dense bins (the tap
    pipeline and every rows-per-warp choice) and, with 300 rows, bins of
    single rows (the direct path).  FP32C 1e-5; the kernel's bounded waits
    must all have completed (status flag 0)."""
    before = arl.tune.get_tuning()
    try:
        arl.tune.set_tuning(degrid_kernel=4, persistent=persistent, chunk=chunk)
        rng = numpy.random.default_rng(41)
        sup = [32, 30, 26, 20, 16, 14, 10, 8, 6, 2]
        im, cf, vis, maps, gax = _random_case(arl, oracle, rng, 256, 4e-3, 8, 32, nvis, 2, 1, len(sup), 20.0, True)
        arl.set_plane_support(cf, sup)
        rgrid = rng.normal(size=gax['shape']) + 1j * rng.normal(size=gax['shape'])
        gd = arl.create_griddata_from_image(im)
        gd.data = rgrid
        got, flags = _degrid_planned_with_flags(arl, vis, gd, cf)
        assert flags == 0
        want = oracle.degrid_vec(rgrid, maps, cf.data)
        assert rel(got, want) < TOL['fp32c']
        # and through the package's degrid_visibility_from_griddata
        out = arl.degrid_visibility_from_griddata(vis, gd, cf, precision='fp32c')
        assert rel(out.vis, want) < TOL['fp32c']
    finally:
        arl.tune.set_tuning(**before)


@pytest.mark.parametrize('small_rows,small_rows_degrid', [(1, 1), (2, 2), (4, 4), (2, 4)])
@pytest.mark.parametrize('npol', [1, 2, 4])
def test_small_support_rows_per_warp_vs_oracle(arl, oracle, small_rows, small_rows_degrid, npol):
    """Supports up to 8 run several rows per warp (16 or 8 lanes each); w-kernel
    planes of supports 8, 6 and 4 put rows of different supports side by side
    in one warp.  Against the oracle, default kernels otherwise."""
    before = arl.tune.get_tuning()
    try:
        arl.tune.set_tuning(small_rows=small_rows, small_rows_degrid=small_rows_degrid)
        for precision in ('fp64', 'fp32c'):
            rng = numpy.random.default_rng(17 + npol)
            im, cf, vis, maps, gax = _random_case(arl, oracle, rng, 128, 4e-3, 8, 8, 5000, 2, npol, 3, 20.0, True)
            arl.set_plane_support(cf, [8, 6, 4])
            gd, sumwt = arl.grid_visibility_to_griddata(vis, arl.create_griddata_from_image(im), cf,
                                                        precision=precision)
            g_ref, sw_ref = oracle.grid_vec(vis.vis, vis.imaging_weight, maps, cf.data, gax['shape'])
            assert rel(gd.data, g_ref) < TOL[precision]
            assert rel(sumwt, sw_ref) < TOLW[precision]
            out = arl.degrid_visibility_from_griddata(vis, gd, cf, precision=precision)
            assert rel(out.vis, oracle.degrid_vec(g_ref, maps, cf.data)) < TOL[precision]
    finally:
        arl.tune.set_tuning(**before)
