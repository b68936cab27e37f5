"""Hogbom CLEAN on the GPU against the reference's own outputs
(tests/golden/ref_hogbom.npz) and the oracle: components and residuals are
bit-identical (FP64, the reference's operation order, numpy.argmax's first
index on ties)."""
import numpy
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module', autouse=True)
def need_cuda(arl):
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    arl._native.load()


def test_hogbom_matches_reference(arl, golden):
    d = golden('ref_hogbom.npz')
    c1, r1 = arl.hogbom(d['dirty'], d['psf'], None, 0.1, 0.0, 400, 0.01)
    assert numpy.array_equal(c1, d['c1']) and numpy.array_equal(r1, d['r1'])
    c2, r2 = arl.hogbom(d['dirty'], d['psf'], d['window'], 0.7, 0.05, 300, 0.001)
    assert numpy.array_equal(c2, d['c2']) and numpy.array_equal(r2, d['r2'])


def test_deconvolve_cube_hogbom_matches_reference(arl, golden):
    d = golden('ref_hogbom.npz')
    im = arl.create_image(npixel=128, cellsize=0.001, frequency=numpy.array([1e8, 1.1e8]),
                          channel_bandwidth=numpy.array([1e7]))
    dim = arl.create_image_from_array(d['d2'], im.wcs, im.polarisation_frame)
    pim = arl.create_image_from_array(d['p2'].copy(), im.wcs, im.polarisation_frame)
    comp, resid = arl.deconvolve_cube(dim, pim, algorithm='hogbom', niter=200, gain=0.2, threshold=0.0,
                                      fractional_threshold=0.05, window_shape='quarter', psf_support=40)
    assert numpy.array_equal(comp.data, d['cube_comp']) and numpy.array_equal(resid.data, d['cube_resid'])


def test_hogbom_larger_image_vs_oracle(arl, oracle):
    """256^2 dirty image, full-size PSF, 1500 iterations: bit-identical to the
    oracle's restatement of the reference loop."""
    rng = numpy.random.default_rng(91)
    N = 256
    samp = numpy.zeros((N, N))
    samp[rng.integers(N // 2 - 60, N // 2 + 60, 20000), rng.integers(N // 2 - 60, N // 2 + 60, 20000)] = 1.0
    samp = samp + samp[::-1, ::-1]
    psf = numpy.real(numpy.fft.fftshift(numpy.fft.ifft2(numpy.fft.ifftshift(samp))))
    psf /= psf.max()
    sky = numpy.zeros((N, N))
    sky[rng.integers(N // 4, 3 * N // 4, 40), rng.integers(N // 4, 3 * N // 4, 40)] = rng.uniform(0.2, 5.0, 40)
    dirty = numpy.real(numpy.fft.fftshift(numpy.fft.ifft2(numpy.fft.fft2(numpy.fft.ifftshift(sky)) *
                                                          numpy.fft.fft2(numpy.fft.ifftshift(psf)))))
    c, r = arl.hogbom(dirty, psf, None, 0.1, 0.0, 1500, 0.001)
    c0, r0 = oracle.hogbom(dirty, psf, None, 0.1, 0.0, 1500, 0.001)
    assert numpy.array_equal(c, c0) and numpy.array_equal(r, r0)


def test_hogbom_complex_matches_reference(arl, golden):
    """Complex Hogbom of Q + iU (cleaners.py:72-131) against the reference's
    outputs, without and with a window.  FP64 in the reference's order; the
    peak magnitude is the hypotenuse, which CUDA and the host C library may
    round one ulp apart, so the check is bit-identical components and
    residuals or, failing that, FP64-tight agreement with the same peaks."""
    d = golden('ref_hogbom_complex.npz')
    for win, gain, thresh, niter, frac, tag in ((None, 0.1, 0.0, 300, 0.01, '1'),
                                                  (d['window'], 0.5, 0.02, 200, 0.001, '2')):
        cq, cu, rq, ru = arl.hogbom_complex(d['dq'], d['du'], d['psf'], d['psf'], win, gain, thresh, niter, frac)
        for got, key in ((cq, 'cq'), (cu, 'cu'), (rq, 'rq'), (ru, 'ru')):
            want = d[key + tag]
            assert numpy.array_equal(got, want) or _close(got, want), key + tag
        assert numpy.array_equal(numpy.nonzero(cq)[0], numpy.nonzero(d['cq' + tag])[0])


def test_deconvolve_cube_hogbom_complex_matches_reference(arl, golden):
    """deconvolve_cube(algorithm='hogbom-complex') on an I, Q, U, V cube: I and
    V by Hogbom, Q and U together; components and residuals in stokesIQUV."""
    d = golden('ref_hogbom_complex.npz')
    frame = arl.PolarisationFrame('stokesIQUV')
    im = arl.create_image(npixel=96, cellsize=0.001, frequency=numpy.array([1e8]),
                          channel_bandwidth=numpy.array([1e7]), polarisation_frame=frame)
    d4 = numpy.stack([d['di'], d['dq'], d['du'], d['dv']])[None]
    p4 = numpy.stack([d['psf']] * 4)[None]
    dim = arl.create_image_from_array(d4, im.wcs, frame)
    pim = arl.create_image_from_array(p4.copy(), im.wcs, frame)
    comp, resid = arl.deconvolve_cube(dim, pim, algorithm='hogbom-complex', niter=150, gain=0.2, threshold=0.0,
                                      fractional_threshold=0.05, window_shape='quarter', psf_support=30)
    assert comp.polarisation_frame == frame and resid.polarisation_frame == frame
    assert numpy.array_equal(comp.data, d['cube_comp']) or _close(comp.data, d['cube_comp'])
    assert numpy.array_equal(resid.data, d['cube_resid']) or _close(resid.data, d['cube_resid'])


def _msmfs_case(arl, d):
    N = d['cube'].shape[-1]
    freqs = d['freqs']
    im = arl.create_image(npixel=N, cellsize=0.001, frequency=freqs, channel_bandwidth=numpy.array([freqs[1] - freqs[0]]))
    dim = arl.create_image_from_array(d['cube'].copy(), im.wcs, im.polarisation_frame)
    pim = arl.create_image_from_array(d['psfs'][:, None].copy(), im.wcs, im.polarisation_frame)
    return dim, pim


def test_frequency_moments_match_reference(arl, golden):
    """calculate_image_frequency_moments (image/operations.py:239-282) of the
    dirty cube and the PSF, and the cube rebuilt from moments."""
    d = golden('ref_msmfsclean.npz')
    dim, pim = _msmfs_case(arl, d)
    dm = arl.calculate_image_frequency_moments(dim, nmoment=2)
    pm = arl.calculate_image_frequency_moments(pim, nmoment=4)
    assert dm.wcs.wcs.ctype[3] == 'MOMENT'
    assert _close(dm.data[:, 0], d['dmom'], 1e-14) and _close(pm.data[:, 0], d['pmom'], 1e-14)
    back = arl.calculate_image_from_frequency_moments(dim, pm)
    want = numpy.zeros_like(d['cube'])
    f = d['freqs']
    f0 = numpy.average(f)
    for c in range(len(f)):
        for m in range(4):
            want[c] += d['pmom'][m][None] * ((f[c] - f0) / f0) ** m
    assert _close(back.data, want, 1e-13)


@pytest.mark.parametrize('tag,findpeak,windowed', [('arl', 'ARL', False), ('casa', 'CASA', False),
                                                   ('alg1', 'Algorithm1', False), ('arlw', 'ARL', True)])
def test_msmfsclean_matches_reference(arl, golden, tag, findpeak, windowed):
    """msmfsclean (cleaners.py:469-600) on two dirty moments with four PSF
    moments, three scales, each findpeak, with and without a window, against
    the reference's outputs.  The set-up's convolutions are cuFFT transforms,
    which round differently from NumPy's: FP64 tolerance 1e-10."""
    d = golden('ref_msmfsclean.npz')
    win = d['window'] if windowed else None
    c, r = arl.msmfsclean(d['dmom'], d['pmom'], win, 0.3, 0.0, 80, [0, 3, 8], 0.02, findpeak)
    assert _close(c, d['c_' + tag], 1e-10) and _close(r, d['r_' + tag], 1e-10)


def test_deconvolve_cube_msmfsclean_matches_reference(arl, golden):
    """deconvolve_cube(algorithm='msmfsclean', nmoment=2) on a five-channel cube:
    components and residuals rebuilt on the channels (deconvolution.py:156-210)."""
    d = golden('ref_msmfsclean.npz')
    dim, pim = _msmfs_case(arl, d)
    comp, resid = arl.deconvolve_cube(dim, pim, algorithm='msmfsclean', nmoment=2, niter=60, gain=0.3,
                                      threshold=0.0, fractional_threshold=0.05, scales=[0, 3, 8])
    assert _close(comp.data, d['cube_comp'], 1e-10) and _close(resid.data, d['cube_resid'], 1e-10)


def _close(a, b, tol=1e-12):
    return numpy.max(numpy.abs(a - b)) <= tol * numpy.max(numpy.abs(b))


def test_msclean_matches_reference(arl, oracle, golden):
    """Multiscale CLEAN with its set-up on the device (scale images and their
    complex128 cuFFT convolutions): against the reference's fixtures and the
    oracle (NumPy FFTs), 1e-10 relative on components and residuals -- the
    two FFT libraries round differently at ~1e-16, which the minor cycle
    carries through its subtractions but which never changes a peak choice
    on these images."""
    h = golden('ref_hogbom.npz')
    d = golden('ref_msclean.npz')
    tol = 1e-10
    c1, r1 = arl.msclean(h['dirty'], h['psf'], None, 0.3, 0.0, 150, [0, 3, 10], 0.01)
    assert _close(c1, d['c1'], tol) and _close(r1, d['r1'], tol)
    o1, q1 = oracle.msclean(h['dirty'], h['psf'], None, 0.3, 0.0, 150, [0, 3, 10], 0.01)
    assert _close(c1, o1, tol) and _close(r1, q1, tol)
    c2, r2 = arl.msclean(h['dirty'], h['psf'][32:96, 32:96], h['window'], 0.7, 0.02, 100, [0, 3], 0.001)
    assert _close(c2, d['c2'], tol) and _close(r2, d['r2'], tol)
    o2, q2 = oracle.msclean(h['dirty'], h['psf'][32:96, 32:96], h['window'], 0.7, 0.02, 100, [0, 3], 0.001)
    assert _close(c2, o2, tol) and _close(r2, q2, tol)


def test_msclean_setup_vs_oracle(arl, oracle):
    """The device set-up alone, on odd and even image sizes (the fftshift /
    ifftshift gathers differ for odd sizes) and a scale wider than half the
    PSF: scale images, convolved stacks, coupling matrix and window stack
    against the oracle's NumPy restatement, 1e-12 relative."""
    import ctypes
    rng = numpy.random.default_rng(93)
    nat = arl._native
    dev = torch.device('cuda')
    for (nx, ny, pnx, pny, scales) in ((96, 80, 48, 40, [0, 3, 10]), (65, 71, 33, 31, [0, 4, 9, 20])):
        dirty = rng.normal(size=(nx, ny))
        psf = rng.normal(size=(pnx, pny)) + 4.0
        window = (rng.uniform(size=(nx, ny)) > 0.3).astype(float)
        ns = len(scales)
        nb = ctypes.c_size_t(0)
        nat.call('arlgpu_msclean_setup_bytes', nx, ny, pnx, pny, ns, ctypes.byref(nb))
        ws = torch.empty(nb.value, dtype=torch.uint8, device=dev)
        f64 = dict(dtype=torch.float64, device=dev)
        t = {k: torch.as_tensor(v, device=dev) for k, v in (('d', dirty), ('p', psf), ('w', window))}
        out = dict(stack=torch.empty((ns, nx, ny), **f64), pss=torch.empty((ns, ns, pnx, pny), **f64),
                   pscale=torch.empty((ns, pnx, pny), **f64), wstack=torch.empty((ns, nx, ny), **f64),
                   coupling=torch.empty((ns, ns), **f64), scalars=torch.empty(2, **f64))
        sc = (ctypes.c_double * ns)(*[float(x) for x in scales])
        nat.call('arlgpu_msclean_setup', nat.ptr(t['d']), nx, ny, nat.ptr(t['p']), pnx, pny, nat.ptr(t['w']), sc, ns,
                 nat.ptr(out['stack']), nat.ptr(out['pss']), nat.ptr(out['pscale']), nat.ptr(out['wstack']),
                 nat.ptr(out['coupling']), nat.ptr(out['scalars']), nat.ptr(ws), ws.numel(), nat.stream_ptr())
        got = {k: v.cpu().numpy() for k, v in out.items()}
        pmax = psf.max()
        ss = oracle.scalestack([ns, nx, ny], scales)
        pss = oracle.scalestack([ns, pnx, pny], scales)
        assert _close(got['pscale'], pss)
        xd = oracle._ft(dirty / pmax)
        stack = numpy.stack([oracle._ift_real(xd * numpy.conjugate(oracle._ft(ss[i]))) for i in range(ns)])
        assert _close(got['stack'], stack)
        xp = oracle._ft(psf / pmax)
        xs = [oracle._ft(pss[i]) for i in range(ns)]
        pp = numpy.array([[oracle._ift_real(xp * xs[b] * numpy.conjugate(xs[a])) for b in range(ns)]
                          for a in range(ns)])
        assert _close(got['pss'], pp)
        assert _close(got['coupling'], pp.max(axis=(2, 3)))
        xw = oracle._ft(window)
        wconv = numpy.stack([oracle._ift_real(xw * numpy.conjugate(oracle._ft(ss[i]))) for i in range(ns)])
        # the 0.9 threshold: cells within rounding of it may go either way
        far = numpy.abs(wconv - 0.9) > 1e-12
        assert numpy.array_equal(got['wstack'][far], (wconv > 0.9).astype(float)[far])
        assert got['scalars'][0] == pmax
        assert abs(got['scalars'][1] - numpy.abs(stack[0]).max()) <= 1e-12 * numpy.abs(stack[0]).max()


def test_deconvolve_cube_msclean_matches_reference(arl, golden):
    h = golden('ref_hogbom.npz')
    d = golden('ref_msclean.npz')
    im = arl.create_image(npixel=128, cellsize=0.001, frequency=numpy.array([1e8, 1.1e8]),
                          channel_bandwidth=numpy.array([1e7]))
    dim = arl.create_image_from_array(h['d2'], im.wcs, im.polarisation_frame)
    pim = arl.create_image_from_array(h['p2'].copy(), im.wcs, im.polarisation_frame)
    comp, resid = arl.deconvolve_cube(dim, pim, algorithm='msclean', niter=60, gain=0.5, threshold=0.0,
                                      fractional_threshold=0.05, scales=[0, 4, 8], psf_support=32)
    assert _close(comp.data, d['cube_comp'], 1e-10) and _close(resid.data, d['cube_resid'], 1e-10)
