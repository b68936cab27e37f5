"""The FP32C path's double-single inverse transform against cuFFT's complex128
transform of the same FP32 grid (tuning key "dsfft" 1 vs 0), on square and
non-square power-of-two planes from 64 to 16384 points per axis, with w-planes
summed, several images per call, the imaginary output and a zero sumwt; and
the batched w-stack image of one grid with the double-single transform and
w-screens against the complex128 transforms.

Tolerances: both transforms are accurate to ~1e-13 of the image scale (the
double-single numbers carry ~48-bit significands); 1e-11 of the image maximum
leaves room for the grid correction (up to 100x here).  The w-stack images also
differ by the FP32 rounding of the w-screens, which both paths evaluate with
FP32 sincospi from arguments that agree to ~1e-13 turns: 1e-6.
"""
import numpy
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module', autouse=True)
def need_cuda(arl):
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    arl._native.load()


@pytest.fixture
def dsfft_switch(arl):
    old = arl.tune.get_tuning()['dsfft']
    yield lambda v: arl.tune.set_tuning(dsfft=v)
    arl.tune.set_tuning(dsfft=old)


def _rel(a, b):
    return float((a - b).abs().max() / b.abs().max())


@pytest.mark.parametrize('ny,nx,nchan,npol,nw,sparse', [
    (64, 64, 1, 1, 1, False), (128, 256, 1, 2, 3, False), (256, 64, 2, 1, 1, False), (1024, 1024, 1, 1, 1, False),
    (4096, 4096, 1, 1, 1, False), (64, 8192, 1, 1, 1, False), (16384, 64, 1, 1, 1, False),
    (512, 2048, 2, 2, 1, False), (256, 512, 1, 1, 1, True), (64, 8192, 1, 2, 1, True)])
def test_dsfft_matches_complex128_transform(arl, dsfft_switch, ny, nx, nchan, npol, nw, sparse):
    """sparse: whole grid rows zero (the row pass skips their arithmetic), as in
    the w-stack slices of C3 / C5."""
    dv = arl.device
    dev = torch.device('cuda')
    g = torch.Generator(device='cpu').manual_seed(ny * 7 + nx)
    shape = (nchan, npol, nw, ny, nx)
    grid = torch.complex(torch.randn(shape, generator=g), torch.randn(shape, generator=g)).to(torch.complex64)
    if sparse:
        keep = torch.rand((nchan, npol, nw, ny, 1), generator=g) < 0.4
        grid = grid * keep
    grid = grid.to(dev)
    gcf = (1.0 + 99.0 * torch.rand((nchan, npol, ny, nx), generator=g, dtype=torch.float64)).to(dev)
    sw = 1.0 + torch.rand((nchan, npol), generator=g, dtype=torch.float64)
    if nchan * npol > 1:
        sw[0, 0] = 0.0
    sw = sw.to(dev)
    im = arl.create_image(npixel=64, cellsize=1e-3, frequency=numpy.array([1e8]),
                          channel_bandwidth=numpy.array([1e6]), phasecentre=arl.PhaseCentre(0.0, -45.0))
    gd = dv.grid_desc(arl.kernels._grid_wcs(im, nw, 1e15), shape)
    out = {}
    for v in (0, 1):
        dsfft_switch(v)
        out[v] = dv.fft_grid_to_image(grid, gd, gcf, 'fp32c', sumwt=sw, imaginary=True)
        out[v, 'raw'] = dv.fft_grid_to_image(grid, gd, gcf, 'fp32c', sumwt=None, imaginary=False)
    torch.cuda.synchronize()
    assert _rel(out[1][0], out[0][0]) < 1e-11
    assert _rel(out[1][1], out[0][1]) < 1e-11
    assert _rel(out[1, 'raw'][0], out[0, 'raw'][0]) < 1e-11
    if nchan * npol > 1:
        assert bool((out[1][0][0, 0] == 0).all()) and bool((out[1][1][0, 0] == 0).all())


@pytest.mark.parametrize('N,K,npol', [(256, 9, 1), (512, 16, 2)])
def test_dsfft_wstack_matches_complex128(arl, dsfft_switch, N, K, npol):
    rng = numpy.random.default_rng(N + K)
    cell, O, S, n = 2e-3, 8, 8, 20000
    pf = {1: 'stokesI', 2: 'stokesIQ'}[npol]
    im = arl.create_image(npixel=N, cellsize=cell, frequency=numpy.array([1.05e8]),
                          channel_bandwidth=numpy.array([1e8]), phasecentre=arl.PhaseCentre(0.0, -45.0),
                          polarisation_frame=arl.PolarisationFrame(pf))
    gcf, cf = arl.create_pswf_convolutionfunction(im, oversampling=O, support=S)
    lim = (N // 2 - S // 2 - 2) / (N * cell)
    uvw = numpy.stack([rng.uniform(-lim, lim, n), rng.uniform(-lim, lim, n), rng.uniform(-500, 500, n)], axis=1)
    v = rng.normal(size=(n, npol)) + 1j * rng.normal(size=(n, npol))
    vis = arl.Visibility(uvw=uvw, frequency=numpy.full(n, 1.05e8), vis=v, weight=numpy.ones((n, npol)),
                         polarisation_frame=arl.PolarisationFrame(pf))
    imager = arl.WStackImager(vis, im, K, gcfcf=(gcf, cf), precision='fp32c')
    imager.grid()  # one grid for both transforms (FP32 flush order varies between griddings)
    imgs = {}
    for sw in (0, 1):
        dsfft_switch(sw)
        imager.grid_to_image()
        imgs[sw] = imager.image.clone()
    assert _rel(imgs[1], imgs[0]) < 1e-6
