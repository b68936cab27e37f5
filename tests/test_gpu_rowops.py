"""Phase rotation (shift_vis_to_image) and scalar gains on the GPU against the oracle."""
import numpy
import pytest
import torch

from helpers import rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module', autouse=True)
def need_cuda(arl):
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')


def test_shift_vis_to_image(arl, oracle):
    rng = numpy.random.default_rng(2)
    n = 1000
    uvw = rng.normal(size=(n, 3)) * 300
    v = rng.normal(size=(n, 2)) + 1j * rng.normal(size=(n, 2))
    vis = arl.Visibility(uvw=uvw, frequency=numpy.full(n, 1e8), vis=v, weight=numpy.ones((n, 2)),
                         polarisation_frame=arl.PolarisationFrame('stokesIQ'))
    vis.phasecentre = arl.PhaseCentre(10.0, -45.0)
    im = arl.create_image(npixel=64, cellsize=1e-3, phasecentre=arl.PhaseCentre(10.3, -44.8),
                          polarisation_frame=arl.PolarisationFrame('stokesIQ'))
    l, m, _ = im.phasecentre.lmn(vis.phasecentre)
    for inverse in (False, True):
        out = arl.shift_vis_to_image(vis, im, inverse=inverse)
        assert rel(out.vis, oracle.phaserotate(v, uvw, l, m, inverse=inverse)) < 1e-12
    same = arl.create_image(npixel=64, cellsize=1e-3, phasecentre=arl.PhaseCentre(10.0, -45.0))
    assert arl.shift_vis_to_image(vis, same) is vis


def test_apply_gains(arl, oracle):
    rng = numpy.random.default_rng(4)
    n, nant = 2000, 16
    a1 = rng.integers(0, nant - 1, n).astype(numpy.int32)
    a2 = numpy.minimum(a1 + rng.integers(1, nant, n), nant - 1).astype(numpy.int32)
    a2 = numpy.where(a2 == a1, a1 + 1, a2).astype(numpy.int32)
    g = (1 + 0.1 * rng.normal(size=nant)) * numpy.exp(1j * rng.uniform(-3, 3, nant))
    v = rng.normal(size=(n, 4)) + 1j * rng.normal(size=(n, 4))
    dev = torch.device('cuda')
    # Device copies held in names until the library calls below have returned.
    t1 = torch.as_tensor(a1, device=dev)
    t2 = torch.as_tensor(a2, device=dev)
    tg = torch.as_tensor(g, device=dev)
    for prec, tol in (('fp64', 1e-13), ('fp32c', 1e-6)):
        for inverse in (False, True):
            t = torch.as_tensor(v, device=dev).to(arl.device.CDTYPE[prec]).contiguous()
            arl._native.call('arlgpu_apply_gains', arl._native.ptr(t), n, 4, arl._native.PRECISIONS[prec],
                             arl._native.ptr(t1), arl._native.ptr(t2), arl._native.ptr(tg), int(inverse),
                             arl._native.stream_ptr())
            gg = 1.0 / g if inverse else g
            assert rel(t.cpu().numpy(), oracle.apply_gains(v, a1, a2, gg)) < tol
