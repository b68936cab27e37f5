"""C4 at full size: the differentiable predict + gain solve.

128 antennas, 8 channels summed onto one 2048^2 image, 240 times (15.6 M rows),
PSWF support 8 x oversampling 8.  The model is 200 Gaussian-smoothed point
sources; V_obs = g[a2] conj(g[a1]) degrid(FFT(model)) + noise (sigma 0.01),
gains with amplitude N(1, 0.1) and phase U(-pi, pi).  The gradients of chi^2
with respect to the image and the gains, taken away from the solution, are
checked against central finite differences (h = 1e-4, relative error <= 1e-4
of the largest gradient) on the FP64 path, and the FP32C gradients against the
FP64 ones.  (The dense-DFT reference gradient runs at 64 x 64 in
test_gpu_autograd.py.)
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


@pytest.fixture(scope='module')
def c4(arl):
    sim = arl.simulation
    w = sim.make_workload('C4')
    im = sim.workload_image(arl, w)
    gcfcf = arl.create_pswf_convolutionfunction(im, oversampling=w['oversampling'], support=w['support'])
    dev = torch.device('cuda')
    n = w['uvw'].shape[0]
    ops = {}
    for p in ('fp64', 'fp32c'):
        dvis = arl.DeviceVisibility(torch.as_tensor(w['uvw'], device=dev), torch.as_tensor(w['frequency'], device=dev),
                                    torch.zeros((n, 1), dtype=arl.device.CDTYPE[p], device=dev),
                                    torch.ones((n, 1), dtype=arl.device.RDTYPE[p], device=dev))
        ops[p] = arl.autograd.GriddingOperator(dvis, im, gcfcf, precision=p)
    model = torch.as_tensor(w['model_image'], device=dev)
    gains = torch.as_tensor(w['gains'], device=dev)
    a1 = torch.as_tensor(w['antenna1'].astype(numpy.int32), device=dev)
    a2 = torch.as_tensor(w['antenna2'].astype(numpy.int32), device=dev)
    vobs = sim.observe(ops['fp64'].predict(model), gains, a1, a2, w['noise'], seed=1004)
    # away from the solution: a fainter model and perturbed gains
    rng = numpy.random.default_rng(44)
    x0 = 0.7 * model
    g0 = gains * torch.as_tensor(1.0 + 0.05 * (rng.normal(size=gains.shape[0]) +
                                               1j * rng.normal(size=gains.shape[0])), device=dev)
    return dict(w=w, ops=ops, vobs=vobs, a1=a1, a2=a2, x0=x0, g0=g0)


def test_c4_gradients_vs_finite_differences(arl, c4):
    op = c4['ops']['fp64']
    args = (c4['vobs'], op, c4['a1'], c4['a2'])
    x, g = c4['x0'], c4['g0']
    c, gx, gg = arl.autograd.gain_chi2_step(x, g, *args)

    def f(xx, gg_):
        with torch.no_grad():
            return float(arl.autograd.chi2(xx, gg_, *args))

    assert abs(f(x, g) - float(c)) <= 1e-12 * float(c)
    h = 1e-4
    # the image pixels with the largest gradients, and a few random ones
    flat = gx.abs().reshape(-1)
    picks = list(torch.topk(flat, 4).indices.cpu().numpy())
    picks += list(numpy.random.default_rng(1).integers(0, flat.numel(), 4))
    scale_x = float(gx.abs().max())
    worst = 0.0
    for k in picks:
        e = torch.zeros_like(x).reshape(-1)
        e[int(k)] = h
        e = e.reshape(x.shape)
        fd = (f(x + e, g) - f(x - e, g)) / (2 * h)
        worst = max(worst, abs(fd - float(gx.reshape(-1)[int(k)])) / scale_x)
    assert worst <= 1e-4, worst
    scale_g = float(gg.abs().max())
    worst = 0.0
    for a in (0, 17, 64, 127):
        for d, part in ((1.0, 'real'), (1j, 'imag')):
            e = torch.zeros_like(g)
            e[a] = h * d
            fd = (f(x, g + e) - f(x, g - e)) / (2 * h)
            worst = max(worst, abs(fd - float(getattr(gg[a], part))) / scale_g)
    assert worst <= 1e-4, worst


def test_c4_fp32c_gradients_close_to_fp64(arl, c4):
    res = {}
    for p in ('fp64', 'fp32c'):
        op = c4['ops'][p]
        res[p] = arl.autograd.gain_chi2_step(c4['x0'], c4['g0'], c4['vobs'], op, c4['a1'], c4['a2'])
    r64, r32 = res['fp64'], res['fp32c']
    assert abs(float(r32[0]) - float(r64[0])) <= 1e-5 * abs(float(r64[0]))
    assert float((r32[2] - r64[2]).abs().max() / r64[2].abs().max()) < 1e-4
    gcf = c4['ops']['fp64'].gcf
    inner = gcf <= 100.0
    d = (r32[1] - r64[1]).abs()
    assert float(d[inner].max() / r64[1].abs().max()) < 1e-4
