"""Point-component (DFT) predict against the oracle's simulate_point sums, on
Visibility rows with several channels and polarisations and on a
BlockVisibility; the DFT adjoint against the predict (adjointness).

Tolerances: FP64 1e-10 relative (the GPU reduces the phase in turns before
the sine and cosine, NumPy takes exp of the full argument: both round
differently at ~1e-12 for these phases); FP32C 1e-6 (FP32 sine and cosine of
the reduced phase, FP32 sums over components)."""
import numpy
import pytest
import torch

from helpers import rel

pytestmark = pytest.mark.gpu

TOL = {'fp64': 1e-10, 'fp32c': 1e-6}


@pytest.fixture(scope='module', autouse=True)
def need_cuda(arl):
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    arl._native.load()


def _components(arl, rng, n, nchan, npol):
    pc = arl.PhaseCentre(0.0, -45.0)
    comps = []
    for _ in range(n):
        d = arl.PhaseCentre(rng.uniform(-4, 4), -45.0 + rng.uniform(-4, 4))
        comps.append(arl.Skycomponent(direction=d, frequency=numpy.linspace(1e8, 1.2e8, nchan),
                                      flux=rng.uniform(0.1, 5.0, (nchan, npol))))
    return pc, comps


def _oracle_predict(oracle, uvw, chan, comps, pc, npol):
    out = numpy.zeros((uvw.shape[0], npol), dtype=complex)
    for c in comps:
        l, m, _ = c.direction.lmn(pc)
        out += c.flux[chan, :] * oracle.simulate_point(uvw, l, m)[:, None]
    return out


@pytest.mark.parametrize('precision', ['fp64', 'fp32c'])
def test_dft_predict_rows_vs_oracle(arl, oracle, precision):
    rng = numpy.random.default_rng(81)
    n, nchan, npol = 50000, 3, 2
    freqs = numpy.array([1.0e8, 1.1e8, 1.2e8])
    f = rng.choice(freqs, n)
    uvw = rng.uniform(-4000, 4000, (n, 3)) * numpy.array([1, 1, 0.1])
    pc, comps = _components(arl, rng, 12, nchan, npol)
    base = rng.normal(size=(n, npol)) + 1j * rng.normal(size=(n, npol))
    vis = arl.Visibility(uvw=uvw, frequency=f, vis=base.copy(), weight=numpy.ones((n, npol)),
                         polarisation_frame=arl.PolarisationFrame('linearnp'))
    vis.phasecentre = pc
    arl.predict_skycomponent_visibility(vis, comps, precision=precision)
    chan = numpy.searchsorted(freqs, f)
    want = base + _oracle_predict(oracle, uvw, chan, comps, pc, npol)
    assert rel(vis.vis, want) < TOL[precision]
    # the same on device-resident rows
    dvis = arl.DeviceVisibility.from_visibility(
        arl.Visibility(uvw=uvw, frequency=f, vis=base.copy(), weight=numpy.ones((n, npol)),
                       polarisation_frame=arl.PolarisationFrame('linearnp')), precision)
    dvis.phasecentre = pc
    arl.predict_skycomponent_visibility(dvis, comps)
    assert rel(dvis.vis.to(torch.complex128).cpu().numpy(), want) < TOL[precision]


def test_dft_predict_blockvisibility(arl, oracle):
    rng = numpy.random.default_rng(82)
    nt, nant, nchan, npol = 4, 7, 3, 1
    freqs = numpy.linspace(1.0e8, 1.2e8, nchan)
    uvw = rng.uniform(-300, 300, (nt, nant, nant, 3))
    pc, comps = _components(arl, rng, 5, nchan, npol)
    bv = arl.BlockVisibility(frequency=freqs, channel_bandwidth=numpy.full(nchan, 1e7), phasecentre=pc, uvw=uvw,
                             time=numpy.arange(nt) * 1.0, vis=numpy.zeros((nt, nant, nant, nchan, npol), complex))
    arl.predict_skycomponent_visibility(bv, comps)
    want = numpy.zeros((nt, nant, nant, nchan, npol), complex)
    for c in comps:
        l, m, _ = c.direction.lmn(pc)
        for ch in range(nchan):
            ph = oracle.simulate_point(uvw * (freqs[ch] / oracle.C_M_S), l, m)
            want[..., ch, :] += c.flux[ch, :] * ph[..., None]
    assert rel(bv.vis, want) < TOL['fp64']


@pytest.mark.parametrize('precision', ['fp64', 'fp32c'])
def test_dft_adjoint(arl, precision):
    """Re <D x, y> = <x, D^H y> for real component fluxes x and complex rows y."""
    sky = arl.skycomponents
    dev = torch.device('cuda')
    rng = numpy.random.default_rng(83)
    n, ncomp = 20000, 300
    uvw = torch.as_tensor(rng.uniform(-2000, 2000, (n, 3)) * numpy.array([1, 1, 0.1]), device=dev)
    l = rng.uniform(-0.05, 0.05, ncomp)
    m = rng.uniform(-0.05, 0.05, ncomp)
    lmn = torch.as_tensor(numpy.stack([l, m, numpy.sqrt(1 - l ** 2 - m ** 2) - 1], axis=1), device=dev)
    x = rng.normal(size=(ncomp, 1, 1))
    cdt = arl.device.CDTYPE[precision]
    v = torch.zeros((n, 1), dtype=cdt, device=dev)
    sky.dft_predict(uvw, None, lmn, torch.as_tensor(x, device=dev), v, precision)
    y = torch.as_tensor(rng.normal(size=(n, 1)) + 1j * rng.normal(size=(n, 1)), device=dev).to(cdt)
    img = sky.dft_adjoint(uvw, lmn, y, precision)
    lhs = float((torch.conj(y.to(torch.complex128)) * v.to(torch.complex128)).real.sum())
    rhs = float((torch.as_tensor(x[:, :, 0], device=dev) * img).sum())
    scale = float(torch.linalg.norm(y.to(torch.complex128)) * torch.linalg.norm(v.to(torch.complex128)))
    assert abs(lhs - rhs) <= (1e-12 if precision == 'fp64' else 1e-6) * scale
