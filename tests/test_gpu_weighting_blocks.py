"""Uniform weighting and BlockVisibility conversion on the GPU against the
reference's own outputs (tests/golden/ref_weighting.npz, ref_blocks.npz) and
the oracle.

Tolerances: the weight grid is summed with FP64 atomics, so a cell that sums
several non-integer weights may differ from NumPy's sequential sum in the last
bit (1e-15 relative); the conversion is a pure gather plus one FP64 multiply
and is bit-identical.
"""
import numpy
import pytest
import torch

from helpers import rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module', autouse=True)
def need_cuda(arl):
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    arl._native.load()


def _weight_case(arl, d):
    im = arl.create_image(npixel=int(d['N']), cellsize=float(d['cell']), frequency=d['freqs'],
                          channel_bandwidth=numpy.array([float(d['dfreq'])]),
                          polarisation_frame=arl.PolarisationFrame('stokesIQ'),
                          phasecentre=arl.PhaseCentre(0.0, -45.0))
    gcfcf = arl.create_pswf_convolutionfunction(im, oversampling=int(d['O']), support=int(d['S']))
    n = d['uvw'].shape[0]
    vis = arl.Visibility(uvw=d['uvw'], frequency=d['frequency'], vis=numpy.zeros((n, 2), complex),
                         weight=d['wt_before'], imaging_weight=d['wt_before'].copy(),
                         polarisation_frame=arl.PolarisationFrame('stokesIQ'))
    return im, gcfcf, vis


def test_grid_weights_and_uniform_weighting_match_reference(arl, golden):
    d = golden('ref_weighting.npz')
    im, gcfcf, vis = _weight_case(arl, d)
    gd, sumwt = arl.grid_weight_to_griddata(vis, arl.create_griddata_from_image(im), gcfcf[1])
    assert rel(gd.data, d['wgrid']) < 1e-15
    assert rel(sumwt, d['sumwt']) < 1e-12  # ~1000 FP64 terms summed in a different order
    out = arl.weight_visibility(vis, im, gcfcf=gcfcf)
    assert out is vis
    assert rel(vis.imaging_weight, d['wt_after']) < 1e-15
    # griddata_reweight from the reference's own weight grid: identical inputs
    _, _, vis2 = _weight_case(arl, d)
    g = arl.create_griddata_from_image(im)
    g.data[...] = d['wgrid']
    arl.griddata_reweight(vis2, g, gcfcf[1])
    assert numpy.array_equal(vis2.imaging_weight, d['wt_after'])


def test_uniform_weighting_device_fp32c(arl, oracle, golden):
    d = golden('ref_weighting.npz')
    im, gcfcf, vis = _weight_case(arl, d)
    dvis = arl.DeviceVisibility.from_visibility(vis, 'fp32c')
    w0 = dvis.imaging_weight
    arl.weight_visibility(dvis, im, gcfcf=gcfcf)
    assert dvis.imaging_weight is w0 and w0.dtype == torch.float32
    assert rel(w0.cpu().numpy(), d['wt_after']) < 1e-6


def test_merge_weights(arl, golden):
    d = golden('ref_weighting.npz')
    im, gcfcf, vis = _weight_case(arl, d)
    a = arl.grid_weight_to_griddata(vis, arl.create_griddata_from_image(im), gcfcf[1])
    b = arl.grid_weight_to_griddata(vis, arl.create_griddata_from_image(im), gcfcf[1])
    m, sw = arl.griddata_merge_weights([a, b])
    assert numpy.allclose(m.data, 2 * d['wgrid'], rtol=1e-15, atol=0)
    assert numpy.allclose(sw, 2 * d['sumwt'], rtol=1e-12, atol=0)


def _block(arl, g, npol):
    frame = {1: 'stokesI', 2: 'linearnp'}[npol]
    nt = g['times'].size
    nchan = g['freqs'].size
    return arl.BlockVisibility(frequency=g['freqs'], channel_bandwidth=numpy.full(nchan, 1e7),
                               phasecentre=arl.PhaseCentre(0.0, -45.0), uvw=g['block_uvw'], time=g['times'],
                               vis=g['block_vis'], weight=g['block_weight'], integration_time=numpy.full(nt, 30.0),
                               polarisation_frame=arl.PolarisationFrame(frame),
                               imaging_weight=g['block_imaging_weight'])


@pytest.mark.parametrize('npol', [1, 2])
def test_block_conversion_matches_reference(arl, golden, npol):
    d = golden('ref_blocks.npz')
    g = {k[3:]: d[k] for k in d.files if k.startswith('p%d_' % npol)}
    bv = _block(arl, g, npol)
    v = arl.convert_blockvisibility_to_visibility(bv)
    for k in ('uvw', 'vis', 'weight', 'imaging_weight', 'time', 'frequency', 'antenna1', 'antenna2', 'cindex'):
        got = getattr(v, k) if k != 'cindex' else v.cindex
        assert numpy.array_equal(numpy.asarray(got), g[k]), k
    v.data['vis'] *= (2.0 + 1.0j)
    v.data['weight'] *= 3.0
    back = arl.convert_visibility_to_blockvisibility(v)
    for col in ('vis', 'weight', 'imaging_weight'):
        assert numpy.array_equal(back.data[col], g['back_' + col]), col


def test_device_rows_from_blocks_feed_the_gridder(arl, oracle):
    """A larger block (96 antennas, 6 times, 8 channels: 273,600 rows) converted
    on the device equals the oracle's conversion, and gridding those device
    rows equals gridding the host-converted Visibility."""
    rng = numpy.random.default_rng(71)
    nt, nant, nchan, npol = 6, 96, 8, 1
    freqs = numpy.linspace(1.0e8, 1.2e8, nchan)
    shape = (nt, nant, nant, nchan, npol)
    uvw = rng.uniform(-80.0, 80.0, (nt, nant, nant, 3))
    bvis = rng.normal(size=shape) + 1j * rng.normal(size=shape)
    wt = rng.uniform(0.5, 2.0, shape)
    bv = arl.BlockVisibility(frequency=freqs, channel_bandwidth=numpy.full(nchan, 2.5e6),
                             phasecentre=arl.PhaseCentre(0.0, -45.0), uvw=uvw, time=numpy.arange(nt) * 10.0,
                             vis=bvis, weight=wt, integration_time=numpy.full(nt, 10.0))
    ref = oracle.convert_blocks(bvis, uvw, wt, wt, numpy.arange(nt) * 10.0, numpy.full(nt, 10.0), freqs,
                                numpy.full(nchan, 2.5e6))
    dv = arl.DeviceVisibility.from_blockvisibility(bv, 'fp64')
    assert numpy.array_equal(dv.uvw.cpu().numpy(), ref[1])
    assert numpy.array_equal(dv.vis.cpu().numpy(), ref[0])
    assert numpy.array_equal(dv.antenna1.cpu().numpy(), ref[7]) and numpy.array_equal(dv.antenna2.cpu().numpy(),
                                                                                        ref[8])
    assert numpy.array_equal(dv.cindex.cpu().numpy(), ref[10])
    im = arl.create_image(npixel=256, cellsize=2e-3, frequency=numpy.array([1.1e8]),
                          channel_bandwidth=numpy.array([1e8]), phasecentre=arl.PhaseCentre(0.0, -45.0))
    gcf, cf = arl.create_pswf_convolutionfunction(im, oversampling=8, support=8)
    hv = arl.convert_blockvisibility_to_visibility(bv)
    g1, s1 = arl.grid_visibility_to_griddata(hv, arl.create_griddata_from_image(im), cf, precision='fp64')
    g2, s2 = arl.grid_visibility_to_griddata(dv, arl.create_griddata_on_device(im, precision='fp64'), cf,
                                             precision='fp64')
    assert rel(g2.data.cpu().numpy(), g1.data) < 1e-12
    assert numpy.allclose(s2.cpu().numpy(), s1, rtol=1e-12)
