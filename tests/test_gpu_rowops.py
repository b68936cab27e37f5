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


# ---------------------------------------------------------------------------
# Against the reference's own outputs (tests/golden/ref_rowops.npz)
# ---------------------------------------------------------------------------
def test_phase_rotation_matches_reference(arl, golden):
    """shift_vis_to_image (both directions) and phaserotate_visibility to a
    far phase centre, against the reference's results with its own
    skycoord_to_lmn.  FP64 1e-10, as the DFT tests: the package forms l and m
    with the direct spherical-trigonometry formula and the reference through
    astropy's rotation matrices; both lose ~1e-16 absolute to cancellation,
    which baselines of ~2e3 wavelengths turn into ~1e-12 of phase.  FP32C 1e-6."""
    d = golden('ref_rowops.npz')
    frame = arl.PolarisationFrame('stokesIQ')
    n = d['rot_uvw'].shape[0]
    vis = arl.Visibility(uvw=d['rot_uvw'], frequency=numpy.full(n, 1e8), vis=d['rot_vis'].copy(),
                         weight=numpy.ones((n, 2)), polarisation_frame=frame)
    vis.phasecentre = arl.PhaseCentre(*d['rot_vis_pc'])
    im = arl.create_image(npixel=64, cellsize=1e-3, phasecentre=arl.PhaseCentre(*d['rot_im_pc']),
                          polarisation_frame=frame)
    fwd = arl.shift_vis_to_image(vis, im, tangent=True, inverse=False)
    assert rel(fwd.vis, d['rot_fwd']) < 1e-10
    assert (fwd.phasecentre.ra_deg, fwd.phasecentre.dec_deg) == tuple(d['rot_im_pc'])
    assert (vis.phasecentre.ra_deg, vis.phasecentre.dec_deg) == tuple(d['rot_vis_pc'])
    inv = arl.shift_vis_to_image(vis, im, tangent=True, inverse=True)
    assert rel(inv.vis, d['rot_inv']) < 1e-10
    far = arl.phaserotate_visibility(vis, arl.PhaseCentre(*d['rot_far_pc']), tangent=True)
    assert rel(far.vis, d['rot_far']) < 1e-10
    assert numpy.array_equal(vis.vis, d['rot_vis'])  # the input is not modified
    dvis = arl.DeviceVisibility.from_visibility(vis, 'fp32c')
    dvis.phasecentre = vis.phasecentre
    dfwd = arl.shift_vis_to_image(dvis, im)
    assert rel(dfwd.vis.to(torch.complex128).cpu().numpy(), d['rot_fwd']) < 1e-6


@pytest.mark.parametrize('inverse', [False, True])
def test_phase_rotation_off_tangent_matches_reference(arl, golden, inverse):
    """phaserotate_visibility(tangent=False) to a far phase centre: phases as on
    the tangent plane (FP64 1e-10, as above), uvw re-projected through earth
    coordinates (1e-13) and the new phase centre, against the reference's
    results; a DeviceVisibility gets the same uvw."""
    d = golden('ref_rowops.npz')
    g = golden('ref_rotate_uvw.npz')
    tag = 'inv' if inverse else 'fwd'
    frame = arl.PolarisationFrame('stokesIQ')
    n = d['rot_uvw'].shape[0]
    vis = arl.Visibility(uvw=d['rot_uvw'], frequency=numpy.full(n, 1e8), vis=d['rot_vis'].copy(),
                         weight=numpy.ones((n, 2)), polarisation_frame=frame)
    vis.phasecentre = arl.PhaseCentre(*d['rot_vis_pc'])
    new = arl.PhaseCentre(*d['rot_far_pc'])
    out = arl.phaserotate_visibility(vis, new, tangent=False, inverse=inverse)
    assert rel(out.vis, g['vis_' + tag]) < 1e-10
    assert rel(out.uvw, g['uvw_' + tag]) < 1e-13
    assert (out.phasecentre.ra_deg, out.phasecentre.dec_deg) == tuple(g['pc_' + tag])
    assert numpy.array_equal(vis.uvw, d['rot_uvw'])  # the input is not modified
    dvis = arl.DeviceVisibility.from_visibility(vis, 'fp64')
    dvis.phasecentre = vis.phasecentre
    dout = arl.phaserotate_visibility(dvis, new, tangent=False, inverse=inverse)
    assert rel(dout.uvw.cpu().numpy(), g['uvw_' + tag]) < 1e-13
    assert rel(dout.vis.cpu().numpy(), g['vis_' + tag]) < 1e-10


@pytest.mark.parametrize('precision,tol', [('fp64', 1e-10), ('fp32c', 1e-6)])
def test_skycomponents_match_reference(arl, golden, precision, tol):
    """predict_skycomponent_visibility on rows (3 channels, 2 polarisations) and
    on a BlockVisibility, against the reference's results (tolerances of
    test_gpu_dft.py)."""
    d = golden('ref_rowops.npz')
    frame = arl.PolarisationFrame('linearnp')
    freqs = numpy.unique(d['dft_freq'])
    comps = [arl.Skycomponent(direction=arl.PhaseCentre(*dr), frequency=freqs, flux=fl, polarisation_frame=frame)
             for dr, fl in zip(d['dft_dir'], d['dft_flux'])]
    n = d['dft_uvw'].shape[0]
    vis = arl.Visibility(uvw=d['dft_uvw'], frequency=d['dft_freq'], vis=d['dft_base'].copy(),
                         weight=numpy.ones((n, 2)), polarisation_frame=frame)
    vis.phasecentre = arl.PhaseCentre(*d['dft_pc'])
    arl.predict_skycomponent_visibility(vis, comps, precision=precision)
    assert rel(vis.vis, d['dft_vis']) < tol
    base = d['dftb_base']
    ntimes = base.shape[0]
    bv = arl.BlockVisibility(frequency=freqs, channel_bandwidth=numpy.full(3, 1e7),
                             phasecentre=arl.PhaseCentre(*d['dft_pc']), uvw=d['dftb_uvw'],
                             time=numpy.arange(ntimes) * 30.0, vis=base.copy(), weight=numpy.ones(base.shape),
                             integration_time=numpy.full(ntimes, 30.0), polarisation_frame=frame)
    arl.predict_skycomponent_visibility(bv, comps, precision=precision)
    assert rel(bv.vis, d['dftb_vis']) < tol


@pytest.mark.parametrize('precision,tol', [('fp64', 1e-12), ('fp32c', 1e-6)])
def test_apply_gaintable_matches_reference(arl, golden, precision, tol):
    """apply_gaintable with scalar gains on a BlockVisibility, forward and
    inverse, with zero gain weights and a zero gain, against the reference."""
    d = golden('ref_rowops.npz')
    gshape = d['gt_vis'].shape
    ntimes, nant, _, nchan, _ = gshape
    gt = arl.GainTable(gain=d['gt_gain'], time=d['gt_time'], interval=d['gt_interval'], weight=d['gt_weight'],
                       residual=numpy.zeros((ntimes, nchan, 1, 1)), frequency=d['gt_freqs'],
                       receptor_frame=arl.ReceptorFrame('stokesI'))
    for inverse, key in ((False, 'gt_fwd'), (True, 'gt_inv')):
        bv = arl.BlockVisibility(frequency=d['gt_freqs'], channel_bandwidth=numpy.full(nchan, 1e7),
                                 phasecentre=arl.PhaseCentre(0.0, -45.0), uvw=numpy.zeros((ntimes, nant, nant, 3)),
                                 time=d['gt_time'], vis=d['gt_vis'].copy(), weight=numpy.ones(gshape),
                                 integration_time=numpy.full(ntimes, 30.0))
        out = arl.apply_gaintable(bv, gt, inverse=inverse, precision=precision)
        assert out is bv
        assert rel(bv.vis, d[key]) < tol, (inverse, precision)
