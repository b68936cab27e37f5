"""The oracle against outputs of the reference's own code (tests/golden/*.npz,
made by tests/golden/make_golden.py from the ARL sources)."""
import numpy
import pytest


def _rel(a, b):
    return numpy.max(numpy.abs(a - b)) / max(numpy.max(numpy.abs(b)), 1e-300)


def _maps(m):
    return tuple(m[i] for i in range(7))


def test_2d_pswf(oracle, golden):
    d = golden('ref_2d_pswf.npz')
    img = oracle.image_geometry(int(d['N']), float(d['cell']), 1, 1, float(d['freq0']), float(d['dfreq']))
    gax, cax = oracle.grid_axes(img), oracle.cf_axes(img, int(d['O']), int(d['S']))
    maps = oracle.convolution_mapping(d['uvw'], d['frequency'], gax, cax)
    for a, b in zip(maps, _maps(d['maps'])):
        assert numpy.array_equal(a, b)
    gcf, cf = oracle.create_pswf_cf(1, 1, int(d['N']), int(d['N']), int(d['O']), int(d['S']))
    assert numpy.array_equal(cf, d['cf']) and numpy.array_equal(gcf, d['gcf'])
    g, sw = oracle.grid_loop(d['vis'], d['wt'], maps, cf, gax['shape'])
    assert numpy.array_equal(g, d['grid']) and numpy.array_equal(sw, d['sumwt'])
    g2, _ = oracle.grid_vec(d['vis'], d['wt'], maps, cf, gax['shape'])
    assert _rel(g2, d['grid']) < 1e-14
    im = oracle.fft_griddata_to_image(d['grid'], d['gcf'])
    assert numpy.array_equal(im.real, d['img_re']) and numpy.array_equal(im.imag, d['img_im'])
    assert numpy.array_equal(oracle.fft_image_to_griddata(d['model'], d['gcf']), d['grid_model'])
    assert numpy.array_equal(oracle.degrid_loop(d['grid_model'], maps, cf), d['degrid'])
    assert _rel(oracle.degrid_vec(d['grid_model'], maps, cf), d['degrid']) < 1e-14
    dirty, sw2 = oracle.invert_2d(d['uvw'], d['frequency'], d['vis'], d['wt'], img, gcf, cf, cax)
    assert _rel(dirty.real, d['dirty']) < 1e-14 and numpy.array_equal(sw2, d['sumwt_dirty'])
    psf, _ = oracle.invert_2d(d['uvw'], d['frequency'], d['vis'], d['wt'], img, gcf, cf, cax, dopsf=True)
    assert _rel(psf.real, d['psf']) < 1e-14
    pv = oracle.predict_2d(d['uvw'], d['frequency'], d['model'], img, gcf, cf, cax)
    assert _rel(pv, d['predict']) < 1e-14


def test_wproj_2chan_2pol(oracle, golden):
    d = golden('ref_wproj_2chan_2pol.npz')
    img = oracle.image_geometry(int(d['N']), float(d['cell']), 2, 2, float(d['freqs'][0]), float(d['dfreq']))
    gax = oracle.grid_axes(img)
    cax = oracle.cf_axes(img, int(d['O']), int(d['S']), nz=int(d['nw']), zstep=float(d['wstep']))
    maps = oracle.convolution_mapping(d['uvw'], d['frequency'], gax, cax)
    for a, b in zip(maps, _maps(d['maps'])):
        assert numpy.array_equal(a, b)
    gcf, cf = oracle.create_awterm_cf(img, nw=int(d['nw']), wstep=float(d['wstep']), oversampling=int(d['O']),
                                      support=int(d['S']), maxsupport=64)
    assert numpy.array_equal(cf, d['cf']) and numpy.array_equal(gcf, d['gcf'])
    g, sw = oracle.grid_loop(d['vis'], d['wt'], maps, cf, gax['shape'])
    assert numpy.array_equal(g, d['grid']) and numpy.array_equal(sw, d['sumwt'])
    assert _rel(oracle.degrid_vec(d['rgrid'], maps, cf), d['degrid']) < 1e-14
    im = oracle.fft_griddata_to_image(d['grid'], d['gcf'])
    assert numpy.array_equal(im.real, d['img_re'])


def test_wstack_workflow(oracle, golden):
    d = golden('ref_wstack.npz')
    img = oracle.image_geometry(int(d['N']), float(d['cell']), 1, 1, float(d['freq0']), float(d['dfreq']))
    cax = oracle.cf_axes(img, int(d['O']), int(d['S']))
    gcf, cf = oracle.create_pswf_cf(1, 1, int(d['N']), int(d['N']), int(d['O']), int(d['S']))
    assert numpy.array_equal(cf, d['cf'])
    dirty, sw = oracle.invert_wstack(d['uvw'], d['frequency'], d['vis'], d['wt'], img, gcf, cf, cax,
                                     int(d['K']), float(d['cell']))
    assert _rel(dirty, d['dirty']) < 1e-13 and numpy.array_equal(sw, d['sumwt'])
    pv = oracle.predict_wstack(d['uvw'], d['frequency'], d['model'], img, gcf, cf, cax, int(d['K']), float(d['cell']))
    assert _rel(pv, d['predict']) < 1e-13


def test_kernels(oracle, golden):
    d = golden('ref_kernels.npz')
    img = oracle.image_geometry(512, 0.0005)
    _, cf8 = oracle.create_pswf_cf(1, 1, 512, 512, 8, 6)
    _, cf1 = oracle.create_pswf_cf(1, 1, 512, 512, 1, 6)
    assert numpy.array_equal(cf8[0, 0, 0], d['pswf8']) and numpy.array_equal(cf1[0, 0, 0], d['pswf1'])
    gcf, cfw = oracle.create_awterm_cf(img, nw=9, wstep=8.0, oversampling=8, support=16)
    assert numpy.array_equal(cfw[0, 0], d['wker']) and numpy.array_equal(gcf[0, 0], d['gcf'])
    bb = oracle.bounding_box(cfw, 1e-3)
    assert numpy.array_equal(numpy.array([[b[0], *b[1], *b[2]] for b in bb]), d['bbox'])


def test_uniform_weighting_matches_reference(oracle, golden):
    """grid_weight_to_griddata and weight_visibility, run by the reference."""
    d = golden('ref_weighting.npz')
    img = oracle.image_geometry(int(d['N']), float(d['cell']), 2, 2, float(d['freqs'][0]), float(d['dfreq']))
    gax = oracle.grid_axes(img)
    cax = oracle.cf_axes(img, int(d['O']), int(d['S']))
    maps = oracle.convolution_mapping(d['uvw'], d['frequency'], gax, cax)
    wgrid, sumwt = oracle.grid_weight(d['wt_before'], maps, gax['shape'])
    assert numpy.array_equal(wgrid, d['wgrid'])
    assert numpy.array_equal(sumwt, d['sumwt'])
    assert numpy.array_equal(oracle.weight_uniform(d['wt_before'], maps, gax['shape']), d['wt_after'])


@pytest.mark.parametrize('npol', [1, 2])
def test_block_conversion_matches_reference(oracle, golden, npol):
    """convert_blockvisibility_to_visibility and convert_visibility_to_blockvisibility."""
    d = golden('ref_blocks.npz')
    g = {k[3:]: d[k] for k in d.files if k.startswith('p%d_' % npol)}
    nt = g['times'].size
    out = oracle.convert_blocks(g['block_vis'], g['block_uvw'], g['block_weight'], g['block_imaging_weight'],
                                g['times'], numpy.full(nt, 30.0), g['freqs'], numpy.full(g['freqs'].size, 1e7))
    names = ('vis', 'uvw', 'weight', 'imaging_weight', 'time', 'frequency', None, 'antenna1', 'antenna2', None,
             'cindex')
    for name, arr in zip(names, out):
        if name is not None:
            assert numpy.array_equal(arr, g[name]), name
    for col, scale in (('vis', 2.0 + 1.0j), ('weight', 3.0), ('imaging_weight', 1.0)):
        back = oracle.decoalesce(g['block_' + col], g[col] * scale, g['cindex'])
        assert numpy.array_equal(back, g['back_' + col]), col


def test_hogbom_matches_reference(oracle, golden):
    """Hogbom CLEAN and deconvolve_cube(algorithm='hogbom'), run by the reference."""
    d = golden('ref_hogbom.npz')
    c1, r1 = oracle.hogbom(d['dirty'], d['psf'], None, 0.1, 0.0, 400, 0.01)
    assert numpy.array_equal(c1, d['c1']) and numpy.array_equal(r1, d['r1'])
    c2, r2 = oracle.hogbom(d['dirty'], d['psf'], d['window'], 0.7, 0.05, 300, 0.001)
    assert numpy.array_equal(c2, d['c2']) and numpy.array_equal(r2, d['r2'])
    comp, resid = oracle.deconvolve_hogbom(d['d2'], d['p2'].copy(), niter=200, gain=0.2, threshold=0.0,
                                           fractional_threshold=0.05, window_shape='quarter', psf_support=40)
    assert numpy.array_equal(comp, d['cube_comp']) and numpy.array_equal(resid, d['cube_resid'])


def test_msclean_matches_reference(oracle, golden):
    """Multiscale CLEAN, run by the reference."""
    h = golden('ref_hogbom.npz')
    d = golden('ref_msclean.npz')
    c1, r1 = oracle.msclean(h['dirty'], h['psf'], None, 0.3, 0.0, 150, [0, 3, 10], 0.01)
    assert numpy.array_equal(c1, d['c1']) and numpy.array_equal(r1, d['r1'])
    c2, r2 = oracle.msclean(h['dirty'], h['psf'][32:96, 32:96], h['window'], 0.7, 0.02, 100, [0, 3], 0.001)
    assert numpy.array_equal(c2, d['c2']) and numpy.array_equal(r2, d['r2'])


# ---------------------------------------------------------------------------
# Row operations (ref_rowops.npz): direction cosines, phase rotation, point
# components, scalar gains
# ---------------------------------------------------------------------------
def test_rowops_lmn(oracle, golden, arl):
    """skycoord_to_lmn: the oracle's sky-offset rotation and the package's
    direction-cosine formula (PhaseCentre.lmn) against the reference's values."""
    d = golden('ref_rowops.npz')
    for pc, dr, want in zip(d['lmn_pc'], d['lmn_dir'], d['lmn']):
        got = oracle.skycoord_to_lmn(dr[0], dr[1], pc[0], pc[1])
        assert numpy.max(numpy.abs(numpy.array(got) - want)) < 1e-15
        got2 = arl.PhaseCentre(dr[0], dr[1]).lmn(arl.PhaseCentre(pc[0], pc[1]))
        assert numpy.max(numpy.abs(numpy.array(got2) - want)) < 1e-14
    l, m, n1 = oracle.skycoord_to_lmn(*d['rot_im_pc'], *d['rot_vis_pc'])
    assert numpy.max(numpy.abs(numpy.array([l, m, n1]) - d['rot_lmn'])) < 1e-15


def test_rowops_phaserotate(oracle, golden):
    """Phases of up to ~1e3 rad: the last-bit differences of l and m (the
    stand-in's rotation against the oracle's) give ~1e-13 relative."""
    d = golden('ref_rowops.npz')
    l, m, _ = oracle.skycoord_to_lmn(*d['rot_im_pc'], *d['rot_vis_pc'])
    assert _rel(oracle.phaserotate(d['rot_vis'], d['rot_uvw'], l, m), d['rot_fwd']) < 1e-12
    assert _rel(oracle.phaserotate(d['rot_vis'], d['rot_uvw'], l, m, inverse=True), d['rot_inv']) < 1e-12
    l, m, _ = oracle.skycoord_to_lmn(*d['rot_far_pc'], *d['rot_vis_pc'])
    assert _rel(oracle.phaserotate(d['rot_vis'], d['rot_uvw'], l, m), d['rot_far']) < 1e-12


def test_rowops_skycomponents(oracle, golden):
    d = golden('ref_rowops.npz')
    freqs = numpy.unique(d['dft_freq'])
    chan = numpy.searchsorted(freqs, d['dft_freq'])
    want = d['dft_base'].copy()
    for dr, fl in zip(d['dft_dir'], d['dft_flux']):
        l, m, _ = oracle.skycoord_to_lmn(dr[0], dr[1], *d['dft_pc'])
        want += fl[chan, :] * oracle.simulate_point(d['dft_uvw'], l, m)[:, None]
    assert _rel(want, d['dft_vis']) < 1e-10  # phases up to ~1e3 rad, as in test_gpu_dft.py
    # blocks: uvw in metres times f / c per channel
    want = d['dftb_base'].copy()
    k = freqs / oracle.C_M_S
    for dr, fl in zip(d['dft_dir'], d['dft_flux']):
        l, m, _ = oracle.skycoord_to_lmn(dr[0], dr[1], *d['dft_pc'])
        for c in range(freqs.size):
            want[..., c, :] += fl[c, :] * oracle.simulate_point(d['dftb_uvw'] * k[c], l, m)[..., None]
    assert _rel(want, d['dftb_vis']) < 1e-10


def test_rowops_gaintable(oracle, golden, arl):
    """The package's slice / gain-row bookkeeping (host logic) with the oracle's
    block update reproduces the reference's apply_gaintable, both directions."""
    d = golden('ref_rowops.npz')
    passes = arl.calibration.gain_rows_per_pass(d['gt_time'], d['gt_time'], d['gt_interval'])
    assert len(passes) == 1 and list(passes[0]) == [0, 1, 2, 3]
    gain, gwt = d['gt_gain'][..., 0, 0], d['gt_weight'][..., 0, 0]
    for inverse, key in ((False, 'gt_fwd'), (True, 'gt_inv')):
        out = d['gt_vis'][..., 0]
        for trow in passes:
            out = oracle.apply_gaintable_block(out, trow, gain, gwt, inverse)
        assert _rel(out, d[key][..., 0]) < 1e-14
    # Two slices of two times, one gain row each: one pass.  Two gain rows per
    # slice with a time on the slice boundary (t = 5 lies in both slices):
    # the second slice's first time collides with the first slice's second
    # time, so it starts a second pass and that time is updated twice.
    t = numpy.array([0.0, 10.0, 20.0, 30.0])
    p = arl.calibration.gain_rows_per_pass(t, numpy.array([5.0, 25.0]), numpy.array([20.0, 20.0]), vis_slices=2)
    assert [x.tolist() for x in p] == [[0, -1, 1, -1]]
    t = numpy.array([0.0, 5.0, 10.0])
    p = arl.calibration.gain_rows_per_pass(t, numpy.array([2.5, 2.5, 7.5, 7.5]), numpy.full(4, 10.0), vis_slices=2)
    assert [x.tolist() for x in p] == [[0, 1, -1], [-1, 2, 3]]
