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
