"""Host-side logic of the package that needs no GPU: WCS, descriptors, the
synthetic-observation generator, plane supports and w-slices."""
import numpy
import pytest


def test_wcs_linear_transforms(arl, oracle):
    w = arl.WCS(2)
    w.wcs.crval = [0.0, 10.0]
    w.wcs.crpix = [513.0, 3.0]
    w.wcs.cdelt = [-1.953125, 0.25]
    x = numpy.linspace(-900, 900, 101)
    p = w.wcs_world2pix(x, x, 0)
    assert numpy.array_equal(p[0], oracle.world2pix0(x, 0.0, 513.0, -1.953125))
    assert numpy.array_equal(p[1], oracle.world2pix0(x, 10.0, 3.0, 0.25))
    back = w.wcs_pix2world(p[0], p[1], 0)
    assert numpy.allclose(back[0], x) and numpy.allclose(back[1], x)
    sub = w.sub([2])
    assert sub.axis(0) == (10.0, 3.0, 0.25)


def test_descriptors_match_oracle_geometry(arl, oracle):
    im = arl.create_image(npixel=256, cellsize=2e-3, frequency=numpy.array([1e8, 1.1e8]),
                          channel_bandwidth=numpy.array([1e7, 1e7]),
                          polarisation_frame=arl.PolarisationFrame('stokesIQ'))
    gd = arl.create_griddata_from_image(im)
    cf = arl.create_convolutionfunction_from_image(im, nz=5, zstep=12.5, oversampling=8, support=8)
    g = arl.device.grid_desc(gd.grid_wcs, gd.data.shape)
    c = arl.device.cf_desc(cf.grid_wcs, cf.data.shape, 0, 0)
    img = oracle.image_geometry(256, 2e-3, 2, 2, 1e8, 1e7)
    gax, cax = oracle.grid_axes(img), oracle.cf_axes(img, 8, 8, nz=5, zstep=12.5)
    for name, ax in (('u', g.u), ('v', g.v), ('w', g.w), ('f', g.f)):
        assert (ax.crval, ax.crpix, ax.cdelt) == gax[name], name
    for name, ax in (('du', c.du), ('dv', c.dv), ('z', c.z)):
        assert (ax.crval, ax.crpix, ax.cdelt) == cax[name], name
    assert (g.nchan, g.npol, g.nw, g.ny, g.nx) == gax['shape']
    assert (c.nchan, c.npol, c.nz, c.oversampling, c.support) == (2, 2, 5, 8, 8)


def test_rows_follow_create_visibility_order(arl):
    sim = arl.simulation if hasattr(arl, 'simulation') else __import__('importlib').import_module(
        'algorithm-reference-library_gb300.simulation')
    rng = numpy.random.default_rng(3)
    xyz = sim.antennas_in_disk(5, 1000.0, rng)
    ha = numpy.array([-0.1, 0.0, 0.2])
    freqs = [1e8, 1.2e8]
    uvw, f, a1, a2, t = sim.rows(xyz, ha, freqs)
    # create_visibility's loops (processing_components/visibility/base.py:111-129)
    row = 0
    for it, h in enumerate(ha):
        pos = sim.xyz_to_uvw(xyz, h, numpy.deg2rad(-45.0))
        for i in range(5):
            for j in range(i + 1, 5):
                for ch, fr in enumerate(freqs):
                    assert a1[row] == i and a2[row] == j and t[row] == it and f[row] == fr
                    assert numpy.array_equal(uvw[row], (pos[j] - pos[i]) * (fr / sim.C_M_S))
                    row += 1
    assert row == uvw.shape[0]


def test_uv_cut_keeps_window_inside(arl, oracle):
    sim = __import__('importlib').import_module('algorithm-reference-library_gb300.simulation')
    w = sim.make_workload('C1', max_rows=5000)
    img = oracle.image_geometry(w['npixel'], w['cellsize'])
    gax, cax = oracle.grid_axes(img), oracle.cf_axes(img, w['oversampling'], w['support'])
    maps = oracle.convolution_mapping(w['uvw'], w['frequency'], gax, cax)
    assert numpy.all(oracle.rows_in_grid(maps, gax['shape'], cax['shape']))


def test_plane_support_zeroes_outside_taps(arl):
    im = arl.create_image(npixel=64, cellsize=8e-3)
    cf = arl.create_convolutionfunction_from_image(im, nz=3, oversampling=2, support=8)
    cf.data[...] = 1.0
    arl.set_plane_support(cf, [8, 4, 2])
    assert numpy.all(cf.data[0, 0, 0] == 1.0)
    assert cf.data[0, 0, 1].sum() == 2 * 2 * 4 * 4 and cf.data[0, 0, 1, 0, 0, 2:6, 2:6].min() == 1.0
    assert cf.data[0, 0, 2].sum() == 2 * 2 * 2 * 2 and cf.data[0, 0, 2, 1, 1, 3:5, 3:5].min() == 1.0
    with pytest.raises(AssertionError):
        arl.set_plane_support(cf, [8, 3, 2])


def test_support_schedule(arl):
    s = arl.support_schedule(numpy.arange(-32, 32) * 10.0, 8, 32)
    assert s.min() == 8 and s.max() == 32 and numpy.all(s % 2 == 0)
    assert s[32] == 8 and s[0] == 32


def test_wslice_iterator_matches_oracle(arl, oracle):
    rng = numpy.random.default_rng(9)
    n = 500
    v = arl.Visibility(uvw=rng.normal(size=(n, 3)) * 50, frequency=numpy.full(n, 1e8), vis=numpy.zeros((n, 1)),
                       weight=numpy.ones((n, 1)))
    got = list(arl.vis_wslice_iter(v, 7))
    want = oracle.wslice_rows(v.w, 7)
    assert len(got) == len(want) and all(numpy.array_equal(a, b) for a, b in zip(got, want))


def test_slice_axis_matches_wslice_iter(arl, oracle):
    """The w-stack grid axis gives every row the slice ARL's vis_wslice_iter
    does.  Rows within rounding of a half-way point (where ARL's strict
    |w - box| < step / 2 may count a row in neither or both neighbours, e.g.
    w = 0 with an even slice count) go to exactly one, by round-half-even."""
    import importlib
    import torch
    slice_axis = importlib.import_module(arl.__name__ + '.wstack').slice_axis
    rng = numpy.random.default_rng(10)
    for K in (2, 7, 8, 32):
        w = numpy.concatenate([rng.uniform(-300, 300, 5000), [300.0, 0.0, -0.0, 1e-13]])
        crval, crpix, cdelt = slice_axis(torch.as_tensor(w), K)
        p = ((w - crval) / cdelt + crpix) - 1.0
        idx = numpy.round(p).astype(int)
        assert numpy.all((idx >= 0) & (idx < K))
        near = numpy.abs(p - numpy.floor(p) - 0.5) < 1e-9
        for k, m in enumerate(oracle.wslice_rows(w, K)):
            assert numpy.array_equal(m[~near], (idx == k)[~near])


def test_phasecentre_lmn(arl):
    a = arl.PhaseCentre(10.0, -45.0)
    assert a.separation_rad(a) == 0.0
    b = arl.PhaseCentre(10.5, -44.0)
    l, m, n1 = b.lmn(a)
    assert l > 0 and m > 0 and n1 < 0
    assert abs(l * l + m * m + (n1 + 1) ** 2 - 1.0) < 1e-14


def test_sparse_oracle_matches_dense(oracle):
    """grid_sparse / degrid_windows (used where the grid is too large to hold
    densely on the host) agree with grid_vec / degrid_vec."""
    rng = numpy.random.default_rng(11)
    img = oracle.image_geometry(64, 4e-3, nchan=1, npol=2)
    gax = oracle.grid_axes(img, nw=3, wstep=10.0)
    cax = oracle.cf_axes(img, 8, 8)
    _, cf = oracle.create_pswf_cf(1, 2, 64, 64, 8, 8)
    lim = (32 - 4 - 2) / (64 * 4e-3)
    n = 500
    uvw = numpy.stack([rng.uniform(-lim, lim, n), rng.uniform(-lim, lim, n), rng.uniform(-14, 14, n)], axis=1)
    maps = oracle.convolution_mapping(uvw, numpy.full(n, 1e8), gax, cax)
    vis = rng.normal(size=(n, 2)) + 1j * rng.normal(size=(n, 2))
    wt = rng.uniform(0.5, 1.5, (n, 2))
    g, sw = oracle.grid_vec(vis, wt, maps, cf, gax['shape'])
    cells, vals, sw2 = oracle.grid_sparse(vis, wt, maps, cf, gax['shape'])
    dense = numpy.zeros(g.size, complex)
    dense[cells] = vals
    assert numpy.max(numpy.abs(dense - g.reshape(-1))) < 1e-12 * numpy.abs(g).max()
    assert numpy.allclose(sw, sw2, rtol=1e-15)
    win = g.reshape(-1)[oracle.window_index(maps, gax['shape'], 8)]
    d1 = oracle.degrid_windows(win, maps, cf)
    d2 = oracle.degrid_vec(g, maps, cf)
    assert numpy.max(numpy.abs(d1 - d2)) < 1e-12 * numpy.abs(d2).max()


def test_workload_shapes(arl):
    """C1-C5 rows: uv-cut keeps every window inside the grid; C3 drops flagged
    rows per channel; multi-frequency synthesis puts every channel on the one
    image channel."""
    sim = arl.simulation
    c3 = sim.make_workload('C3', max_rows=200000)
    for name in ('C1', 'C3', 'C4', 'C5'):
        w = c3 if name == 'C3' else sim.make_workload(name, max_rows=20000)
        lim = (w['npixel'] // 2 - w['support'] // 2 - 2) / (w['npixel'] * w['cellsize'])
        assert numpy.abs(w['uvw'][:, :2]).max() < lim
        if w.get('mfs'):
            p = numpy.round((w['frequency'] - w['image_frequency'][0]) / w['image_bandwidth'])
            assert numpy.all(p == 0)
    frac = 1.0 - c3['nrows_generated'] / (512 * 511 // 2 * 12 * 64)
    assert frac == 0.0
    counts = numpy.bincount(numpy.searchsorted(numpy.asarray(c3['freqs']), c3['frequency']), minlength=64)
    assert counts.min() < 0.7 * counts.max()  # uneven per-channel counts after flagging
    c4 = sim.make_workload('C4', max_rows=1000)
    assert c4['vis'] is None and c4['model_image'].shape == (1, 1, 2048, 2048)
    assert abs(numpy.abs(c4['gains']).mean() - 1.0) < 0.05


def test_clean_windows_and_psf_crop(arl):
    """deconvolve_cube's windows: 'quarter' keeps rows / columns q + 1 .. 3 q - 1
    (q = n // 4), 'no_edge' keeps edge + 1 .. n - edge - 1; the PSF crop keeps
    2 support pixels around the centre (deconvolution.py:82-113)."""
    import numpy
    dc = arl.deconvolution
    w = dc.clean_window((1, 1, 32, 20), 'quarter')
    rows, cols = numpy.nonzero(w[0, 0])
    assert (rows.min(), rows.max(), cols.min(), cols.max()) == (9, 23, 6, 14)
    assert w.sum() == 15 * 9
    w = dc.clean_window((2, 1, 32, 20), 'no_edge', 3)
    rows, cols = numpy.nonzero(w[1, 0])
    assert (rows.min(), rows.max(), cols.min(), cols.max()) == (4, 28, 4, 16)
    assert dc.clean_window((1, 1, 8, 8), 'no_edge', 6).sum() == 0
    assert dc.clean_window((1, 1, 8, 8), None) is None
    with pytest.raises(ValueError):
        dc.clean_window((1, 1, 8, 8), 'circle')
    psf = arl.create_image_from_array(numpy.arange(16 * 12, dtype=float).reshape(1, 1, 16, 12),
                                      arl.create_image(npixel=16).wcs, arl.PolarisationFrame('stokesI'))
    full = psf.data.copy()
    dc.crop_psf_to_support(psf, 4)
    assert psf.data.shape == (1, 1, 8, 8) and numpy.array_equal(psf.data, full[..., 4:12, 2:10])
    dc.crop_psf_to_support(psf, 5)  # larger than half the cropped PSF: unchanged
    assert psf.data.shape == (1, 1, 8, 8)


def test_uvw_reprojection_matches_reference(arl, golden):
    """phaserotate_visibility(tangent=False)'s uvw re-projection through earth
    coordinates (coordinate_support.py:59-113), on the CPU: the reference's
    rotated uvw for the phase-rotation rows, forward and inverse (the same
    rotation: both move the rows to the new phase centre's tangent plane)."""
    import numpy
    import torch
    d = golden('ref_rowops.npz')
    g = golden('ref_rotate_uvw.npz')
    old, new = arl.PhaseCentre(*d['rot_vis_pc']), arl.PhaseCentre(*d['rot_far_pc'])
    got = arl.imaging._reproject_uvw(torch.as_tensor(d['rot_uvw']), old, new).numpy()
    for tag in ('fwd', 'inv'):
        want = g['uvw_' + tag]
        assert numpy.max(numpy.abs(got - want)) <= 1e-13 * numpy.max(numpy.abs(want))
