"""Seeded synthetic observations with the shapes of the benchmark workloads.

Rows are generated the way ARL's ``create_visibility`` lays them out
(``processing_components/visibility/base.py:50-150``): for each hour angle,
each baseline (a1 < a2), each channel; uvw = (xyz[a2] - xyz[a1]) * f / c after
``xyz_to_uvw`` (``processing_library/util/coordinate_support.py:59-85``).
Antennas are uniform in a disk of the stated radius in the local horizontal
plane, rotated to celestial XYZ with ``xyz_at_latitude`` (:37-56).  The array
sits at latitude -45 deg observing dec -45 deg over +/-2 h, so no row falls
below ARL's 15 deg elevation limit.

No public dataset is involved: these stand in for ARL's LOWBD2 configuration
files with the sizes of each workload.
"""
import numpy
import torch

C_M_S = 299792458.0  # astropy.constants.c


def xyz_at_latitude(local_xyz, lat):
    """Local (east, north, up) -> celestial XYZ (coordinate_support.py:37-56)."""
    x, y, z = numpy.hsplit(local_xyz, 3)
    lat2 = numpy.pi / 2 - lat
    y2 = -z * numpy.sin(lat2) + y * numpy.cos(lat2)
    z2 = z * numpy.cos(lat2) + y * numpy.sin(lat2)
    return numpy.hstack([x, y2, z2])


def xyz_to_uvw(xyz, ha, dec):
    """Rotate XYZ to (u, v, w) for hour angle ha and declination dec (:59-85)."""
    x, y, z = numpy.hsplit(xyz, 3)
    u = x * numpy.cos(ha) - y * numpy.sin(ha)
    v0 = x * numpy.sin(ha) + y * numpy.cos(ha)
    w = z * numpy.sin(dec) - v0 * numpy.cos(dec)
    v = z * numpy.cos(dec) + v0 * numpy.sin(dec)
    return numpy.hstack([u, v, w])


def antennas_in_disk(nants, radius_m, rng, latitude=numpy.deg2rad(-45.0)):
    r = radius_m * numpy.sqrt(rng.uniform(size=nants))
    th = 2 * numpy.pi * rng.uniform(size=nants)
    local = numpy.stack([r * numpy.cos(th), r * numpy.sin(th), numpy.zeros(nants)], axis=1)
    return xyz_at_latitude(local, latitude)


def rows(xyz, hour_angles, frequencies, dec=numpy.deg2rad(-45.0)):
    """(uvw [nrows, 3] wavelengths, frequency [nrows], a1, a2, time index) in
    ARL's row order: time, baseline (a1 < a2), channel."""
    nants = xyz.shape[0]
    a1, a2 = numpy.triu_indices(nants, 1)
    nb, nch, nt = a1.size, len(frequencies), len(hour_angles)
    k = numpy.asarray(frequencies, dtype=numpy.float64) / C_M_S
    uvw = numpy.empty((nt, nb, nch, 3))
    for t, ha in enumerate(hour_angles):
        pos = xyz_to_uvw(xyz, ha, dec)
        d = pos[a2] - pos[a1]
        uvw[t] = d[:, None, :] * k[None, :, None]
    n = nt * nb * nch
    freq = numpy.broadcast_to(numpy.asarray(frequencies, numpy.float64)[None, None, :], (nt, nb, nch)).reshape(n)
    ia1 = numpy.broadcast_to(a1[None, :, None], (nt, nb, nch)).reshape(n)
    ia2 = numpy.broadcast_to(a2[None, :, None], (nt, nb, nch)).reshape(n)
    it = numpy.broadcast_to(numpy.arange(nt)[:, None, None], (nt, nb, nch)).reshape(n)
    return uvw.reshape(n, 3), numpy.ascontiguousarray(freq), ia1, ia2, it


def uv_cut(uvw, npixel, cellsize, support, margin=2):
    """Rows whose support x support kernel window stays inside an npixel grid:
    |u|, |v| < (npixel/2 - support/2 - margin) / (npixel * cellsize)."""
    lim = (npixel // 2 - support // 2 - margin) / (npixel * cellsize)
    return (numpy.abs(uvw[:, 0]) < lim) & (numpy.abs(uvw[:, 1]) < lim)


def point_sources(n, rng, radius=0.1, fmin=0.1, fmax=10.0):
    """(l, m, flux) of n sources: l, m uniform in +/-radius, flux log-uniform."""
    l = rng.uniform(-radius, radius, n)
    m = rng.uniform(-radius, radius, n)
    flux = numpy.exp(rng.uniform(numpy.log(fmin), numpy.log(fmax), n))
    return l, m, flux


def predict_point_sources(uvw, l, m, flux, npol=1, device=None, dtype=torch.complex128, chunk=1 << 22):
    """sum_k flux_k exp(-2 pi i (u l_k + v m_k + w (n_k - 1)))  (simulate_point,
    coordinate_support.py:192-212), FP64, on ``device`` (CPU or CUDA), returned
    as [nrows, npol] (the same value in every polarisation)."""
    device = device or torch.device('cpu')
    u = torch.as_tensor(uvw, dtype=torch.float64, device=device)
    s = torch.as_tensor(numpy.stack([l, m, numpy.sqrt(1 - l ** 2 - m ** 2) - 1.0]), dtype=torch.float64,
                        device=device)
    fl = torch.as_tensor(flux, dtype=torch.float64, device=device)
    out = torch.empty((u.shape[0], npol), dtype=dtype, device=device)
    for b in range(0, u.shape[0], chunk):
        ph = -2.0 * numpy.pi * (u[b:b + chunk] @ s)
        v = (torch.polar(fl[None, :].expand_as(ph), ph)).sum(dim=1)
        out[b:b + chunk] = v[:, None].to(dtype)
    return out


WORKLOADS = {
    # Plain 2-D imaging, PSWF kernel, no w-correction (w used as is, one plane).
    'C1': dict(nants=64, radius=1000.0, ntimes=60, freqs=[1e8], npol=1, npixel=512, cellsize=1e-3,
               kernel='pswf', support=8, oversampling=8, nsources=10, seed=1001),
    # W-projection, 64 w-kernel planes whose support grows 8 -> 32 with |w|.
    'C2': dict(nants=256, radius=5000.0, ntimes=120, freqs=list(numpy.linspace(100e6, 120e6, 4)), npol=1,
               npixel=1024, cellsize=5e-4, kernel='wproj', nwplanes=64, support=32, support_min=8,
               oversampling=8, nsources=50, seed=1002),
    # Batched w-stacking, 4 polarisations, 64 channels with seeded per-channel
    # flagging of U(0, 0.6) of the rows (flagged rows dropped), channels summed
    # into one image (multi-frequency synthesis).
    'C3': dict(nants=512, radius=10000.0, ntimes=12, freqs=list(numpy.linspace(100e6, 130e6, 64)), npol=4,
               npixel=4096, cellsize=5e-5, kernel='pswf', support=8, oversampling=16, nsources=20,
               source_radius=0.08, vis_slices=20, flag_max=0.6, mfs=True, seed=1003),
    # Differentiable predict + gain solve: the model is an image of Gaussian-
    # smoothed point sources; observed visibilities come from the gridded
    # predict of that model with per-antenna gains and Gaussian noise.
    'C4': dict(nants=128, radius=2000.0, ntimes=240, freqs=list(numpy.linspace(100e6, 120e6, 8)), npol=1,
               npixel=2048, cellsize=3e-4, kernel='pswf', support=8, oversampling=8, nsources=200,
               source_radius=0.25, smooth_px=2.0, gain_amp_sigma=0.1, noise=0.01, mfs=True, model='image',
               seed=1004),
    # Large single-GPU stress: ~1e8 rows, 8192^2 grid, 32 w-stack planes.
    'C5': dict(nants=512, radius=40000.0, ntimes=3, freqs=list(numpy.linspace(100e6, 150e6, 256)), npol=1,
               npixel=8192, cellsize=1.2e-5, kernel='pswf', support=8, oversampling=16, nsources=20,
               source_radius=0.04, vis_slices=32, mfs=True, seed=1005),
}


def flag_rows(freq, freqs, flag_max, rng):
    """Keep-mask of per-channel flagging: channel c drops each of its rows with
    probability f_c ~ U(0, flag_max) (ARL's Visibility has no flag column, so
    flagged rows are removed)."""
    frac = rng.uniform(0.0, flag_max, len(freqs))
    ch = numpy.searchsorted(numpy.asarray(freqs), freq)
    return rng.uniform(size=freq.shape[0]) >= frac[ch]


def smoothed_point_image(npixel, cellsize, nsources, radius, sigma_px, rng, fmin=0.1, fmax=10.0):
    """[1, 1, npixel, npixel] image of nsources point sources (random pixels
    within +/-radius rad of the centre, flux log-uniform in [fmin, fmax]) each
    smoothed by a unit-sum Gaussian of sigma_px pixels."""
    half = int(radius / cellsize)
    c = npixel // 2
    img = numpy.zeros((npixel, npixel))
    ys = rng.integers(c - half, c + half, nsources)
    xs = rng.integers(c - half, c + half, nsources)
    flux = numpy.exp(rng.uniform(numpy.log(fmin), numpy.log(fmax), nsources))
    numpy.add.at(img, (ys, xs), flux)
    r = int(numpy.ceil(4 * sigma_px))
    k = numpy.exp(-0.5 * (numpy.arange(-r, r + 1) / sigma_px) ** 2)
    k /= k.sum()
    img = numpy.apply_along_axis(lambda a: numpy.convolve(a, k, mode='same'), 0, img)
    img = numpy.apply_along_axis(lambda a: numpy.convolve(a, k, mode='same'), 1, img)
    return img[None, None]


def antenna_gains(nants, amp_sigma, rng):
    """Complex per-antenna gains: amplitude N(1, amp_sigma), phase U(-pi, pi)."""
    return rng.normal(1.0, amp_sigma, nants) * numpy.exp(1j * rng.uniform(-numpy.pi, numpy.pi, nants))


def observe(model_vis, gains, a1, a2, noise, seed):
    """V_obs = g[a2] conj(g[a1]) M + n, n complex Gaussian of std `noise` per
    component (torch, on model_vis's device; gains, a1, a2 tensors there)."""
    gen = torch.Generator(device=model_vis.device).manual_seed(seed)
    rdt = torch.float64 if model_vis.dtype == torch.complex128 else torch.float32
    nr = torch.randn(model_vis.shape, dtype=rdt, device=model_vis.device, generator=gen)
    ni = torch.randn(model_vis.shape, dtype=rdt, device=model_vis.device, generator=gen)
    gg = (gains[a2] * torch.conj(gains[a1])).to(model_vis.dtype)[:, None]
    return gg * model_vis + noise * torch.complex(nr, ni)


def make_workload(name, max_rows=None, device=None, rng_seed=None):
    """Rows, vis and image geometry of a named workload (after the uv-cut and
    any flagging).  ``max_rows`` keeps a seeded random subset of rows (for the
    CPU oracle).  Workloads with ``model='image'`` carry a model image and
    antenna gains instead of point-source visibilities (``vis`` is None)."""
    cfg = dict(WORKLOADS[name])
    rng = numpy.random.default_rng(cfg['seed'] if rng_seed is None else rng_seed)
    xyz = antennas_in_disk(cfg['nants'], cfg['radius'], rng)
    ha = numpy.linspace(-numpy.pi / 6, numpy.pi / 6, cfg['ntimes'])
    uvw, freq, a1, a2, tix = rows(xyz, ha, cfg['freqs'])
    keep = uv_cut(uvw, cfg['npixel'], cfg['cellsize'], cfg['support'])
    nrows_generated = uvw.shape[0]
    if cfg.get('flag_max'):
        keep &= flag_rows(freq, cfg['freqs'], cfg['flag_max'], numpy.random.default_rng(cfg['seed'] + 3))
    uvw, freq, a1, a2, tix = uvw[keep], freq[keep], a1[keep], a2[keep], tix[keep]
    del keep
    if max_rows is not None and uvw.shape[0] > max_rows:
        sel = numpy.sort(numpy.random.default_rng(cfg['seed'] + 7).choice(uvw.shape[0], max_rows, replace=False))
        uvw, freq, a1, a2, tix = uvw[sel], freq[sel], a1[sel], a2[sel], tix[sel]
    uvw = numpy.ascontiguousarray(uvw)
    out = dict(cfg, uvw=uvw, frequency=freq, antenna1=a1, antenna2=a2, time_index=tix,
               nrows_generated=nrows_generated)
    freqs = numpy.asarray(cfg['freqs'])
    out['channel_bandwidth'] = float(freqs[1] - freqs[0]) if len(freqs) > 1 else 1e6
    if cfg.get('mfs'):
        # One image channel whose FREQ pixel is wide enough that every row's
        # channel rounds to it: the channels are summed on the grid.
        out['image_frequency'] = [float(freqs.mean())]
        out['image_bandwidth'] = float(2.0 * (freqs.max() - freqs.min()) + out['channel_bandwidth'])
    else:
        out['image_frequency'] = list(cfg['freqs'])
        out['image_bandwidth'] = out['channel_bandwidth']
    # Natural weighting: unit weights (a read-only broadcast view; index or
    # copy it before writing).
    out['weight'] = numpy.broadcast_to(numpy.ones(1), (uvw.shape[0], cfg['npol']))
    if cfg.get('model') == 'image':
        out['vis'] = None
        out['model_image'] = smoothed_point_image(cfg['npixel'], cfg['cellsize'], cfg['nsources'],
                                                  cfg['source_radius'], cfg['smooth_px'], rng)
        out['gains'] = antenna_gains(cfg['nants'], cfg['gain_amp_sigma'], rng)
    else:
        l, m, flux = point_sources(cfg['nsources'], rng, radius=cfg.get('source_radius', 0.1))
        out['vis'] = predict_point_sources(uvw, l, m, flux, cfg['npol'], device=device)
        out['sources'] = (l, m, flux)
    if cfg['kernel'] == 'wproj':
        wmax = numpy.max(numpy.abs(uvw[:, 2]))
        nwp = cfg['nwplanes']
        out['wstep'] = float(wmax / (nwp // 2 - 1)) * 1.0001
        wplanes = (numpy.arange(nwp) - nwp // 2) * out['wstep']
        from_min, to_max = cfg['support_min'], cfg['support']
        w = numpy.abs(wplanes)
        s = from_min + (to_max - from_min) * w / w.max()
        out['plane_support'] = (2 * numpy.ceil(s / 2)).astype(numpy.int32).clip(from_min, to_max)
    return out


def workload_image(arl, w):
    """Template image of a workload (phase centre at dec -45 deg, the
    observation's pointing), with the workload's polarisation count."""
    frame = {1: 'stokesI', 2: 'linearnp', 4: 'linear'}[w['npol']]
    return arl.create_image(npixel=w['npixel'], cellsize=w['cellsize'],
                            frequency=numpy.asarray(w['image_frequency']),
                            channel_bandwidth=numpy.array([w['image_bandwidth']]),
                            polarisation_frame=arl.PolarisationFrame(frame),
                            phasecentre=arl.PhaseCentre(0.0, -45.0))
