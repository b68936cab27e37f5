"""FP64 CPU oracle for ARL's convolutional gridding / degridding imaging path.

TEST INFRASTRUCTURE ONLY.  This module is the checker: ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may import
it; the product package (``algorithm-reference-library_gb300``) never does.

What it is
    A complex128 NumPy restatement of ARL's hot path, written from the
    reference's behaviour (every function cites the reference file:line it
    follows, paths relative to the ARL project root).  The per-row loops of
    ``grid_loop`` / ``degrid_loop`` follow the reference's own loop bodies
    (``processing_components/griddata/gridding.py:127-130`` and ``:256-265``);
    ``grid_vec`` / ``degrid_vec`` are vectorised equivalents used for larger
    parity cases.

How it is pinned
    * Kernel known-answer values from
      ``tests/processing_components/test_griddata_kernels.py`` (PSWF peaks,
      w-kernel peak, clipped peak, symmetry) are reproduced by
      ``tests/test_oracle_kat.py``.
    * ``tests/golden/make_golden.py`` imports the reference's own Python
      modules (with a linear-axis stand-in for astropy's WCS, astropy being
      absent here) and records grid / degrid / FFT / kernel outputs on seeded
      inputs; ``tests/test_oracle_golden.py`` checks this module against them.

Coordinate conventions
    astropy's WCS is replaced by the FITS linear-axis transform with identity
    PC matrix: ``world2pix0(x) = ((x - crval) / cdelt + crpix) - 1`` and
    ``pix2world0(p) = ((p + 1) - crpix) * cdelt + crval`` (origin 0).  Every
    axis ARL uses on this path (UU, VV, DUU, DVV, WW, FREQ) is linear.
"""
import numpy as np

D2R = np.pi / 180.0
C_M_S = 299792458.0


# ---------------------------------------------------------------------------
# Linear WCS axes
# ---------------------------------------------------------------------------
def world2pix0(x, crval, crpix, cdelt):
    """Linear world->pixel (origin 0); stands in for ``wcs_world2pix(..., 0)``."""
    return ((x - crval) / cdelt + crpix) - 1.0


def pix2world0(p, crval, crpix, cdelt):
    """Linear pixel->world (origin 0); stands in for ``wcs_pix2world(..., 0)``."""
    return ((p + 1.0) - crpix) * cdelt + crval


def image_geometry(npixel, cellsize, nchan=1, npol=1, frequency0=1e8, channel_bandwidth=1e6):
    """Image template WCS numbers as ``create_image`` sets them
    (``processing_library/image/operations.py:31-69``)."""
    return dict(nchan=nchan, npol=npol, ny=npixel, nx=npixel,
                cdelt_ra=-cellsize * 180.0 / np.pi, cdelt_dec=cellsize * 180.0 / np.pi,
                crpix_ra=float(npixel // 2 + 1), crpix_dec=float(npixel // 2 + 1),
                crval_f=float(frequency0), cdelt_f=float(channel_bandwidth), crpix_f=1.0)


def grid_axes(img, nw=1, wstep=1e15):
    """GridData axes UU, VV, WW, FREQ (``processing_components/griddata/operations.py:91-145``)."""
    return dict(
        u=(0.0, float(img['nx'] // 2 + 1), 1.0 / (img['nx'] * D2R * img['cdelt_ra'])),
        v=(0.0, float(img['ny'] // 2 + 1), 1.0 / (img['ny'] * D2R * img['cdelt_dec'])),
        w=(0.0, float(nw // 2 + 1), float(wstep)),
        f=(img['crval_f'], img['crpix_f'], img['cdelt_f']),
        shape=(img['nchan'], img['npol'], nw, img['ny'], img['nx']))


def cf_axes(img, oversampling, support, nz=1, zstep=1e15):
    """ConvolutionFunction axes UU, VV, DUU, DVV, WW
    (``processing_components/griddata/convolution_functions.py:62-147``)."""
    cu = 1.0 / (img['nx'] * D2R * img['cdelt_ra'])
    cv = 1.0 / (img['ny'] * D2R * img['cdelt_dec'])
    return dict(
        u=(0.0, float(support // 2) + 1.0, cu),
        v=(0.0, float(support // 2) + 1.0, cv),
        du=(0.0, float(oversampling // 2) + 1.0, cu / oversampling),
        dv=(0.0, float(oversampling // 2) + 1.0, cv / oversampling),
        z=(0.0, float(nz // 2 + 1), float(zstep)),
        shape=(img['nchan'], img['npol'], nz, oversampling, oversampling, support, support))


# ---------------------------------------------------------------------------
# a1: convolution_mapping   (processing_components/griddata/gridding.py:24-96)
# ---------------------------------------------------------------------------
def convolution_mapping(uvw, frequency, gax, cax):
    """Row -> (pu, pu_off, pv, pv_off, pwg, pwc, pfreq), int64 arrays.

    Nearest grid point by round-half-even (``numpy.round``, :42), sub-pixel
    index by floor of the DUU/DVV world2pix of the remainder (:50-54),
    w-plane and channel by round (:58-85).  The reference's range asserts are
    returned as a boolean ``ok`` array instead (the caller raises)."""
    u, v, w = uvw[:, 0], uvw[:, 1], uvw[:, 2]
    pu = np.round(world2pix0(u, *gax['u'])).astype(np.int64)
    pv = np.round(world2pix0(v, *gax['v'])).astype(np.int64)
    wu = pix2world0(pu, *gax['u'])
    wv = pix2world0(pv, *gax['v'])
    pu_off = np.floor(world2pix0(u - wu, *cax['du'])).astype(np.int64)
    pv_off = np.floor(world2pix0(v - wv, *cax['dv'])).astype(np.int64)
    pwg = np.round(world2pix0(w, *gax['w'])).astype(np.int64)
    pwc = np.round(world2pix0(w, *cax['z'])).astype(np.int64)
    pfreq = np.round(world2pix0(frequency, *gax['f'])).astype(np.int64)
    return pu, pu_off, pv, pv_off, pwg, pwc, pfreq


def rows_in_grid(maps, gshape, cshape):
    """True for rows whose whole S x S window and plane/channel indices lie
    inside the grid and cf: the rows ARL's asserts and slicing accept
    (``gridding.py:43-46,64-65,75-76,83-84,128``)."""
    pu, pu_off, pv, pv_off, pwg, pwc, pfreq = maps
    nchan, npol, nw, ny, nx = gshape
    S = cshape[-1]
    h = S // 2
    O = cshape[3]
    return ((pu - h >= 0) & (pu + h <= nx) & (pv - h >= 0) & (pv + h <= ny)
            & (pwg >= 0) & (pwg < nw) & (pwc >= 0) & (pwc < cshape[2])
            & (pfreq >= 0) & (pfreq < min(nchan, cshape[0]))
            & (pu_off >= 0) & (pu_off < O) & (pv_off >= 0) & (pv_off < O))


# ---------------------------------------------------------------------------
# a2 / a3: grid and degrid
# ---------------------------------------------------------------------------
def grid_loop(vis, wt, maps, cf, gshape, out=None, ccf=None):
    """Per-row gridding loop (``gridding.py:99-133``); returns (grid, sumwt).

    grid[c, :, zg, pv-S/2:pv+S/2, pu-S/2:pu+S/2] += conj(cf[c, :, zc, pv_off, pu_off]) * (vis*wt)[:, None, None]
    sumwt[c, :] += wt
    ``out`` = (grid, sumwt) accumulates into existing arrays; ``ccf`` passes a
    precomputed conj(cf) (the reference conjugates cf once per call, :123)."""
    pu, pu_off, pv, pv_off, pwg, pwc, pfreq = maps
    if out is None:
        grid = np.zeros(gshape, dtype=np.complex128)
        sumwt = np.zeros(gshape[:2])
    else:
        grid, sumwt = out
    if ccf is None:
        ccf = np.conjugate(cf)
    dv = cf.shape[-2] // 2
    du = cf.shape[-1] // 2
    vw = vis * wt
    for r in range(vis.shape[0]):
        c = pfreq[r]
        grid[c, :, pwg[r], pv[r] - dv:pv[r] + dv, pu[r] - du:pu[r] + du] += \
            ccf[c, :, pwc[r], pv_off[r], pu_off[r], :, :] * vw[r][:, None, None]
        sumwt[c, :] += wt[r]
    return grid, sumwt


def grid_vec(vis, wt, maps, cf, gshape, chunk=1 << 15):
    """Vectorised gridding, same result as ``grid_loop`` up to summation order."""
    pu, pu_off, pv, pv_off, pwg, pwc, pfreq = maps
    nchan, npol, nw, ny, nx = gshape
    S = cf.shape[-1]
    grid = np.zeros(gshape, dtype=np.complex128)
    sumwt = np.zeros((nchan, npol))
    np.add.at(sumwt, pfreq, wt)
    flat = grid.reshape(-1)
    jj = np.arange(S) - S // 2
    vw = vis * wt
    for s in range(0, vis.shape[0], chunk):
        e = min(s + chunk, vis.shape[0])
        for p in range(npol):
            taps = np.conjugate(cf[pfreq[s:e], p, pwc[s:e], pv_off[s:e], pu_off[s:e]])  # [n,S,S]
            base = ((pfreq[s:e] * npol + p) * nw + pwg[s:e]) * ny
            idx = ((base[:, None] + pv[s:e, None] + jj[None, :]) * nx)[:, :, None] + \
                (pu[s:e, None] + jj[None, :])[:, None, :]
            np.add.at(flat, idx.reshape(-1), (taps * vw[s:e, p][:, None, None]).reshape(-1))
    return grid, sumwt


def degrid_loop(grid, maps, cf):
    """Per-row degridding loop (``gridding.py:233-267``): returns vis [nvis, npol]."""
    pu, pu_off, pv, pv_off, pwg, pwc, pfreq = maps
    dv = cf.shape[-2] // 2
    du = cf.shape[-1] // 2
    out = np.zeros((pu.shape[0], grid.shape[1]), dtype=np.complex128)
    for r in range(pu.shape[0]):
        c = pfreq[r]
        out[r, :] += np.einsum('ijk,ijk->i',
                               grid[c, :, pwg[r], pv[r] - dv:pv[r] + dv, pu[r] - du:pu[r] + du],
                               cf[c, :, pwc[r], pv_off[r], pu_off[r], :, :])
    return out


def degrid_vec(grid, maps, cf, chunk=1 << 15):
    """Vectorised degridding, same result as ``degrid_loop`` up to summation order."""
    pu, pu_off, pv, pv_off, pwg, pwc, pfreq = maps
    nchan, npol, nw, ny, nx = grid.shape
    S = cf.shape[-1]
    jj = np.arange(S) - S // 2
    flat = grid.reshape(-1)
    out = np.zeros((pu.shape[0], npol), dtype=np.complex128)
    for s in range(0, pu.shape[0], chunk):
        e = min(s + chunk, pu.shape[0])
        for p in range(npol):
            taps = cf[pfreq[s:e], p, pwc[s:e], pv_off[s:e], pu_off[s:e]]
            base = ((pfreq[s:e] * npol + p) * nw + pwg[s:e]) * ny
            idx = ((base[:, None] + pv[s:e, None] + jj[None, :]) * nx)[:, :, None] + \
                (pu[s:e, None] + jj[None, :])[:, None, :]
            out[s:e, p] = np.einsum('rij,rij->r', flat[idx], taps)
    return out


def window_index(maps, gshape, S):
    """Flat indices [nvis, npol, S, S] of each row's S x S window in a grid of
    shape gshape: the slice ``grid[c, p, zg, pv-S/2:pv+S/2, pu-S/2:pu+S/2]`` of
    ``gridding.py:128`` and ``:261``."""
    pu, pu_off, pv, pv_off, pwg, pwc, pfreq = maps
    nchan, npol, nw, ny, nx = gshape
    jj = np.arange(S) - S // 2
    base = ((pfreq[:, None] * npol + np.arange(npol)[None, :]) * nw + pwg[:, None]) * ny
    rows = (base[:, :, None] + pv[:, None, None] + jj[None, None, :]) * nx
    return rows[:, :, :, None] + (pu[:, None, None, None] + jj[None, None, None, :])


def grid_sparse(vis, wt, maps, cf, gshape):
    """``grid_vec`` restricted to the cells the rows touch, for grids too large
    to hold densely: (sorted flat cell indices, complex128 cell values, sumwt)."""
    pu, pu_off, pv, pv_off, pwg, pwc, pfreq = maps
    nchan, npol = gshape[:2]
    S = cf.shape[-1]
    idx = window_index(maps, gshape, S).reshape(-1)
    taps = np.conjugate(cf[pfreq, :, pwc, pv_off, pu_off])          # [n, npol, S, S]
    val = (taps * (vis * wt)[:, :, None, None]).reshape(-1)
    cells, inv = np.unique(idx, return_inverse=True)
    out = np.bincount(inv, weights=val.real, minlength=cells.size) + \
        1j * np.bincount(inv, weights=val.imag, minlength=cells.size)
    sumwt = np.zeros((nchan, npol))
    np.add.at(sumwt, pfreq, wt)
    return cells, out, sumwt


def degrid_windows(windows, maps, cf):
    """``degrid_vec`` from each row's window of grid values, windows[nvis, npol,
    S, S] gathered at ``window_index``: vis[r, p] = sum(window * cf taps)
    (``gridding.py:256-265``)."""
    pu, pu_off, pv, pv_off, pwg, pwc, pfreq = maps
    taps = cf[pfreq, :, pwc, pv_off, pu_off]
    return np.einsum('rpij,rpij->rp', windows, taps)


def grid_weight(wt, maps, gshape):
    """``grid_weight_to_griddata`` (``gridding.py:161-183``): nearest-cell weight sum."""
    pu, pu_off, pv, pv_off, pwg, pwc, pfreq = maps
    nchan, npol, nw, ny, nx = gshape
    grid = np.zeros(gshape, dtype=np.complex128)
    sumwt = np.zeros((nchan, npol))
    for r in range(wt.shape[0]):
        grid[pfreq[r], :, pwg[r], pv[r], pu[r]] += wt[r]
        sumwt[pfreq[r], :] += wt[r]
    return grid, sumwt


def reweight(wt, maps, wgrid):
    """``griddata_reweight`` (``gridding.py:213-230``): each row's imaging weight
    divided by the real part of its nearest cell of the weight grid, when every
    polarisation's cell is non-zero (the reference tests ``real(cell).all() > 0``,
    i.e. all non-zero).  Returns a new array."""
    pu, pu_off, pv, pv_off, pwg, pwc, pfreq = maps
    out = np.array(wt, dtype=np.float64, copy=True)
    for r in range(out.shape[0]):
        cell = np.real(wgrid[pfreq[r], :, pwg[r], pv[r], pu[r]])
        if cell.all() > 0.0:
            out[r] /= cell
    return out


def weight_uniform(wt, maps, gshape):
    """``weight_visibility`` (``imaging/weighting.py:19-40``): grid the weights,
    then reweight the rows."""
    wgrid, _ = grid_weight(wt, maps, gshape)
    return reweight(wt, maps, wgrid)


# ---------------------------------------------------------------------------
# a15: BlockVisibility <-> Visibility (visibility/coalesce.py:85-143,331-443)
# ---------------------------------------------------------------------------
def convert_blocks(vis, uvw, wts, imaging_wts, times, integration_time, frequency, channel_bandwidth):
    """``convert_blocks`` (``coalesce.py:331-443``): rows ordered (time, a2, a1,
    channel) over the baselines a2 > a1 of the [ntimes, nant, nant, nchan, npol]
    block; uvw converted from metres to wavelengths as uvw * (f / c).  Returns
    (vis, uvw, wts, imaging_wts, time, frequency, channel_bandwidth, a1, a2,
    integration_time, cindex)."""
    ntimes, nant, _, nchan, npol = vis.shape
    a2, a1 = np.tril_indices(nant, -1)
    order = np.lexsort((a1, a2))          # a2 ascending, then a1
    a2, a1 = a2[order], a1[order]
    nbl = a1.size
    t = np.repeat(np.arange(ntimes), nbl * nchan)
    b = np.tile(np.repeat(np.arange(nbl), nchan), ntimes)
    c = np.tile(np.arange(nchan), ntimes * nbl)
    ca1, ca2 = a1[b], a2[b]
    cfreq = np.asarray(frequency)[c]
    cuvw = uvw[t, ca2, ca1, :] * (cfreq / C_M_S)[:, None]
    cvis = vis[t, ca2, ca1, c, :]
    cwts = wts[t, ca2, ca1, c, :]
    cimw = imaging_wts[t, ca2, ca1, c, :]
    cindex = np.zeros(ntimes * nant * nant * nchan, dtype=np.int64)
    cindex[((t * nant + ca2) * nant + ca1) * nchan + c] = np.arange(t.size)
    return (cvis, cuvw, cwts, cimw, np.asarray(times)[t], cfreq, np.asarray(channel_bandwidth)[c], ca1, ca2,
            np.asarray(integration_time)[t], cindex)


def decoalesce(block, rows, cindex):
    """The overwrite loop of ``decoalesce_visibility`` (``coalesce.py:128-137``)
    for one column: for i over the block's cells, flat[i:i + npol] =
    rows[cindex[i]].  The slices overlap when npol > 1, so the reference's
    result is reproduced as written: position k holds element k - i of row
    cindex[i] for the last i that wrote it, and positions past N + npol - 2
    keep the block's values."""
    out = np.array(block, copy=True)
    flat = out.reshape(-1)
    npol = block.shape[-1]
    n = flat.size // npol
    for i in range(n):
        flat[i:i + npol] = rows[cindex[i]]
    return out


# ---------------------------------------------------------------------------
# (f4) deconvolution: Hogbom CLEAN (processing_library/arrays/cleaners.py:12-69,
#      processing_components/image/deconvolution.py:43-300)
# ---------------------------------------------------------------------------
def overlap_indices(res, psf, peakx, peaky):
    """``overlapIndices`` (``cleaners.py:134-154``)."""
    nx, ny = res.shape[0], res.shape[1]
    wx, wy = psf.shape[0] // 2, psf.shape[1] // 2
    res_lo = (max(0, peakx - wx), max(0, peaky - wy))
    res_hi = (min(nx, peakx + wx), min(peaky + wy, ny))
    psf_lo = (max(0, wx + (res_lo[0] - peakx)), max(0, wy + (res_lo[1] - peaky)))
    psf_hi = (min(psf.shape[0], wx + (res_hi[0] - peakx)), min(wy + (res_hi[1] - peaky), psf.shape[1]))
    return (res_lo[0], res_hi[0], res_lo[1], res_hi[1]), (psf_lo[0], psf_hi[0], psf_lo[1], psf_hi[1])


def hogbom(dirty, psf, window, gain, thresh, niter, fracthresh):
    """``hogbom`` (``cleaners.py:12-69``): returns (components, residual)."""
    absolutethresh = max(thresh, fracthresh * np.fabs(dirty).max())
    comps = np.zeros(dirty.shape)
    res = np.array(dirty)
    pmax = psf.max()
    for i in range(niter):
        a = np.fabs(res * window) if window is not None else np.fabs(res)
        mx, my = np.unravel_index(a.argmax(), dirty.shape)
        mval = res[mx, my] * gain / pmax
        comps[mx, my] += mval
        a1o, a2o = overlap_indices(dirty, psf, mx, my)
        res[a1o[0]:a1o[1], a1o[2]:a1o[3]] -= psf[a2o[0]:a2o[1], a2o[2]:a2o[3]] * mval
        if np.abs(res[mx, my]) < 0.9 * absolutethresh:
            break
    return comps, res


def deconvolve_hogbom(dirty, psf, niter=100, gain=0.7, threshold=0.0, fractional_threshold=0.1,
                      window_shape=None, window_edge=16, psf_support=None):
    """The 'hogbom' branch of ``deconvolve_cube`` (``deconvolution.py:43-300``)
    on arrays [nchan, npol, ny, nx]: window shapes, PSF crop, per-plane CLEAN."""
    ny, nx = dirty.shape[2], dirty.shape[3]
    if window_shape == 'quarter':
        qx, qy = nx // 4, ny // 4
        window = np.zeros_like(dirty)
        window[..., (qy + 1):3 * qy, (qx + 1):3 * qx] = 1.0
    elif window_shape == 'no_edge':
        window = np.zeros_like(dirty)
        window[..., (window_edge + 1):(ny - window_edge), (window_edge + 1):(nx - window_edge)] = 1.0
    else:
        window = None
    if psf_support is None:
        psf_support = max(dirty.shape[2] // 2, dirty.shape[3] // 2)
    if psf_support <= psf.shape[2] // 2 and psf_support <= psf.shape[3] // 2:
        c = [psf.shape[2] // 2, psf.shape[3] // 2]
        psf = psf[..., (c[0] - psf_support):(c[0] + psf_support), (c[1] - psf_support):(c[1] + psf_support)]
    comp = np.zeros(dirty.shape)
    resid = np.zeros(dirty.shape)
    for ch in range(dirty.shape[0]):
        for p in range(dirty.shape[1]):
            if psf[ch, p].max():
                comp[ch, p], resid[ch, p] = hogbom(dirty[ch, p], psf[ch, p],
                                                   None if window is None else window[ch, p], gain, threshold,
                                                   niter, fractional_threshold)
    return comp, resid


def _sph_scalar(vnu):
    """``spheroidal_function`` (``cleaners.py:398-440``), one scalar."""
    if 0.0 <= vnu < 0.75:
        part, nuend = 0, 0.75
    elif 0.75 <= vnu <= 1.0:
        part, nuend = 1, 1.0
    else:
        return 0.0
    top, bot = _SPH_P[part, 0], _SPH_Q[part, 0]
    d = vnu ** 2 - nuend ** 2
    for k in range(1, 5):
        top += _SPH_P[part, k] * d ** k
    for k in range(1, 3):
        bot += _SPH_Q[part, k] * d ** k
    v = top / bot if bot != 0.0 else 0.0
    return v if v >= 0.0 else 0.0


def scalestack(shape, scales):
    """``create_scalestack`` (``cleaners.py:283-316``, norm=True)."""
    basis = np.zeros(shape)
    nx, ny = shape[1], shape[2]
    xc, yc = int(np.ceil(float(nx) / 2.0)), int(np.ceil(float(ny) / 2.0))
    for i in np.arange(len(scales)):
        h = int(np.ceil(scales[i] / 2.0))
        if scales[i] > 0.0:
            rs2 = 1.0 / (float(scales[i]) / 2.0) ** 2
            for y in range(yc - h - 1, yc + h + 1):
                for x in range(xc - h - 1, xc + h + 1):
                    r = np.sqrt(rs2 * (float(x - xc) ** 2 + float(y - yc) ** 2))
                    basis[i, x, y] = _sph_scalar(r) * (1.0 - r ** 2)
            basis[basis < 0.0] = 0.0
            basis[i] /= np.sum(basis[i])
        else:
            basis[i, xc, yc] = 1.0
    return basis


def _ft(a):
    return np.fft.fftshift(np.fft.fft2(np.fft.fftshift(a)))


def _ift_real(a):
    return np.real(np.fft.ifftshift(np.fft.ifft2(np.fft.ifftshift(a))))


def msclean(dirty, psf, window, gain, thresh, niter, scales, fracthresh):
    """``msclean`` (``cleaners.py:165-280``): returns (components, residual)."""
    comps = np.zeros(dirty.shape)
    pmax = psf.max()
    lpsf, ldirty = psf / pmax, dirty / pmax
    ns = len(scales)
    ss = scalestack([ns, ldirty.shape[0], ldirty.shape[1]], scales)
    pss = scalestack([ns, lpsf.shape[0], lpsf.shape[1]], scales)
    xd = _ft(ldirty)
    stack = np.stack([_ift_real(xd * np.conjugate(_ft(ss[i]))) for i in range(ns)])
    xp = _ft(lpsf)
    xs = [_ft(pss[i]) for i in range(ns)]
    pp = np.zeros([ns, ns, lpsf.shape[0], lpsf.shape[1]])
    for a in range(ns):
        for b in range(ns):
            pp[a, b] = _ift_real(xp * xs[b] * np.conjugate(xs[a]))
    cm = np.array([[np.max(pp[a, b]) for b in range(ns)] for a in range(ns)])
    if window is None:
        ws = None
    else:
        xw = _ft(window)
        ws = np.zeros_like(ss)
        ws[np.stack([_ift_real(xw * np.conjugate(_ft(ss[i]))) for i in range(ns)]) > 0.9] = 1.0
    athresh = max(thresh, fracthresh * np.fabs(stack[0]).max())
    for _ in range(niter):
        best, px, py, psc = 0.0, 0, 0, 0
        for i in range(ns):
            r = stack[i] * ws[i] / cm[i, i] if ws is not None else stack[i] / cm[i, i]
            mx, my = np.unravel_index(np.abs(r).argmax(), r.shape)
            if np.abs(r[mx, my]) > best:
                best, px, py, psc = np.abs(r[mx, my]), mx, my, i
        mval = stack[psc, px, py] / cm[psc, psc]
        if np.fabs(stack[psc, px, py]) < 0.9 * athresh:
            break
        lhs, rhs = overlap_indices(dirty, psf, px, py)
        if np.abs(mval) > 0:
            for i in range(ns):
                stack[i, lhs[0]:lhs[1], lhs[2]:lhs[3]] -= pp[i, psc, rhs[0]:rhs[1], rhs[2]:rhs[3]] * gain * mval
            comps[lhs[0]:lhs[1], lhs[2]:lhs[3]] += pss[psc, rhs[0]:rhs[1], rhs[2]:rhs[3]] * gain * mval
        else:
            break
    return comps, pmax * stack[0]


# ---------------------------------------------------------------------------
# a6: centred FFTs (processing_library/fourier_transforms/fft_support.py:21-89)
# ---------------------------------------------------------------------------
def fft(a):
    """fftshift(fft2(ifftshift(a))) over the last two axes, unnormalised."""
    ax = (-2, -1)
    return np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(a, axes=ax), axes=ax), axes=ax)


def ifft(a):
    """fftshift(ifft2(ifftshift(a))) over the last two axes, 1/N^2 normalised."""
    ax = (-2, -1)
    return np.fft.fftshift(np.fft.ifft2(np.fft.ifftshift(a, axes=ax), axes=ax), axes=ax)


def fft_griddata_to_image(grid, gcf):
    """``gridding.py:270-289``: sum over w, ifft, times gcf * nx * ny.
    Returns the complex image (real part = ARL's image, imag = its ``imaginary``)."""
    projected = np.sum(grid, axis=2)
    ny, nx = projected.shape[-2:]
    return ifft(projected) * gcf * float(nx) * float(ny)


def fft_image_to_griddata(im, gcf, nw=1):
    """``gridding.py:292-302``: grid[:, :, z] = fft(im * gcf) for every z."""
    g = fft(im * gcf)
    return np.repeat(g[:, :, None], nw, axis=2)


def normalize_sumwt(im, sumwt):
    """``processing_components/imaging/base.py:84-101``."""
    out = np.array(im, copy=True)
    for c in range(out.shape[0]):
        for p in range(out.shape[1]):
            if sumwt[c, p] > 0.0:
                out[c, p] = out[c, p] / sumwt[c, p]
            else:
                out[c, p] = 0.0
    return out


# ---------------------------------------------------------------------------
# a7 / a8: PSWF (processing_library/fourier_transforms/convolutional_gridding.py:72-117,
#           processing_components/griddata/kernels.py:52-97)
# ---------------------------------------------------------------------------
# Schwab's rational approximation to the m=6, alpha=1 spheroidal function
# (F. Schwab, "Optimal gridding of visibility data in radio interferometry",
# Indirect Imaging, 1984): two intervals [0, 0.75) and [0.75, 1].
_SPH_P = np.array([[8.203343e-2, -3.644705e-1, 6.278660e-1, -5.335581e-1, 2.312756e-1],
                   [4.028559e-3, -3.697768e-2, 1.021332e-1, -1.201436e-1, 6.412774e-2]])
_SPH_Q = np.array([[1.0000000e0, 8.212018e-1, 2.078043e-1],
                   [1.0000000e0, 9.599102e-1, 2.918724e-1]])


def grdsf(nu):
    """Returns (grdsf(nu), (1 - nu^2) grdsf(nu)); zero beyond |nu| > 1."""
    nu = np.abs(np.asarray(nu, dtype=np.float64))
    part = np.where(nu >= 0.75, 1, 0)
    nuend = np.where(nu >= 0.75, 1.0, 0.75)
    d = nu ** 2 - nuend ** 2
    top = _SPH_P[part, 0].copy()
    for k in range(1, _SPH_P.shape[1]):
        top += _SPH_P[part, k] * np.power(d, k)
    bot = _SPH_Q[part, 0].copy()
    for k in range(1, _SPH_Q.shape[1]):
        bot += _SPH_Q[part, k] * np.power(d, k)
    g = np.zeros_like(nu)
    ok = bot > 0.0
    g[ok] = top[ok] / bot[ok]
    g[nu > 1.0] = 0.0
    return g, (1 - nu ** 2) * g


def coordinates(n):
    """``convolutional_gridding.py:37-41``."""
    return (np.arange(n) - n // 2) / n


def pswf_kernel1d(oversampling, support):
    """kernel[s, g] of ``kernels.py:68-74`` (normalised by the sum of the centre row)."""
    k = np.zeros((oversampling, support))
    for g in range(support):
        for s in range(oversampling):
            nu = ((g - support // 2) - (s - oversampling // 2) / oversampling)
            k[s, g] = grdsf(np.array([nu / (support // 2)]))[1][0]
    k /= np.sum(np.real(k[oversampling // 2, :]))
    return k


def pswf_gcf(nx):
    """Grid-correction image of ``kernels.py:87-91`` ([nx, nx], real)."""
    g1 = grdsf(np.abs(2.0 * coordinates(nx)))[0]
    gcf = np.outer(g1, g1)
    pos = gcf > 0.0
    gcf[pos] = gcf.max() / gcf[pos]
    return gcf


def create_pswf_cf(nchan, npol, ny, nx, oversampling=8, support=6):
    """(gcf [nchan,npol,ny,nx], cf [nchan,npol,1,O,O,S,S]) of ``kernels.py:52-97``."""
    k = pswf_kernel1d(oversampling, support)
    cf = np.zeros((nchan, npol, 1, oversampling, oversampling, support, support), dtype=np.complex128)
    for y in range(oversampling):
        for x in range(oversampling):
            cf[:, :, 0, y, x] = np.outer(k[y], k[x])[None, None]
    cf /= np.sum(np.real(cf[0, 0, 0, 0, 0]))
    gcf = np.broadcast_to(pswf_gcf(nx), (nchan, npol, ny, nx)).copy()
    return gcf, cf


def create_box_cf(nchan, npol, ny, nx):
    """``kernels.py:19-49``: unit tap at (2, 2) of a 4x4 kernel, O=1; gcf = 1/sinc^2."""
    cf = np.zeros((nchan, npol, 1, 1, 1, 4, 4), dtype=np.complex128)
    cf[..., 2, 2] = 1.0
    g1 = np.sinc(np.abs(coordinates(nx)))
    gcf = 1.0 / np.outer(g1, g1)
    return np.broadcast_to(gcf, (nchan, npol, ny, nx)).copy(), cf


# ---------------------------------------------------------------------------
# a9: w-kernels  (kernels.py:100-200, convolutional_gridding.py:120-188,
#                 processing_library/image/operations.py:335-408)
# ---------------------------------------------------------------------------
def w_beam(npixel, field_of_view, w, cx=None, cy=None):
    """Fresnel w-screen exp(-2 pi i w (1 - sqrt(1 - r^2))), zero for r >= 1, one at r = 0.
    The reference builds one quadrant and mirrors it; for even npixel with the
    centre at npixel//2 that equals direct evaluation on the full grid."""
    if cx is None:
        cx = npixel // 2
    if cy is None:
        cy = npixel // 2
    mg = np.mgrid[0:npixel, 0:npixel]
    ly = (mg[0] - cy) / npixel
    mx = (mg[1] - cx) / npixel
    r2 = field_of_view ** 2 * (ly ** 2 + mx ** 2)
    with np.errstate(invalid='ignore'):
        ph = -2 * np.pi * w * (1 - np.sqrt(1.0 - r2))
    ph[r2 >= 1.0] = 0.0
    cp = np.exp(1j * ph)
    cp[r2 >= 1.0] = 0.0
    cp[r2 == 0] = 1.0
    return cp


def w_term_image(npixel, cellsize_rad, w):
    """``create_w_term_like`` (operations.py:364-408) for a square image with
    crpix = npixel//2 + 1 and |cdelt| = cellsize."""
    return w_beam(npixel, npixel * cellsize_rad, w, cx=float(npixel // 2), cy=float(npixel // 2))


def create_awterm_cf(img, nw=1, wstep=1e15, oversampling=8, support=6, maxsupport=512, planes=None):
    """(gcf, cf [nchan,npol,nw,O,O,S,S]) of ``create_awterm_convolutionfunction``
    with ``use_aaf=True`` and no primary beam (``kernels.py:100-200``).
    ``planes`` restricts the work to the listed w-planes (others stay zero); it
    must include the centre plane nw//2, which sets the normalisation."""
    nchan, npol, ony, onx = img['nchan'], img['npol'], img['ny'], img['nx']
    w_list = pix2world0(np.arange(nw, dtype=np.float64), 0.0, float(nw // 2 + 1), float(wstep)) \
        if abs(wstep) > 0.0 else np.array([0.0])
    nx = max(maxsupport, 2 * oversampling * support)
    ny = nx
    qnx = nx // oversampling
    qny = ny // oversampling
    ccell = onx * np.abs(D2R * img['cdelt_ra']) / qnx
    sub_cdelt = -ccell / D2R
    sub_cell = abs(sub_cdelt) * np.pi / 180.0
    norm = 1.0 / pswf_gcf(qnx)
    cf = np.zeros((nchan, npol, nw, oversampling, oversampling, support, support), dtype=np.complex128)
    ycen, xcen = ny // 2, nx // 2
    for z, w in enumerate(w_list):
        if planes is not None and z not in planes:
            continue
        plane = w_beam(qnx, qnx * sub_cell, w, cx=float(qnx // 2), cy=float(qny // 2)) * norm
        padded = np.zeros((ny, nx), dtype=np.complex128)
        ys = ny // 2 - qny // 2
        xs = nx // 2 - qnx // 2
        padded[ys:ys + qny, xs:xs + qnx] = plane
        padded = ifft(padded)
        for y in range(oversampling):
            ybeg = y + ycen + (support * oversampling) // 2 - oversampling // 2
            yend = y + ycen - (support * oversampling) // 2 - oversampling // 2
            for x in range(oversampling):
                xbeg = x + xcen + (support * oversampling) // 2 - oversampling // 2
                xend = x + xcen - (support * oversampling) // 2 - oversampling // 2
                cf[:, :, z, y, x] = padded[ybeg:yend:-oversampling, xbeg:xend:-oversampling][None, None]
    cf /= np.sum(np.real(cf[0, 0, nw // 2, oversampling // 2, oversampling // 2]))
    cf = np.conjugate(cf)
    gcf, _ = create_pswf_cf(nchan, npol, ony, onx, oversampling=1, support=6)
    return gcf, cf


def bounding_box(cf, fractional_level=1e-4):
    """``calculate_bounding_box_convolutionfunction`` (convolution_functions.py:187-207)."""
    out = []
    threshold = fractional_level * np.max(np.abs(cf))
    for z in range(cf.shape[2]):
        mask = np.max(np.abs(cf[:, :, z]), axis=(0, 1, 2, 3))
        coords = np.argwhere(mask > threshold)
        x0, y0 = coords.min(axis=0)
        x1, y1 = coords.max(axis=0)
        out.append((z, (y0, y1), (x0, x1)))
    return out


def apply_bounding_box(cf, crpix_u, crpix_v, fractional_level=1e-4):
    """``apply_bounding_box_convolutionfunction`` (convolution_functions.py:159-184):
    returns (cropped cf, new crpix_u, new crpix_v)."""
    nx = cf.shape[-1]
    ny = cf.shape[-2]
    mask = np.max(np.abs(cf), axis=(0, 1, 2, 3, 4))
    coords = np.argwhere(mask > fractional_level * np.max(np.abs(cf)))
    crpx = int(np.round(crpix_u))
    crpy = int(np.round(crpix_v))
    x0, y0 = coords.min(axis=0)
    dx = crpx - x0
    dy = crpy - y0
    x0 -= 1
    y0 -= 1
    x1 = crpx + dx - 1
    y1 = crpy + dy - 1
    new = cf[..., y0:y1, x0:x1].copy()
    nny, nnx = new.shape[-2], new.shape[-1]
    return new, crpix_u + nnx / 2 - nx / 2, crpix_v + nny / 2 - ny / 2


def crop_cf_planes(cf, supports):
    """Per-plane support: taps outside the central supports[z] x supports[z]
    window of plane z are zeroed (the oracle side of a plane-dependent support)."""
    out = cf.copy()
    S = cf.shape[-1]
    for z, sz in enumerate(supports):
        lo = S // 2 - sz // 2
        hi = lo + sz
        m = np.zeros((S, S), dtype=bool)
        m[lo:hi, lo:hi] = True
        out[:, :, z, :, :, ~m] = 0.0
    return out


# ---------------------------------------------------------------------------
# a11 / a12: invert_2d and predict_2d on arrays (imaging/base.py:104-189)
# ---------------------------------------------------------------------------
def invert_2d(uvw, frequency, vis, wt, img, gcf, cf, cax, nw=1, wstep=1e15, dopsf=False,
              normalize=True, vectorised=True):
    """Returns (complex image [nchan,npol,ny,nx] before Re(), sumwt).  Phase
    centres are taken to coincide (no shift)."""
    gax = grid_axes(img, nw, wstep)
    maps = convolution_mapping(uvw, frequency, gax, cax)
    if not np.all(rows_in_grid(maps, gax['shape'], cf.shape)):
        raise AssertionError("rows outside the grid")
    v = np.ones_like(vis) if dopsf else vis
    g, sumwt = (grid_vec if vectorised else grid_loop)(v, wt, maps, cf, gax['shape'])
    im = fft_griddata_to_image(g, gcf)
    if normalize:
        im = normalize_sumwt(im, sumwt)
    return im, sumwt


def predict_2d(uvw, frequency, model, img, gcf, cf, cax, vectorised=True):
    """Returns predicted vis [nvis, npol] (``imaging/base.py:104-138``)."""
    gax = grid_axes(img, 1, 1e15)
    maps = convolution_mapping(uvw, frequency, gax, cax)
    if not np.all(rows_in_grid(maps, gax['shape'], cf.shape)):
        raise AssertionError("rows outside the grid")
    g = fft_image_to_griddata(model, gcf, 1)
    return (degrid_vec if vectorised else degrid_loop)(g, maps, cf)


# ---------------------------------------------------------------------------
# a14: w-stacking (imaging/wstack_single.py:26-96, visibility/iterators.py:91-109,
#      workflows/serial/imaging/imaging_serial.py:41-216)
# ---------------------------------------------------------------------------
def wslice_rows(w, vis_slices):
    """Boolean row masks of ``vis_wslice_iter``."""
    wmaxabs = np.max(np.abs(w))
    boxes = np.linspace(-wmaxabs, +wmaxabs, vis_slices)
    wstack = boxes[1] - boxes[0] if vis_slices > 1 else 2 * wmaxabs
    return [np.abs(w - box) < 0.5 * wstack for box in boxes]


def invert_wstack(uvw, frequency, vis, wt, img, gcf, cf, cax, vis_slices, cellsize, dopsf=False):
    """Serial w-stack invert: per slice invert_2d at w - mean(w), multiply by the
    slice's w-beam, sumwt-weighted sum, normalise.  Returns (image real, sumwt)."""
    nchan, npol, ny, nx = img['nchan'], img['npol'], img['ny'], img['nx']
    acc = np.zeros((nchan, npol, ny, nx))
    acc_wt = np.zeros((nchan, npol))
    for rows in wslice_rows(uvw[:, 2], vis_slices):
        if not np.any(rows):
            continue
        suvw = uvw[rows].copy()
        wav = np.average(suvw[:, 2])
        suvw[:, 2] -= wav
        im, sumwt = invert_2d(suvw, frequency[rows], vis[rows], wt[rows], img, gcf, cf, cax, dopsf=dopsf)
        wb = w_term_image(nx, cellsize, wav)
        slice_im = wb.real * im.real - wb.imag * im.imag
        acc += sumwt[:, :, None, None] * slice_im
        acc_wt += sumwt
    return normalize_sumwt(acc, acc_wt), acc_wt


def predict_wstack(uvw, frequency, model, img, gcf, cf, cax, vis_slices, cellsize):
    """Serial w-stack predict (``wstack_single.py:26-64``): V = P(Re(wb) M) - i P(Im(wb) M)."""
    out = np.zeros((uvw.shape[0], img['npol']), dtype=np.complex128)
    for rows in wslice_rows(uvw[:, 2], vis_slices):
        if not np.any(rows):
            continue
        suvw = uvw[rows].copy()
        wav = np.average(suvw[:, 2])
        suvw[:, 2] -= wav
        wb = w_term_image(img['nx'], cellsize, wav)
        vr = predict_2d(suvw, frequency[rows], wb.real * model, img, gcf, cf, cax)
        vi = predict_2d(suvw, frequency[rows], wb.imag * model, img, gcf, cf, cax)
        out[rows] = vr - 1j * vi
    return out


# ---------------------------------------------------------------------------
# a13 / a17: point-source phasor and scalar gains
# ---------------------------------------------------------------------------
def simulate_point(uvw, l, m):
    """``processing_library/util/coordinate_support.py:192-212``."""
    s = np.array([l, m, np.sqrt(1 - l ** 2 - m ** 2) - 1.0])
    return np.exp(-2j * np.pi * np.dot(uvw, s))


def phaserotate(vis, uvw, l, m, inverse=False):
    """Visibility part of ``phaserotate_visibility`` with tangent=True
    (``processing_components/visibility/base.py:295-334``)."""
    ph = simulate_point(uvw, l, m)[:, None]
    return vis * ph if inverse else vis * np.conj(ph)


def apply_gains(vis, a1, a2, gain):
    """Scalar ``apply_gaintable`` (``processing_components/calibration/operations.py:134-137``)
    for rows of baseline (a1 < a2), stored at [a2, a1]: V *= g[a2] * conj(g[a1])."""
    return vis * (gain[a2] * np.conj(gain[a1]))[:, None]


def skycoord_to_lmn(ra_deg, dec_deg, ra0_deg, dec0_deg):
    """``skycoord_to_lmn`` (``processing_library/util/coordinate_support.py:150-169``)
    for a direction (ra, dec) relative to the phase centre (ra0, dec0), all in
    degrees: the direction's unit vector in the sky-offset frame of the phase
    centre (astropy's frame: axes rotated by lon0 about z, then by -lat0 about
    y), returned as (y, z, x - 1)."""
    ra, dec, ra0, dec0 = ra_deg * D2R, dec_deg * D2R, ra0_deg * D2R, dec0_deg * D2R
    v = np.array([np.cos(dec) * np.cos(ra), np.cos(dec) * np.sin(ra), np.sin(dec)])
    c, s = np.cos(ra0), np.sin(ra0)
    rz = np.array([[c, s, 0.0], [-s, c, 0.0], [0.0, 0.0, 1.0]])
    c, s = np.cos(-dec0), np.sin(-dec0)
    ry = np.array([[c, 0.0, -s], [0.0, 1.0, 0.0], [s, 0.0, c]])
    x, y, z = ry @ (rz @ v)
    return y, z, x - 1.0


def apply_gaintable_block(vis, time_row, gain, gain_weight, inverse=False):
    """Scalar branch of ``apply_gaintable`` (``processing_components/calibration/
    operations.py:124-140``) on a block [ntimes, nants, nants, nchan] (one
    polarisation) for block times t with a gain-table row time_row[t] >= 0:
    V[t, i, j, c] * lg[i, c] conj(lg[j, c]), lg = gain (or 1/gain where
    |gain| > 0, else 1, for the inverse), zero where the two gain weights
    multiply to 0.  Returns a new array."""
    out = vis.copy()
    for t, k in enumerate(time_row):
        if k < 0:
            continue
        g = gain[k]
        if inverse:
            lg = np.ones_like(g)
            lg[np.abs(g) > 0.0] = 1.0 / g[np.abs(g) > 0.0]
        else:
            lg = g
        for c in range(vis.shape[3]):
            m = np.outer(lg[:, c], np.conjugate(lg[:, c]))
            ww = np.outer(gain_weight[k][:, c], gain_weight[k][:, c])
            out[t, :, :, c] = out[t, :, :, c] * m
            out[t, :, :, c][ww == 0.0] = 0.0
    return out
