"""ARL data models used on the gridding path, without astropy.

Field names, array shapes and axis orders follow ARL's
``data_models/memory_data_models.py`` so code written against ARL keeps
working:

* ``Visibility.data``   structured array with fields index, uvw (wavelengths),
  time, frequency, channel_bandwidth, integration_time, antenna1, antenna2,
  vis [npol], weight [npol], imaging_weight [npol]  (:745-937)
* ``BlockVisibility``   uvw [ntimes, nants, nants, 3] in metres, vis
  [ntimes, nants, nants, nchan, npol]  (:940-1093)
* ``Image.data``        [nchan, npol, ny, nx]  (:349-434)
* ``GridData.data``     [nchan, npol, nw, ny, nx]  (:437-524)
* ``ConvolutionFunction.data`` [nchan, npol, nz, O, O, S, S]  (:527-614)

``data`` may also be a CUDA ``torch.Tensor`` of the same shape for the
grid, image and convolution-function models, in which case the GPU entry
points use it in place without host copies.
"""
import copy

import numpy

from .wcs import WCS


class PolarisationFrame:
    """Named polarisation frames (``data_models/polarisation.py:66``)."""
    fits_codes = {
        'circular': [-1, -2, -3, -4], 'circularnp': [-1, -4], 'linear': [-5, -6, -7, -8],
        'linearnp': [-5, -8], 'stokesIQUV': [1, 2, 3, 4], 'stokesIV': [1, 4], 'stokesIQ': [1, 2],
        'stokesI': [1]}

    def __init__(self, name):
        if name not in self.fits_codes:
            raise ValueError('Unknown polarisation frame %s' % name)
        self.type = name
        self.translations = {i: i for i in range(len(self.fits_codes[name]))}

    @property
    def npol(self):
        return len(self.fits_codes[self.type])

    def __eq__(self, other):
        return isinstance(other, PolarisationFrame) and other.type == self.type

    def __repr__(self):
        return 'Polarisation frame: %s' % self.type


class PhaseCentre:
    """Celestial direction in degrees (stands in for SkyCoord on this path)."""

    def __init__(self, ra_deg, dec_deg):
        self.ra_deg = float(ra_deg)
        self.dec_deg = float(dec_deg)

    @property
    def ra_rad(self):
        return numpy.deg2rad(self.ra_deg)

    @property
    def dec_rad(self):
        return numpy.deg2rad(self.dec_deg)

    def lmn(self, phasecentre):
        """(l, m, n - 1) of this direction relative to ``phasecentre``
        (``skycoord_to_lmn``, coordinate_support.py:150-169)."""
        ra, dec, ra0, dec0 = self.ra_rad, self.dec_rad, phasecentre.ra_rad, phasecentre.dec_rad
        dra = ra - ra0
        l = numpy.cos(dec) * numpy.sin(dra)
        m = numpy.sin(dec) * numpy.cos(dec0) - numpy.cos(dec) * numpy.sin(dec0) * numpy.cos(dra)
        x = numpy.sin(dec) * numpy.sin(dec0) + numpy.cos(dec) * numpy.cos(dec0) * numpy.cos(dra)
        return l, m, x - 1.0

    def separation_rad(self, other):
        l, m, n1 = self.lmn(other)
        return float(numpy.arctan2(numpy.hypot(l, m), n1 + 1.0))

    def __repr__(self):
        return 'PhaseCentre(ra=%.6f deg, dec=%.6f deg)' % (self.ra_deg, self.dec_deg)


def _vis_dtype(npol):
    return [('index', 'i8'), ('uvw', 'f8', (3,)), ('time', 'f8'), ('frequency', 'f8'),
            ('channel_bandwidth', 'f8'), ('integration_time', 'f8'), ('antenna1', 'i8'), ('antenna2', 'i8'),
            ('vis', 'c16', (npol,)), ('weight', 'f8', (npol,)), ('imaging_weight', 'f8', (npol,))]


class Visibility:
    """Row-based visibility table (``memory_data_models.py:745-937``)."""

    def __init__(self, data=None, frequency=None, channel_bandwidth=None, phasecentre=None, configuration=None,
                 uvw=None, time=None, antenna1=None, antenna2=None, vis=None, weight=None, imaging_weight=None,
                 integration_time=None, polarisation_frame=PolarisationFrame('stokesI'), cindex=None,
                 blockvis=None, source='anonymous', meta=None):
        if data is None and vis is not None:
            if imaging_weight is None:
                imaging_weight = weight
            nvis = vis.shape[0]
            data = numpy.zeros(shape=[nvis], dtype=_vis_dtype(polarisation_frame.npol))
            data['index'] = numpy.arange(nvis)
            data['uvw'] = uvw
            data['time'] = time if time is not None else 0.0
            data['frequency'] = frequency
            data['channel_bandwidth'] = channel_bandwidth if channel_bandwidth is not None else 0.0
            data['integration_time'] = integration_time if integration_time is not None else 0.0
            data['antenna1'] = antenna1 if antenna1 is not None else 0
            data['antenna2'] = antenna2 if antenna2 is not None else 0
            data['vis'] = vis
            data['weight'] = weight
            data['imaging_weight'] = imaging_weight
        self.data = data
        self.cindex = cindex
        self.blockvis = blockvis
        self.phasecentre = phasecentre
        self.configuration = configuration
        self.polarisation_frame = polarisation_frame
        self.source = source
        self.meta = meta

    @property
    def npol(self):
        return self.polarisation_frame.npol

    @property
    def nvis(self):
        return self.data['vis'].shape[0]

    @property
    def uvw(self):
        return self.data['uvw']

    @property
    def u(self):
        return self.data['uvw'][:, 0]

    @property
    def v(self):
        return self.data['uvw'][:, 1]

    @property
    def w(self):
        return self.data['uvw'][:, 2]

    @property
    def time(self):
        return self.data['time']

    @property
    def frequency(self):
        return self.data['frequency']

    @property
    def channel_bandwidth(self):
        return self.data['channel_bandwidth']

    @property
    def antenna1(self):
        return self.data['antenna1']

    @property
    def antenna2(self):
        return self.data['antenna2']

    @property
    def vis(self):
        return self.data['vis']

    @property
    def weight(self):
        return self.data['weight']

    @property
    def imaging_weight(self):
        return self.data['imaging_weight']

    def size(self):
        return self.data.nbytes / 1024.0 ** 3


class BlockVisibility:
    """Baseline-block visibility table (``memory_data_models.py:940-1093``).

    ``data`` is ARL's structured array with one record per time: index, uvw
    [nants, nants, 3] in metres, time, integration_time, vis / weight /
    imaging_weight [nants, nants, nchan, npol].  Baseline (a1 < a2) is stored
    at [a2, a1]."""

    def __init__(self, data=None, frequency=None, channel_bandwidth=None, phasecentre=None, configuration=None,
                 uvw=None, time=None, vis=None, weight=None, integration_time=None,
                 polarisation_frame=PolarisationFrame('stokesI'), imaging_weight=None, source='anonymous',
                 meta=None):
        if data is None and vis is not None:
            ntimes, nants, _, nchan, npol = vis.shape
            if weight is None:
                weight = numpy.ones(vis.shape)
            if imaging_weight is None:
                imaging_weight = weight
            assert numpy.shape(weight) == vis.shape
            assert len(frequency) == nchan and len(channel_bandwidth) == nchan
            desc = [('index', 'i8'), ('uvw', 'f8', (nants, nants, 3)), ('time', 'f8'),
                    ('integration_time', 'f8'), ('vis', 'c16', (nants, nants, nchan, npol)),
                    ('weight', 'f8', (nants, nants, nchan, npol)),
                    ('imaging_weight', 'f8', (nants, nants, nchan, npol))]
            data = numpy.zeros(shape=[ntimes], dtype=desc)
            data['index'] = numpy.arange(ntimes)
            data['uvw'] = uvw
            data['time'] = time if time is not None else 0.0
            data['integration_time'] = integration_time if integration_time is not None else 0.0
            data['vis'] = vis
            data['weight'] = weight
            data['imaging_weight'] = imaging_weight
        self.data = data
        self.frequency = numpy.asarray(frequency, dtype=numpy.float64)
        self.channel_bandwidth = numpy.asarray(channel_bandwidth, dtype=numpy.float64)
        self.phasecentre = phasecentre
        self.configuration = configuration
        self.polarisation_frame = polarisation_frame
        self.source = source
        self.meta = meta

    @property
    def nants(self):
        return self.data['vis'].shape[1]

    @property
    def nchan(self):
        return self.data['vis'].shape[3]

    @property
    def npol(self):
        return self.data['vis'].shape[4]

    @property
    def uvw(self):
        return self.data['uvw']

    @property
    def time(self):
        return self.data['time']

    @property
    def integration_time(self):
        return self.data['integration_time']

    @property
    def vis(self):
        return self.data['vis']

    @property
    def weight(self):
        return self.data['weight']

    @property
    def imaging_weight(self):
        return self.data['imaging_weight']


def copy_blockvisibility(bvis, zero=False):
    """``copy_visibility`` for a BlockVisibility (``visibility/base.py``)."""
    out = copy.copy(bvis)
    out.data = bvis.data.copy()
    if zero:
        out.data['vis'][...] = 0.0
    return out


class Skycomponent:
    """A point component (``memory_data_models.py`` Skycomponent): direction,
    frequency [nchan], flux [nchan, npol], shape 'Point'."""

    def __init__(self, direction=None, frequency=None, name=None, flux=None, shape='Point',
                 polarisation_frame=PolarisationFrame('stokesI'), params=None):
        self.direction = direction
        self.frequency = numpy.asarray(frequency, dtype=numpy.float64)
        self.name = name
        self.flux = numpy.asarray(flux, dtype=numpy.float64)
        self.shape = shape
        self.polarisation_frame = polarisation_frame
        self.params = params if params is not None else {}

    @property
    def nchan(self):
        return self.flux.shape[0]

    @property
    def npol(self):
        return self.flux.shape[1]


class ReceptorFrame:
    """Receptors of a gain table (``data_models/polarisation.py`` ReceptorFrame):
    'circular' (R, L), 'linear' (X, Y) or 'stokesI' (I)."""
    _frames = {'circular': ('R', 'L'), 'linear': ('X', 'Y'), 'stokesI': ('I',)}

    def __init__(self, name):
        if name not in self._frames:
            raise ValueError('Unknown receptor frame %s' % str(name))
        self.type = name

    @property
    def nrec(self):
        return len(self._frames[self.type])


class GainTable:
    """Antenna gains over time (``memory_data_models.py`` GainTable): ARL's
    structured array with one record per solution time: gain [nants, nchan,
    nrec, nrec] complex, weight [nants, nchan, nrec, nrec], residual [nchan,
    nrec, nrec], time and interval (seconds).  V_obs = g_i g_j^* V_model."""

    def __init__(self, data=None, gain=None, time=None, interval=None, weight=None, residual=None, frequency=None,
                 receptor_frame=ReceptorFrame('linear'), phasecentre=None, configuration=None):
        if data is None and gain is not None:
            nrec = receptor_frame.nrec
            nrows, nants, nchan = gain.shape[0], gain.shape[1], gain.shape[2]
            assert len(frequency) == nchan, 'Discrepancy in frequency channels'
            desc = [('gain', 'c16', (nants, nchan, nrec, nrec)), ('weight', 'f8', (nants, nchan, nrec, nrec)),
                    ('residual', 'f8', (nchan, nrec, nrec)), ('time', 'f8'), ('interval', 'f8')]
            data = numpy.zeros(shape=[nrows], dtype=desc)
            data['gain'] = gain
            data['weight'] = weight
            data['time'] = time
            data['interval'] = interval
            data['residual'] = residual
        self.data = data
        self.frequency = numpy.asarray(frequency, dtype=numpy.float64)
        self.receptor_frame = receptor_frame
        self.phasecentre = phasecentre
        self.configuration = configuration

    @property
    def time(self):
        return self.data['time']

    @property
    def interval(self):
        return self.data['interval']

    @property
    def gain(self):
        return self.data['gain']

    @property
    def weight(self):
        return self.data['weight']

    @property
    def ntimes(self):
        return self.data['gain'].shape[0]

    @property
    def nants(self):
        return self.data['gain'].shape[1]

    @property
    def nchan(self):
        return self.data['gain'].shape[2]

    @property
    def nrec(self):
        return self.receptor_frame.nrec


class Image:
    """Image [nchan, npol, ny, nx] with its WCS (``memory_data_models.py:349-434``)."""

    def __init__(self, data=None, wcs=None, polarisation_frame=None):
        self.data = data
        self.wcs = wcs
        self.polarisation_frame = polarisation_frame

    @property
    def shape(self):
        return tuple(self.data.shape)

    @property
    def nchan(self):
        return self.data.shape[0]

    @property
    def npol(self):
        return self.data.shape[1]

    @property
    def phasecentre(self):
        return PhaseCentre(self.wcs.wcs.crval[0], self.wcs.wcs.crval[1])

    @property
    def frequency(self):
        w = self.wcs.wcs
        return w.crval[3] + w.cdelt[3] * (numpy.arange(self.nchan) + 1.0 - w.crpix[3])


class GridData:
    """Gridded visibilities [nchan, npol, nw, ny, nx] (``memory_data_models.py:437-524``)."""

    def __init__(self, data=None, grid_wcs=None, projection_wcs=None, polarisation_frame=None):
        self.data = data
        self.grid_wcs = grid_wcs
        self.projection_wcs = projection_wcs
        self.polarisation_frame = polarisation_frame

    @property
    def shape(self):
        return tuple(self.data.shape)


class ConvolutionFunction:
    """Oversampled gridding kernel [nchan, npol, nz, O, O, S, S]
    (``memory_data_models.py:527-614``).

    ``plane_support`` (optional, GB300 extension) holds an even support per
    z-plane; taps outside the central plane_support[z] square of plane z are
    zero in ``data`` and skipped on the GPU."""

    def __init__(self, data=None, grid_wcs=None, projection_wcs=None, polarisation_frame=None):
        self._data = data
        self.version = 0
        self.grid_wcs = grid_wcs
        self.projection_wcs = projection_wcs
        self.polarisation_frame = polarisation_frame
        self.plane_support = None
        self._device_cache = {}

    @property
    def data(self):
        return self._data

    @data.setter
    def data(self, value):
        self._data = value
        self.version += 1
        self._device_cache = {}

    @property
    def shape(self):
        return tuple(self._data.shape)


class QA:
    """Quality assessment record (``memory_data_models.py:1096-1122``)."""

    def __init__(self, origin=None, data=None, context=None):
        self.origin = origin
        self.data = data
        self.context = context

    def __str__(self):
        return 'Quality assessment: origin %s, context %s, data %s' % (self.origin, self.context, self.data)


def copy_visibility(vis, zero=False):
    """``processing_components/visibility/base.py:33-47``."""
    newvis = copy.copy(vis)
    newvis.data = numpy.copy(vis.data)
    if zero:
        newvis.data['vis'][...] = 0.0
    return newvis


def create_visibility_from_rows(vis, rows, makecopy=True):
    """``processing_components/visibility/base.py:252-292``."""
    if rows is None or numpy.sum(rows) == 0:
        return None
    assert len(rows) == vis.nvis, "Length of rows does not agree with length of visibility"
    newvis = copy_visibility(vis) if makecopy else vis
    newvis.data = copy.deepcopy(vis.data[rows])
    return newvis


def create_image(npixel=512, cellsize=0.000015, polarisation_frame=PolarisationFrame('stokesI'),
                 frequency=numpy.array([1e8]), channel_bandwidth=numpy.array([1e6]), phasecentre=None, nchan=None):
    """Empty template image (``processing_library/image/operations.py:31-69``)."""
    if phasecentre is None:
        phasecentre = PhaseCentre(15.0, -35.0)
    if polarisation_frame is None:
        polarisation_frame = PolarisationFrame('stokesI')
    npol = polarisation_frame.npol
    if nchan is None:
        nchan = len(frequency)
    w = WCS(4)
    w.wcs.cdelt = [-cellsize * 180.0 / numpy.pi, cellsize * 180.0 / numpy.pi, 1.0, channel_bandwidth[0]]
    w.wcs.crpix = [npixel // 2 + 1, npixel // 2 + 1, 1.0, 1.0]
    w.wcs.ctype = ['RA---SIN', 'DEC--SIN', 'STOKES', 'FREQ']
    w.wcs.crval = [phasecentre.ra_deg, phasecentre.dec_deg, 1.0, frequency[0]]
    w.naxis = 4
    return Image(numpy.zeros([nchan, npol, npixel, npixel]), w, polarisation_frame)


def create_image_from_array(data, wcs, polarisation_frame):
    """``processing_library/image/operations.py:72-97`` (keeps a reference to data)."""
    return Image(data, None if wcs is None else wcs.deepcopy(), polarisation_frame)


def copy_image(im):
    return Image(im.data.clone() if hasattr(im.data, 'clone') else copy.deepcopy(im.data),
                 None if im.wcs is None else im.wcs.deepcopy(), im.polarisation_frame)


def create_empty_image_like(im):
    return Image(numpy.zeros(im.shape), None if im.wcs is None else im.wcs.deepcopy(), im.polarisation_frame)
