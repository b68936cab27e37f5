"""Minimal stand-in for the parts of astropy that ARL's gridding path touches.

Used only by ``make_golden.py`` to import the reference's own Python modules in
a container where astropy is not installed.  Everything the gridding path
computes with is a *linear* FITS axis (UU, VV, DUU, DVV, WW, STOKES, FREQ),
so ``WCS`` below implements exactly the linear world<->pixel transform with an
identity PC matrix.

Celestial directions (``SkyCoord``) carry real RA / Dec and implement the
three operations the reference's phase rotation and component predict use
(``processing_library/util/coordinate_support.py:150-169``):
``separation`` (the Vincenty great-circle formula), ``skyoffset_frame`` /
``transform_to`` (astropy's sky-offset frame: the rotation matrix product
R_x(-rotation) R_y(-lat0) R_z(lon0) applied to the unit vector, with astropy's
``rotation_matrix`` convention of rotating the coordinate axes) and
``represent_as(CartesianRepresentation)`` (through the unit-spherical
representation, as astropy stores a direction without distance).  astropy is
not pinned by the reference (``requirements.txt`` lists it without a
version); the restatement follows its published frame definitions and is
checked in ``make_golden.py`` against every expectation of the reference's own
``test_skycoord_to_lmn`` (``tests/processing_library/test_coordinate_support.py:125-141``).
Other units and celestial objects are inert placeholders.
"""
import copy
import importlib.abc
import importlib.machinery
import sys
import types

import numpy


class _Inert:
    """Absorbs any attribute access / call / arithmetic (unused astropy API)."""

    def __init__(self, *a, **k):
        pass

    def __call__(self, *a, **k):
        return _Inert()

    def __getattr__(self, name):
        if name.startswith('__'):
            raise AttributeError(name)
        return _Inert()

    def __mul__(self, other):
        return self

    __rmul__ = __mul__


class _Unit:
    """An angle unit: ``x * u.deg`` makes a quantity in degrees."""

    def __init__(self, name, to_deg):
        self.name = name
        self.to_deg = to_deg

    def __rmul__(self, x):
        return _Quantity(x, self)

    __mul__ = __rmul__


_DEG = _Unit('deg', 1.0)
_RAD = _Unit('rad', 180.0 / numpy.pi)


class _Quantity:
    def __init__(self, value, unit):
        self.value = value
        self.unit = unit

    def deg(self):
        return numpy.asarray(self.value, dtype=numpy.float64) * self.unit.to_deg


def _as_deg(x, unit=None):
    if isinstance(x, _Quantity):
        return float(x.deg())
    if isinstance(x, (int, float, numpy.floating, numpy.integer)):
        scale = unit.to_deg if isinstance(unit, _Unit) else 1.0
        return float(x) * scale
    return 0.0  # inert placeholder input


class _Angle:
    def __init__(self, deg):
        self.deg = float(deg)
        self.rad = float(deg) * numpy.pi / 180.0
        self.radian = self.rad


class _Separation:
    def __init__(self, rad):
        self.rad = rad
        self.radian = rad
        self.deg = rad * 180.0 / numpy.pi


def _rotation_matrix(angle, axis):
    """astropy's ``rotation_matrix``: rotates the coordinate axes by ``angle``
    (radians) about ``axis`` (0 = x, 1 = y, 2 = z)."""
    c, s = numpy.cos(angle), numpy.sin(angle)
    a1, a2 = (axis + 1) % 3, (axis + 2) % 3
    r = numpy.zeros((3, 3))
    r[axis, axis] = 1.0
    r[a1, a1] = c
    r[a1, a2] = s
    r[a2, a1] = -s
    r[a2, a2] = c
    return r


class _Value:
    def __init__(self, v):
        self.value = v


class _Cartesian:
    def __init__(self, x, y, z):
        self.x, self.y, self.z = _Value(x), _Value(y), _Value(z)


class _SkyOffsetFrame:
    def __init__(self, origin, rotation=0.0):
        self.origin = origin
        self.rotation = rotation


class _OffsetCoord:
    """A direction in a sky-offset frame, stored as (lon, lat) radians."""

    def __init__(self, lon, lat):
        self.lon, self.lat = lon, lat

    def represent_as(self, cls):
        cl = numpy.cos(self.lat)
        return _Cartesian(cl * numpy.cos(self.lon), cl * numpy.sin(self.lon), numpy.sin(self.lat))


class SkyCoord:
    """ICRS direction: ``ra`` / ``dec`` in degrees (numbers, or quantities
    made with ``astropy.units`` deg / rad)."""

    def __init__(self, ra=0.0, dec=0.0, *a, **k):
        unit = k.get('unit')
        self.ra = _Angle(_as_deg(ra, unit))
        self.dec = _Angle(_as_deg(dec, unit))

    def _xyz(self):
        cd = numpy.cos(self.dec.rad)
        return numpy.array([cd * numpy.cos(self.ra.rad), cd * numpy.sin(self.ra.rad), numpy.sin(self.dec.rad)])

    def separation(self, other):
        """Vincenty's formula for the angle between two directions."""
        sd1, cd1 = numpy.sin(self.dec.rad), numpy.cos(self.dec.rad)
        sd2, cd2 = numpy.sin(other.dec.rad), numpy.cos(other.dec.rad)
        dl = other.ra.rad - self.ra.rad
        sdl, cdl = numpy.sin(dl), numpy.cos(dl)
        num1 = cd2 * sdl
        num2 = cd1 * sd2 - sd1 * cd2 * cdl
        den = sd1 * sd2 + cd1 * cd2 * cdl
        return _Separation(float(numpy.arctan2(numpy.hypot(num1, num2), den)))

    def skyoffset_frame(self, rotation=0.0):
        return _SkyOffsetFrame(self, rotation)

    def transform_to(self, frame):
        assert isinstance(frame, _SkyOffsetFrame), frame
        o = frame.origin
        m = _rotation_matrix(-frame.rotation, 0) @ _rotation_matrix(-o.dec.rad, 1) @ _rotation_matrix(o.ra.rad, 2)
        x, y, z = m @ self._xyz()
        return _OffsetCoord(numpy.arctan2(y, x), numpy.arctan2(z, numpy.hypot(x, y)))

    def __repr__(self):
        return 'SkyCoord(%.6f deg, %.6f deg)' % (self.ra.deg, self.dec.deg)


class _WcsPrm:
    def __init__(self, naxis):
        self.naxis = naxis
        self.ctype = [''] * naxis
        self.cunit = [''] * naxis
        self.axis_types = [0] * naxis
        self._crval = numpy.zeros(naxis)
        self._crpix = numpy.zeros(naxis)
        self._cdelt = numpy.ones(naxis)
        self.radesys = ''
        self.equinox = 2000.0

    def _set(name):
        def fget(self):
            return getattr(self, '_' + name)

        def fset(self, value):
            setattr(self, '_' + name, numpy.array(value, dtype=numpy.float64))
        return property(fget, fset)

    crval = _set('crval')
    crpix = _set('crpix')
    cdelt = _set('cdelt')


class WCS:
    """Linear-axis WCS: pix0 = ((x - crval) / cdelt + crpix) - 1 and its inverse."""

    def __init__(self, naxis=2, *a, **k):
        self.wcs = _WcsPrm(naxis)
        self.naxis = naxis

    def deepcopy(self):
        return copy.deepcopy(self)

    def sub(self, axes):
        # 'spectral' / 'celestial' select axes by type, as astropy's sub does
        named = []
        for a in axes:
            if a == 'spectral':
                named += [k + 1 for k in range(self.naxis) if str(self.wcs.ctype[k]).startswith('FREQ')]
            elif a == 'celestial':
                named += [k + 1 for k in range(self.naxis) if str(self.wcs.ctype[k])[:2] in ('RA', 'DE')]
            else:
                named.append(a)
        axes = named
        out = WCS(naxis=len(axes))
        for i, a in enumerate(axes):
            out.wcs.ctype[i] = self.wcs.ctype[a - 1]
            out.wcs.axis_types[i] = self.wcs.axis_types[a - 1]
            out.wcs.crval[i] = self.wcs.crval[a - 1]
            out.wcs.crpix[i] = self.wcs.crpix[a - 1]
            out.wcs.cdelt[i] = self.wcs.cdelt[a - 1]
        return out

    def wcs_world2pix(self, *args):
        *xs, origin = args
        return [((numpy.asarray(x, dtype=numpy.float64) - self.wcs.crval[i]) / self.wcs.cdelt[i]
                 + self.wcs.crpix[i]) - (1.0 - origin) for i, x in enumerate(xs)]

    def wcs_pix2world(self, *args):
        *ps, origin = args
        return [((numpy.asarray(list(p) if isinstance(p, range) else p, dtype=numpy.float64)
                  + (1.0 - origin)) - self.wcs.crpix[i]) * self.wcs.cdelt[i] + self.wcs.crval[i]
                for i, p in enumerate(ps)]


def pixel_to_skycoord(x, y, wcs, origin=0, *a, **k):
    return SkyCoord(float(wcs.wcs.crval[0]), float(wcs.wcs.crval[1]))


class _SpeedOfLight:
    """astropy.constants.c (SI, exact); ``c.to('m s^-1')`` is itself."""
    value = 299792458.0

    def to(self, unit):
        return self


class _Mod(types.ModuleType):
    def __getattr__(self, name):
        if name.startswith('__'):
            raise AttributeError(name)
        full = self.__name__ + '.' + name
        if full in _SPECIAL:  # e.g. ``from astropy import constants``
            return importlib.import_module(full)
        return _Inert


_SPECIAL = {
    # speed of light as astropy.constants.c.value (SI, exact)
    'astropy.constants': {'c': _SpeedOfLight()},
    'astropy.wcs': {'WCS': WCS, 'FITSFixedWarning': UserWarning},
    'astropy.wcs.utils': {'pixel_to_skycoord': pixel_to_skycoord},
    'astropy.coordinates': {'SkyCoord': SkyCoord},
    'astropy.units': {'deg': _DEG, 'rad': _RAD, 'degree': _DEG, 'radian': _RAD},
    'astropy.utils.exceptions': {'AstropyDeprecationWarning': UserWarning},
}
_STUB_ROOTS = ('astropy', 'photutils', 'reproject', 'h5py', 'matplotlib', 'aotools', 'pyfftw')


class _Finder(importlib.abc.MetaPathFinder, importlib.abc.Loader):
    def find_spec(self, name, path, target=None):
        if name.split('.')[0] in _STUB_ROOTS:
            if name.split('.')[0] == 'pyfftw':
                return None
            return importlib.machinery.ModuleSpec(name, self, is_package=True)
        return None

    def create_module(self, spec):
        m = _Mod(spec.name)
        m.__path__ = []
        for k, v in _SPECIAL.get(spec.name, {}).items():
            setattr(m, k, v)
        return m

    def exec_module(self, module):
        pass


def install():
    if not any(isinstance(f, _Finder) for f in sys.meta_path):
        sys.meta_path.insert(0, _Finder())
