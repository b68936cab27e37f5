"""Minimal stand-in for the parts of astropy that ARL's gridding path touches.

Used only by ``make_golden.py`` to import the reference's own Python modules in
a container where astropy is not installed.  Everything the gridding path
computes with is a *linear* FITS axis (UU, VV, DUU, DVV, WW, STOKES, FREQ),
so ``WCS`` below implements exactly the linear world<->pixel transform with an
identity PC matrix.  Celestial objects (SkyCoord, units) are inert
placeholders: the fixtures are built with visibility and image phase centres
equal, so no phase rotation is ever computed through them.
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


class _Angle:
    def __init__(self, deg):
        self.deg = float(deg)
        self.rad = float(deg) * numpy.pi / 180.0


class _Separation:
    rad = 0.0


class SkyCoord:
    """Phase-centre placeholder: every separation is zero."""

    def __init__(self, ra=0.0, dec=0.0, *a, **k):
        ra = ra if isinstance(ra, (int, float)) else 0.0
        dec = dec if isinstance(dec, (int, float)) else 0.0
        self.ra = _Angle(ra)
        self.dec = _Angle(dec)

    def separation(self, other):
        return _Separation()


class _WcsPrm:
    def __init__(self, naxis):
        self.naxis = naxis
        self.ctype = [''] * naxis
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
    'astropy.constants': {'c': types.SimpleNamespace(value=299792458.0)},
    'astropy.wcs': {'WCS': WCS, 'FITSFixedWarning': UserWarning},
    'astropy.wcs.utils': {'pixel_to_skycoord': pixel_to_skycoord},
    'astropy.coordinates': {'SkyCoord': SkyCoord},
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
