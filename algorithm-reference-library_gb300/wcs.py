"""Linear world coordinate system used by the data models.

ARL describes images, grids and convolution functions with astropy WCS objects
(``data_models/memory_data_models.py``).  On the gridding path every axis it
transforms is a linear FITS axis (UU, VV, DUU, DVV, WW, STOKES, FREQ; the
RA---SIN / DEC--SIN image axes are only read for their cdelt / crpix), so this
class carries the same ``wcs.crval / crpix / cdelt / ctype`` numbers and the
linear transform with an identity PC matrix:

    pix (origin 0) = ((world - crval) / cdelt + crpix) - 1
    world          = ((pix + 1) - crpix) * cdelt + crval
"""
import copy

import numpy


class _Prm:
    def __init__(self, naxis):
        self.naxis = naxis
        self.ctype = [''] * naxis
        self.axis_types = [0] * naxis
        self._crval = numpy.zeros(naxis)
        self._crpix = numpy.zeros(naxis)
        self._cdelt = numpy.ones(naxis)
        self.radesys = 'ICRS'
        self.equinox = 2000.0

    def _arr(name):
        def get(self):
            return getattr(self, '_' + name)

        def put(self, value):
            setattr(self, '_' + name, numpy.array(value, dtype=numpy.float64))
        return property(get, put)

    crval = _arr('crval')
    crpix = _arr('crpix')
    cdelt = _arr('cdelt')


class WCS:
    """Subset of ``astropy.wcs.WCS`` for linear axes."""

    def __init__(self, naxis=2):
        self.wcs = _Prm(naxis)
        self.naxis = naxis

    def deepcopy(self):
        return copy.deepcopy(self)

    def sub(self, axes):
        """New WCS made of the given 1-relative axes."""
        out = WCS(len(axes))
        for i, a in enumerate(axes):
            out.wcs.ctype[i] = self.wcs.ctype[a - 1]
            out.wcs.axis_types[i] = self.wcs.axis_types[a - 1]
            out.wcs.crval[i] = self.wcs.crval[a - 1]
            out.wcs.crpix[i] = self.wcs.crpix[a - 1]
            out.wcs.cdelt[i] = self.wcs.cdelt[a - 1]
        return out

    def axis(self, i):
        """(crval, crpix, cdelt) of 0-relative axis i."""
        return float(self.wcs.crval[i]), float(self.wcs.crpix[i]), float(self.wcs.cdelt[i])

    def wcs_world2pix(self, *args):
        *xs, origin = args
        return [((numpy.asarray(x, dtype=numpy.float64) - self.wcs.crval[i]) / self.wcs.cdelt[i]
                 + self.wcs.crpix[i]) - (1.0 - origin) for i, x in enumerate(xs)]

    def wcs_pix2world(self, *args):
        *ps, origin = args
        return [((numpy.asarray(list(p) if isinstance(p, range) else p, dtype=numpy.float64)
                  + (1.0 - origin)) - self.wcs.crpix[i]) * self.wcs.cdelt[i] + self.wcs.crval[i]
                for i, p in enumerate(ps)]

    def __repr__(self):
        return 'WCS(ctype=%s, crval=%s, crpix=%s, cdelt=%s)' % (self.wcs.ctype, self.wcs.crval.tolist(),
                                                               self.wcs.crpix.tolist(), self.wcs.cdelt.tolist())
