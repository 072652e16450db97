"""
GPU matched filter behind the reference's MatchedFilter class
(sa_library/matched_filter_c.py:44-100): same constructor arguments, same
convolve() / cleanup() and the same exception on a shape mismatch.  The
PSF is recentred for circular convolution as the reference recentres it
(sa_library/recenter_psf.py:11-19) and handed to saFilterCreate.
"""
import ctypes

import numpy

from . import loadclib


class MatchedFilterException(Exception):
    pass


def recenterPSF(psf):
    rc = numpy.roll(psf, int(psf.shape[0] / 2), axis=0)
    return numpy.roll(rc, int(psf.shape[1] / 2), axis=1)


class MatchedFilter(object):

    def __init__(self, psf, fftw_estimate=False, memoize=False, max_diff=0.1):
        self.clib = loadclib.load()
        self.memoize = memoize
        self.psf_shape = psf.shape
        rc = numpy.ascontiguousarray(recenterPSF(psf), dtype=numpy.float64)
        self.mfilter = self.clib.saFilterCreate(rc, float(max_diff) if memoize else 0.0,
                                                rc.shape[0], rc.shape[1], int(fftw_estimate))
        if not self.mfilter:
            raise MatchedFilterException(loadclib.last_error())

    def cleanup(self):
        if self.mfilter:
            self.clib.saFilterCleanup(self.mfilter)
        self.mfilter = None

    def convolve(self, image):
        if (image.shape[0] != self.psf_shape[0]) or (image.shape[1] != self.psf_shape[1]):
            raise MatchedFilterException("Image shape must match psf shape! " + str(image.shape) +
                                         " != " + str(self.psf_shape))
        image = numpy.ascontiguousarray(image, dtype=numpy.float64)
        result = numpy.zeros(self.psf_shape, dtype=numpy.float64)
        fn = self.clib.saFilterConvolveMemo if self.memoize else self.clib.saFilterConvolve
        if fn(self.mfilter, image, result) != 0:
            raise MatchedFilterException(loadclib.last_error())
        return result

    def info(self):
        """(separable, taps along rows, taps along columns, first row
        offset, first column offset, frames allocated)."""
        out = numpy.zeros(6, dtype=numpy.int32)
        self.clib.saFilterInfo(self.mfilter, out)
        return tuple(int(v) for v in out)

    def handle(self):
        return self.mfilter
