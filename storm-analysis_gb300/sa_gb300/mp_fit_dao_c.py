"""
The reference's Gaussian multi-plane fitters (multi_plane/mp_fit_dao_c.py:
MPFitDao, MPFitDao2D) over libsa_cuda.so's mpDaoInitialize2DChannel /
mpDaoNewPeaks: one 2D Gaussian channel per image plane, independent
heights and widths, x / y tied through the planes' affine maps.
"""
import ctypes

import numpy

from . import mp_fit_c
from .dao_fit_c import formatPeaksGaussianPSF


class MPFitDao(mp_fit_c.MPFit):

    def __init__(self, n_channels=None, roi_size=None, sigma_range=None, **kwds):
        super(MPFitDao, self).__init__(**kwds)
        self.independent_heights = 1
        self.n_channels = n_channels
        self.roi_size = roi_size
        self.sigma_range = sigma_range

    def formatPeaks(self, peaks, peaks_type):
        return formatPeaksGaussianPSF(peaks, peaks_type)

    def newPeaks(self, peaks, peaks_type):
        c_peaks = formatPeaksGaussianPSF(peaks, peaks_type)
        self._clear_error()
        self.clib.mpDaoNewPeaks(self.mfit, c_peaks, ctypes.c_char_p(peaks_type.encode()), c_peaks.shape[0])
        self._check("newPeaks")


class MPFitDao2D(MPFitDao):

    def initializeChannel(self, rqe, variance, channel):
        super(MPFitDao2D, self).initializeChannel(rqe, variance, channel)
        width_max = 1.0 / (2.0 * self.sigma_range[0] * self.sigma_range[0])
        width_min = 1.0 / (2.0 * self.sigma_range[1] * self.sigma_range[1])
        self.clib.mpDaoInitialize2DChannel(self.mfit, numpy.ascontiguousarray(rqe, dtype=numpy.float64),
                                           numpy.ascontiguousarray(variance, dtype=numpy.float64), width_min,
                                           width_max, self.roi_size, channel)
        self._channel_ready(channel, "mpDaoInitialize2DChannel")

    def setWeights(self, weights=None, verbose=True):
        """Equal weights for every channel (the fit has no z to weight by)."""
        super(MPFitDao2D, self).setWeights(mp_fit_c.equal_weights(self.n_channels), 0.0, 0.0, verbose=verbose)
