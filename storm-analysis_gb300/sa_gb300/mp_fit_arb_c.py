"""
The reference's arbitrary-PSF multi-plane fitters (multi_plane/
mp_fit_arb_c.py: MPFitArb, MPPSFFnFit, MPPupilFnFit, MPSplineFit) over
libsa_cuda.so's mpArbInitialize*Channel / mpArbNewPeaks.  psf_objects: one
PSF object per channel (psf_fft_c.PSFFnBase / pupil_fn.PupilFunction /
cubic_fit_c.SplineToPSF3D-like objects with getCPointer(), getSize() and,
for the z weights, getZMin() / getZMax() / getZSize()).
"""
import ctypes

import numpy

from . import mp_fit_c
from .dao_fit_c import formatPeaksArbitraryPSF


class MPFitArb(mp_fit_c.MPFit):

    def __init__(self, independent_heights=None, psf_objects=None, **kwds):
        super(MPFitArb, self).__init__(**kwds)
        self.independent_heights = int(bool(independent_heights))
        self.n_channels = len(psf_objects)
        self.psf_objects = psf_objects

    def getSize(self):
        return self.psf_objects[0].getSize()

    def formatPeaks(self, peaks, peaks_type):
        return formatPeaksArbitraryPSF(peaks, peaks_type)

    def newPeaks(self, peaks, peaks_type):
        c_peaks = formatPeaksArbitraryPSF(peaks, peaks_type)
        self._clear_error()
        self.clib.mpArbNewPeaks(self.mfit, c_peaks, ctypes.c_char_p(peaks_type.encode()), c_peaks.shape[0])
        self._check("newPeaks")


class MPPSFFnFit(MPFitArb):
    """PSF FFT channels (mpArbInitializePSFFFTChannel)."""

    def initializeChannel(self, rqe, variance, channel):
        super(MPPSFFnFit, self).initializeChannel(rqe, variance, channel)
        self.clib.mpArbInitializePSFFFTChannel(self.mfit, self.psf_objects[channel].getCPointer(),
                                               numpy.ascontiguousarray(rqe, dtype=numpy.float64),
                                               numpy.ascontiguousarray(variance, dtype=numpy.float64), channel)
        self._channel_ready(channel, "mpArbInitializePSFFFTChannel")

    def rescaleZ(self, z):
        return self.psf_objects[0].rescaleZ(z)

    def setWeights(self, weights, verbose=True):
        if weights is None:
            super(MPPSFFnFit, self).setWeights(mp_fit_c.equal_weights(self.n_channels), 0.0, 0.0, verbose=verbose)
        else:
            z_offset = -0.5 * float(self.psf_objects[0].getZSize())
            z_scale = float(weights["bg"].shape[0] - 1) / float(self.psf_objects[0].getZSize())
            super(MPPSFFnFit, self).setWeights(weights, z_offset, z_scale, verbose=verbose)


class MPPupilFnFit(MPFitArb):
    """Pupil-function channels (mpArbInitializePupilFnChannel), z range in
    microns from the PSF objects' nanometers."""

    def initializeChannel(self, rqe, variance, channel):
        super(MPPupilFnFit, self).initializeChannel(rqe, variance, channel)
        zmax = self.psf_objects[0].getZMax() * 1.0e-3
        zmin = self.psf_objects[0].getZMin() * 1.0e-3
        self.clib.mpArbInitializePupilFnChannel(self.mfit, self.psf_objects[channel].getCPointer(),
                                                numpy.ascontiguousarray(rqe, dtype=numpy.float64),
                                                numpy.ascontiguousarray(variance, dtype=numpy.float64),
                                                zmin, zmax, channel)
        self._channel_ready(channel, "mpArbInitializePupilFnChannel")

    def setWeights(self, weights, verbose=True):
        if weights is None:
            super(MPPupilFnFit, self).setWeights(mp_fit_c.equal_weights(self.n_channels), 0.0, 0.0, verbose=verbose)
        else:
            zmax = self.psf_objects[0].getZMax() * 1.0e-3
            zmin = self.psf_objects[0].getZMin() * 1.0e-3
            z_scale = float(weights["bg"].shape[0] - 1) / (zmax - zmin + 1.0e-12)
            super(MPPupilFnFit, self).setWeights(weights, zmin, z_scale, verbose=verbose)


class MPSplineFit(MPFitArb):
    """3D spline channels (mpArbInitializeSplineChannel)."""

    def initializeChannel(self, rqe, variance, channel):
        super(MPSplineFit, self).initializeChannel(rqe, variance, channel)
        self.clib.mpArbInitializeSplineChannel(self.mfit, self.psf_objects[channel].getCPointer(),
                                               numpy.ascontiguousarray(rqe, dtype=numpy.float64),
                                               numpy.ascontiguousarray(variance, dtype=numpy.float64), channel)
        self._channel_ready(channel, "mpArbInitializeSplineChannel")

    def rescaleZ(self, z):
        return self.psf_objects[0].rescaleZ(z)

    def setWeights(self, weights, verbose=True):
        if weights is None:
            super(MPSplineFit, self).setWeights(mp_fit_c.equal_weights(self.n_channels), 0.0, 0.0, verbose=verbose)
        else:
            assert weights["bg"].shape[0] == (self.psf_objects[0].getSize() + 1), "Incorrect shape for weights array."
            super(MPSplineFit, self).setWeights(weights, 0.0, 1.0, verbose=verbose)
