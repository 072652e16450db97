"""
The reference's multi-plane fitter base class (multi_plane/mp_fit_c.py
MPFit) over libsa_cuda.so: mpInitialize / mpIterateLM / mpSetTransforms /
mpSetWeights / mpSetWeightsIndexing / mpCleanup, and the per-channel mFit*
calls on the channel handles in the multi-plane handle's fit_data array.
"""
import ctypes

import numpy

from . import loadclib
from .dao_fit_c import MultiFitter, MultiFitterException, printFittingInfo


class MPFit(MultiFitter):
    """Base class for multi-plane fitting: one channel handle per image
    plane; images and backgrounds are lists of n_channels arrays."""

    def __init__(self, **kwds):
        kwds.setdefault("precision", 64)
        super(MPFit, self).__init__(**kwds)
        self.independent_heights = None
        self.n_channels = None

    def _channel(self, i):
        return self.mfit.contents.fit_data[i]

    def cleanup(self, spacing="  ", verbose=True):
        if self.mfit is not None:
            if verbose:
                for i in range(self.n_channels):
                    print()
                    print("Channel", i)
                    printFittingInfo(self._channel(i), spacing=spacing)
                print()
                print(spacing, self.n_proximity, "peaks lost to proximity.")
                print(spacing, self.n_significance, "peaks lost to low significance.")
                print(spacing, "{0:0d} fitting iterations.".format(self.iterations))
            self.clib.mpCleanup(self.mfit)
            self.mfit = None

    def doFit(self, max_iterations=2000):
        """MultiFitter.doFit (sa_library/dao_fit_c.py:332-356) with the
        coupled sweep: one sweep, then sweeps while channel 0 has RUNNING
        groups."""
        i = 0
        self.iterate()
        while self.getUnconverged() and (i < max_iterations):
            self.iterate()
            i += 1
        self.getIterations()

    def getFitImage(self):
        fit_images = []
        for i in range(self.n_channels):
            fit_image = numpy.zeros(self.im_shape)
            self.clib.mFitGetFitImage(self._channel(i), fit_image)
            fit_images.append(fit_image)
        return fit_images

    def getIterations(self):
        for i in range(self.n_channels):
            fit_data = self._channel(i)
            self.iterations += fit_data.contents.n_iterations
            fit_data.contents.n_iterations = 0
        return self.iterations

    def getNError(self, channel=0):
        return self.clib.mFitGetNError(self._channel(channel))

    def getNFit(self, channel=0):
        return self._channel(channel).contents.nfit

    def getNFitMax(self, channel=0):
        return self._channel(channel).contents.max_nfit

    def getPeakProperty(self, p_name, channel=0):
        if p_name not in self.peak_properties:
            raise MultiFitterException("No such property '" + p_name + "'")
        kind = self.peak_properties[p_name]
        if kind == "compound":
            if self.getNFit() == 0:
                return numpy.zeros(0, dtype=numpy.float64)
            bg_sum = numpy.zeros(self.getNFit(), dtype=numpy.float64)
            fg_sum = numpy.zeros(self.getNFit(), dtype=numpy.float64)
            for i in range(self.n_channels):
                bg_sum += self.getPeakProperty("bg_sum", channel=i)
                fg_sum += self.getPeakProperty("fg_sum", channel=i)
            return fg_sum / numpy.sqrt(bg_sum)
        if kind == "float":
            values = numpy.ascontiguousarray(numpy.zeros(self.getNFit(), dtype=numpy.float64))
            self.clib.mFitGetPeakPropertyDouble(self._channel(channel), values, ctypes.c_char_p(p_name.encode()))
            return values
        values = numpy.ascontiguousarray(numpy.zeros(self.getNFit(), dtype=numpy.int32))
        self.clib.mFitGetPeakPropertyInt(self._channel(channel), values, ctypes.c_char_p(p_name.encode()))
        return values

    def getUnconverged(self, channel=0):
        return self.clib.mFitGetUnconverged(self._channel(channel))

    def initializeC(self, variance):
        self.im_shape = variance.shape
        self.mfit = self.clib.mpInitialize(self.default_tol * self.n_channels, self.n_channels,
                                           self.independent_heights, variance.shape[1], variance.shape[0])
        if not self.mfit:
            raise MultiFitterException("mpInitialize failed: " + loadclib.last_error())

    def initializeChannel(self, rqe, variance, channel):
        if self.mfit is None:
            self.initializeC(variance)
        if (rqe.shape[0] != self.im_shape[0]) or (rqe.shape[1] != self.im_shape[1]):
            raise MultiFitterException("Current RQE shape and the original variance shape are not the same.")
        if (variance.shape[0] != self.im_shape[0]) or (variance.shape[1] != self.im_shape[1]):
            raise MultiFitterException("Current variance shape and the original variance shape are not the same.")

    def _channel_ready(self, channel, what):
        if not self._channel(channel):
            raise MultiFitterException(what + " failed: " + loadclib.last_error())

    def iterate(self):
        self._clear_error()
        self.clib.mpIterateLM(self.mfit)
        self._check("mpIterateLM")

    def newBackground(self, background):
        if len(background) != self.n_channels:
            raise MultiFitterException("Number of images does not match number of channels.")
        for i in range(self.n_channels):
            if (background[i].shape[0] != self.im_shape[0]) or (background[i].shape[1] != self.im_shape[1]):
                raise MultiFitterException("Background image shape and the original image shape are not the same.")
            self.clib.mFitNewBackground(self._channel(i), numpy.ascontiguousarray(background[i], dtype=numpy.float64))

    def newImage(self, image):
        if len(image) != self.n_channels:
            raise MultiFitterException("Number of images does not match number of channels.")
        for i in range(self.n_channels):
            if (image[i].shape[0] != self.im_shape[0]) or (image[i].shape[1] != self.im_shape[1]):
                raise MultiFitterException("Current image shape and the original image shape are not the same.")
            self.clib.mFitNewImage(self._channel(i), numpy.ascontiguousarray(image[i], dtype=numpy.float64))

    def removeErrorPeaks(self, check=True):
        for i in range(self.n_channels):
            self.clib.mFitRemoveErrorPeaks(self._channel(i))
        if check:
            for i in range(1, self.n_channels):
                assert self.getNFit(0) == self.getNFit(i)

    def removeRunningPeaks(self, check=True):
        for i in range(self.n_channels):
            self.clib.mFitRemoveRunningPeaks(self._channel(i))
        if check:
            for i in range(1, self.n_channels):
                assert self.getNFit(0) == self.getNFit(i)

    def rescaleZ(self, z):
        return z

    def fitBatch(self, images, backgrounds, peaks, peaks_type, max_iterations=2000):
        """Batched multi-plane fit of many frames at once (no reference
        counterpart; the channels must be initialised and the mapping and
        weights set): images / backgrounds per channel an (F, ny, nx)
        array, peaks a list of F dicts of columns (channel 0's
        coordinates).  Returns (per channel a dict of the frames' peaks'
        x, y, z, height, background, xsigma, ysigma, error, status,
        iterations, frames one after another; the number of sweeps)."""
        rows = [self.formatPeaks(p, peaks_type) for p in peaks]
        counts = [r.shape[0] for r in rows]
        allrows = numpy.ascontiguousarray(numpy.concatenate(rows, axis=0))
        return _batch_fit(self, images, backgrounds, allrows, counts, peaks_type, max_iterations)

    def setMapping(self, xt_0toN, yt_0toN, xt_Nto0, yt_Nto0):
        self.clib.mpSetTransforms(self.mfit, numpy.ascontiguousarray(xt_0toN, dtype=numpy.float64),
                                  numpy.ascontiguousarray(yt_0toN, dtype=numpy.float64),
                                  numpy.ascontiguousarray(xt_Nto0, dtype=numpy.float64),
                                  numpy.ascontiguousarray(yt_Nto0, dtype=numpy.float64))

    def setPeakStatus(self, status):
        assert status.size == self.getNFit()
        for i in range(self.n_channels):
            self.clib.mFitSetPeakStatus(self._channel(i), numpy.ascontiguousarray(status, dtype=numpy.int32))

    def setWeights(self, weights, z_offset, z_scale, verbose=True):
        """weights: dict of (z_size, n_channels) arrays "bg", "h", "x", "y",
        "z", all positive (z the slow index)."""
        assert weights["h"].shape[1] == self.n_channels, "Incorrect shape for weights array."
        ws = [numpy.ascontiguousarray(weights[k], dtype=numpy.float64) for k in ("bg", "h", "x", "y", "z")]
        for w in ws:
            assert numpy.count_nonzero(w > 0.0) == w.size
        self.clib.mpSetWeights(self.mfit, *ws, ws[0].shape[0])
        if verbose:
            print("weights z scaling - offset: {0:.3f} scale: {1:.3f}".format(z_offset, z_scale))
        self.clib.mpSetWeightsIndexing(self.mfit, z_offset, z_scale)


def _batch_fit(fitter, images, backgrounds, rows, counts, peaks_type, max_iterations):
    """The batched multi-plane fit behind MPFit.fitBatch."""
    lib = fitter.clib
    n_frames = images[0].shape[0]
    cap = max(1, int(max(counts)))
    if lib.mpSetFrames(fitter.mfit, n_frames, cap) != 0:
        raise MultiFitterException("mpSetFrames: " + loadclib.last_error())
    for c in range(fitter.n_channels):
        ch = fitter._channel(c)
        a = numpy.ascontiguousarray(images[c], dtype=numpy.float64)
        b = numpy.ascontiguousarray(backgrounds[c], dtype=numpy.float64)
        if lib.saNewImages(ch, a.ctypes.data_as(ctypes.c_void_p), n_frames, 64, 0) != 0:
            raise MultiFitterException("saNewImages: " + loadclib.last_error())
        if lib.saNewBackgrounds(ch, b.ctypes.data_as(ctypes.c_void_p), n_frames, 64, 0) != 0:
            raise MultiFitterException("saNewBackgrounds: " + loadclib.last_error())
    counts = numpy.ascontiguousarray(counts, dtype=numpy.int32)
    if lib.mpNewPeaksBatch(fitter.mfit, rows, counts, peaks_type.encode()) != 0:
        raise MultiFitterException("mpNewPeaksBatch: " + loadclib.last_error())
    sweeps = lib.mpDoFitBatch(fitter.mfit, int(max_iterations))
    if sweeps < 0:
        raise MultiFitterException("mpDoFitBatch: " + loadclib.last_error())
    out = []
    n = int(counts.sum())
    for c in range(fitter.n_channels):
        vals = numpy.zeros((n, 8), dtype=numpy.float64)
        ints = numpy.zeros((n, 2), dtype=numpy.int32)
        if n and lib.saGetResultsBatch(fitter._channel(c), vals, ints) < 0:
            raise MultiFitterException("saGetResultsBatch: " + loadclib.last_error())
        d = {k: vals[:, i] for i, k in enumerate(("x", "y", "z", "height", "background", "xsigma", "ysigma",
                                                     "error"))}
        d["status"] = ints[:, 0]
        d["iterations"] = ints[:, 1]
        out.append(d)
    return out, sweeps


def equal_weights(n_channels):
    """Equal weights for every channel at two z points (the reference's
    default when no weights are given)."""
    w = numpy.ones((2, n_channels)) / float(n_channels)
    return {"bg": w, "h": w, "x": w, "y": w, "z": w}
