"""
MultiFitter classes backed by the GPU engine (libsa_cuda.so).

Same class names, constructor arguments, methods and exceptions as the
reference's sa_library/dao_fit_c.py:257-829, so the reference's callers
(sa_library/fitting.py PeakFitter, daostorm_3d/find_peaks.py) can use them
unchanged.  Extra keyword arguments:

  precision    32 (default: FP32 model/Jacobian with FP64 solve and
               decisions) or 64 (FP64 throughout)
  device_loop  True (default): doFit runs its sweep loop on the device;
               False: the reference's host loop of iterate()/getUnconverged()
               (dao_fit_c.py:332-356), one synchronised sweep per call.
"""
import ctypes

import numpy

from . import loadclib

STATUS_RUNNING, STATUS_CONVERGED, STATUS_ERROR = 0, 1, 2


class MultiFitterException(Exception):
    pass


def formatPeaksArbitraryPSF(peaks, peaks_type):
    """(N,3) x, y, z or (N,5) x, y, z, background, height (dao_fit_c.py:80-111)."""
    if peaks_type in ("testing", "finder"):
        cols = ["x", "y", "z"]
    elif peaks_type in ("text", "hdf5"):
        cols = ["x", "y", "z", "background", "height"]
    else:
        raise MultiFitterException("Unknown peaks type '" + peaks_type + "'")
    return numpy.ascontiguousarray(numpy.stack([numpy.asarray(peaks[c], dtype=numpy.float64)
                                                for c in cols], axis=1), dtype=numpy.float64)


def formatPeaksGaussianPSF(peaks, peaks_type):
    """(N,4) x, y, z, sigma or (N,7) x, y, z, background, height, xsigma, ysigma
    (dao_fit_c.py:114-144)."""
    if peaks_type in ("testing", "finder"):
        cols = ["x", "y", "z", "sigma"]
    elif peaks_type in ("text", "hdf5"):
        cols = ["x", "y", "z", "background", "height", "xsigma", "ysigma"]
    else:
        raise MultiFitterException("Unknown peaks type '" + peaks_type + "'")
    return numpy.ascontiguousarray(numpy.stack([numpy.asarray(peaks[c], dtype=numpy.float64)
                                                for c in cols], axis=1), dtype=numpy.float64)


def printFittingInfo(mfit, spacing="  "):
    c = mfit.contents
    print(spacing, c.n_dposv, "fits reset due to Cholesky failure.")
    print(spacing, c.n_margin, "fits reset due to image margin.")
    print(spacing, c.n_neg_fi, "fits reset due to negative value in fit function.")
    print(spacing, c.n_neg_height, "fits reset due to negative height.")
    print(spacing, c.n_non_decr, "fits reset due to non-decreasing error (LM).")
    print(spacing, c.n_non_converged, "fits did not converge.")
    print(spacing, c.n_lost, "fits were lost.")


class MultiFitter(object):
    """Base class; call order as the reference (newImage, newBackground,
    newPeaks, doFit, getPeakProperty, cleanup)."""

    def __init__(self, rqe=None, scmos_cal=None, verbose=False, min_z=None, max_z=None,
                 precision=32, device_loop=True, dilation=None, **kwds):
        super(MultiFitter, self).__init__(**kwds)
        self.dilation = dilation
        self.clib = loadclib.load()
        self.default_tol = 1.0e-6
        self.device_loop = device_loop
        self.im_shape = None
        self.iterations = 0
        self.max_z = max_z
        self.mfit = None
        self.min_z = min_z
        self.n_proximity = 0
        self.n_significance = 0
        self.precision = precision
        self.peak_properties = {"background": "float", "bg_sum": "float", "error": "float",
                                "fg_sum": "float", "height": "float", "iterations": "int",
                                "jacobian": "float", "significance": "compound", "sum": "float",
                                "status": "int", "x": "float", "xsigma": "float", "y": "float",
                                "ysigma": "float", "z": "float"}
        self.rqe = rqe
        self.scmos_cal = scmos_cal
        self.verbose = verbose

    def _check(self, what):
        err = loadclib.last_error()
        if err:
            raise MultiFitterException(what + ": " + err)

    def _clear_error(self):
        self.clib.saClearLastError()

    def cleanup(self, spacing="  ", verbose=True):
        if self.mfit is not None and verbose:
            printFittingInfo(self.mfit, spacing=spacing)
            print(spacing, self.n_proximity, "peaks lost to proximity filter.")
            print(spacing, self.n_significance, "peaks lost to low significance.")
            print(spacing, self.iterations, "fitting iterations.")

    def doFit(self, max_iterations=2000):
        """dao_fit_c.py:332-356: one sweep, then sweeps while peaks are RUNNING."""
        if self.device_loop:
            r = self.clib.saDoFit(self.mfit, max_iterations)
            if r < 0:
                raise MultiFitterException("doFit failed: " + loadclib.last_error())
        else:
            i = 0
            self.iterate()
            while self.getUnconverged() and (i < max_iterations):
                self.iterate()
                i += 1
        self.getIterations()

    def getFitImage(self):
        out = numpy.ascontiguousarray(numpy.zeros(self.im_shape, dtype=numpy.float64))
        self.clib.mFitGetFitImage(self.mfit, out)
        return out

    def getGoodPeaks(self):
        """Convenience: drop ERROR and RUNNING peaks (removeErrorPeaks then
        removeRunningPeaks) and return the number left."""
        self.removeErrorPeaks()
        self.removeRunningPeaks()
        return self.getNFit()

    def getIterations(self):
        self.iterations += self.mfit.contents.n_iterations
        self.mfit.contents.n_iterations = 0
        return self.iterations

    def getNError(self):
        return self.clib.mFitGetNError(self.mfit)

    def getNFit(self):
        return self.mfit.contents.nfit

    def getNFitMax(self):
        return self.mfit.contents.max_nfit

    def getPeakProperty(self, p_name):
        if p_name not in self.peak_properties:
            raise MultiFitterException("No such property '" + p_name + "'")
        kind = self.peak_properties[p_name]
        if kind == "compound":
            if self.getNFit() == 0:
                return numpy.zeros(0, dtype=numpy.float64)
            bg_sum = self.getPeakProperty("bg_sum")
            fg_sum = self.getPeakProperty("fg_sum")
            return fg_sum / numpy.sqrt(bg_sum)
        if kind == "float":
            if p_name == "jacobian":
                values = numpy.zeros((self.getNFit(), self.mfit.contents.jac_size), dtype=numpy.float64)
            else:
                values = numpy.zeros(self.getNFit(), dtype=numpy.float64)
            self.clib.mFitGetPeakPropertyDouble(self.mfit, values, ctypes.c_char_p(p_name.encode()))
            return values
        values = numpy.zeros(self.getNFit(), dtype=numpy.int32)
        self.clib.mFitGetPeakPropertyInt(self.mfit, values, ctypes.c_char_p(p_name.encode()))
        return values

    def getResidual(self):
        out = numpy.ascontiguousarray(numpy.zeros(self.im_shape, dtype=numpy.float64))
        self.clib.mFitGetResidual(self.mfit, out)
        return out

    def getUnconverged(self):
        return self.clib.mFitGetUnconverged(self.mfit)

    def incProximityCounter(self, n_inc):
        self.n_proximity += n_inc

    def incSignificanceCounter(self, n_inc):
        self.n_significance += n_inc

    def initializeC(self, image):
        """dao_fit_c.py:461-488: defaults and shape checks of rqe / sCMOS arrays."""
        if self.scmos_cal is None:
            self.scmos_cal = numpy.ascontiguousarray(numpy.zeros(image.shape), dtype=numpy.float64)
        else:
            self.scmos_cal = numpy.ascontiguousarray(self.scmos_cal, dtype=numpy.float64)
        if self.rqe is None:
            self.rqe = numpy.ascontiguousarray(numpy.ones(image.shape), dtype=numpy.float64)
        else:
            self.rqe = numpy.ascontiguousarray(self.rqe, dtype=numpy.float64)
        if (image.shape[0] != self.scmos_cal.shape[0]) or (image.shape[1] != self.scmos_cal.shape[1]):
            raise MultiFitterException("Image shape and sCMOS calibration shape do not match.")
        if (image.shape[0] != self.rqe.shape[0]) or (image.shape[1] != self.rqe.shape[1]):
            raise MultiFitterException("Image shape and RQE shape do not match.")
        self.im_shape = self.scmos_cal.shape

    def _after_create(self, what):
        if not self.mfit:
            raise MultiFitterException(what + " failed: " + loadclib.last_error())
        if self.clib.saSetPrecision(self.mfit, int(self.precision)) != 0:
            raise MultiFitterException(loadclib.last_error())
        if self.dilation is not None and self.clib.saSetDilation(self.mfit, int(self.dilation)) != 0:
            raise MultiFitterException(loadclib.last_error())

    def isInitialized(self):
        return self.mfit is not None

    def iterate(self):
        self.clib.mFitIterateLM(self.mfit)

    def newBackground(self, background):
        if (background.shape[0] != self.im_shape[0]) or (background.shape[1] != self.im_shape[1]):
            raise MultiFitterException("Background image shape and the original image shape are not the same.")
        self.clib.mFitNewBackground(self.mfit, numpy.ascontiguousarray(background, dtype=numpy.float64))

    def newImage(self, image):
        if (image.shape[0] != self.im_shape[0]) or (image.shape[1] != self.im_shape[1]):
            raise MultiFitterException("Current image shape and the original image shape are not the same.")
        self._clear_error()
        self.clib.mFitNewImage(self.mfit, numpy.ascontiguousarray(image, dtype=numpy.float64))
        self._check("newImage")

    def newPeaks(self, peaks, peaks_type):
        raise MultiFitterException("newPeaks() method not defined.")

    def removeErrorPeaks(self):
        self.clib.mFitRemoveErrorPeaks(self.mfit)

    def removeRunningPeaks(self):
        self.clib.mFitRemoveRunningPeaks(self.mfit)

    def rescaleZ(self, z):
        return z

    def setPeakStatus(self, status):
        assert (status.size == self.getNFit())
        self.clib.mFitSetPeakStatus(self.mfit, numpy.ascontiguousarray(status, dtype=numpy.int32))

    def counters(self):
        """Device counter totals (reference order + starting-error failures)."""
        out = numpy.zeros(9, dtype=numpy.int64)
        self.clib.saGetCounters(self.mfit, out)
        return dict(zip(["n_dposv", "n_iterations", "n_lost", "n_margin", "n_neg_fi",
                         "n_neg_height", "n_non_converged", "n_non_decr", "n_start_fail"],
                        out.tolist()))


class MultiFitterArbitraryPSF(MultiFitter):
    def formatPeaks(self, peaks, peaks_type):
        return formatPeaksArbitraryPSF(peaks, peaks_type)


class MultiFitterGaussian(MultiFitter):
    """Gaussian fitters (3D-DAOSTORM and sCMOS), dao_fit_c.py:560-603."""

    def __init__(self, roi_size=10, wx_params=None, wy_params=None, **kwds):
        super(MultiFitterGaussian, self).__init__(**kwds)
        self.roi_size = roi_size
        self.wx_params = wx_params
        self.wy_params = wy_params

    def cleanup(self, verbose=True):
        super(MultiFitterGaussian, self).cleanup(verbose=verbose)
        if self.mfit is not None:
            self.clib.daoCleanup(self.mfit)
            self.mfit = None

    def formatPeaks(self, peaks, peaks_type):
        return formatPeaksGaussianPSF(peaks, peaks_type)

    def initializeC(self, image):
        super(MultiFitterGaussian, self).initializeC(image)
        self.mfit = self.clib.daoInitialize(self.rqe, self.scmos_cal, self.default_tol,
                                            self.scmos_cal.shape[1], self.scmos_cal.shape[0],
                                            self.roi_size)
        self._after_create("daoInitialize")

    def newPeaks(self, peaks, peaks_type):
        c_peaks = self.formatPeaks(peaks, peaks_type)
        self._clear_error()
        self.clib.daoNewPeaks(self.mfit, c_peaks, ctypes.c_char_p(peaks_type.encode()), c_peaks.shape[0])
        self._check("newPeaks")


def _widths(sigma_range):
    width_max = 1.0 / (2.0 * sigma_range[0] * sigma_range[0])
    width_min = 1.0 / (2.0 * sigma_range[1] * sigma_range[1])
    return width_min, width_max


class MultiFitter2DFixed(MultiFitterGaussian):
    def initializeC(self, image):
        super(MultiFitter2DFixed, self).initializeC(image)
        self.clib.daoInitialize2DFixed(self.mfit)


class MultiFitter2D(MultiFitterGaussian):
    def __init__(self, sigma_range=None, **kwds):
        super(MultiFitter2D, self).__init__(**kwds)
        self.sigma_range = sigma_range

    def initializeC(self, image):
        super(MultiFitter2D, self).initializeC(image)
        self.clib.daoInitialize2D(self.mfit, *_widths(self.sigma_range))


class MultiFitter3D(MultiFitterGaussian):
    def __init__(self, sigma_range=None, **kwds):
        super(MultiFitter3D, self).__init__(**kwds)
        self.sigma_range = sigma_range

    def initializeC(self, image):
        super(MultiFitter3D, self).initializeC(image)
        self.clib.daoInitialize3D(self.mfit, *_widths(self.sigma_range))


class MultiFitterZ(MultiFitterGaussian):
    def initializeC(self, image):
        super(MultiFitterZ, self).initializeC(image)
        self.clib.daoInitializeZ(self.mfit, numpy.ascontiguousarray(self.wx_params, dtype=numpy.float64),
                                 numpy.ascontiguousarray(self.wy_params, dtype=numpy.float64),
                                 float(self.min_z), float(self.max_z))


class _Unsupported(MultiFitterGaussian):
    """Error models other than MLE are not implemented by this engine."""

    def __init__(self, sigma_range=None, **kwds):
        super(_Unsupported, self).__init__(**kwds)
        self.sigma_range = sigma_range

    def initializeC(self, image):
        raise MultiFitterException(type(self).__name__ + ": only the MLE error model is implemented "
                                   "by the GPU engine")


class MultiFitter2DFixedALS(_Unsupported):
    pass


class MultiFitter2DFixedLS(_Unsupported):
    pass


class MultiFitter2DFixedDWLS(_Unsupported):
    pass


class MultiFitter2DFixedFWLS(_Unsupported):
    pass


class MultiFitter2DALS(_Unsupported):
    pass


class MultiFitter2DLS(_Unsupported):
    pass


class MultiFitter2DDWLS(_Unsupported):
    pass


class MultiFitter2DFWLS(_Unsupported):
    pass


class MultiFitter2DFixedNC(MultiFitter2DFixed):
    """dao_fit_c.py:663-681: RQE forced to 1."""

    def __init__(self, **kwds):
        super(MultiFitter2DFixedNC, self).__init__(**kwds)
        self.rqe = None


class MultiFitter2DFixedDWLSNC(MultiFitter2DFixedDWLS):
    def __init__(self, **kwds):
        super(MultiFitter2DFixedDWLSNC, self).__init__(**kwds)
        self.rqe = None
