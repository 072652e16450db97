"""
The find / fit loop of 3D-DAOSTORM and sCMOS analysis on the GPU: the
reference's PeakFitter, PeakFinderFitter (sa_library/fitting.py:674-935)
and initFindAndFit (daostorm_3d/find_peaks.py:16-135) over this package's
GPU finder (fitting.PeakFinderGaussian), culling (ia_utilities_c) and
fitter (dao_fit_c).  Same control flow as the reference: per frame, up to
`iterations` passes of background estimate -> new peaks -> fit -> culling,
then the unconverged peaks are removed.
"""
import numpy

from . import dao_fit_c
from . import ia_utilities_c as iaUtilsC
from .fitting import PeakFinderGaussian, _Params, padArray


class PeakFitter(object):
    """fitting.py:674-806."""

    def __init__(self, mfitter=None, parameters=None, **kwds):
        super(PeakFitter, self).__init__(**kwds)
        parameters = _Params(parameters)
        self.no_fitting = parameters.getAttr("no_fitting", 0)
        self.mfitter = mfitter
        self.minimum_significance = parameters.getAttr("threshold")
        self.sigma = parameters.getAttr("sigma")
        self.neighborhood = self.sigma * PeakFinderFitter.unconverged_dist

    def cleanUp(self):
        self.mfitter.cleanup()

    def fitPeaks(self, new_peaks, peaks_type):
        """One fitting pass; returns the current fit image."""
        if new_peaks["x"].size > 0:
            if self.mfitter.getNFit() > 0:
                c_x = self.mfitter.getPeakProperty("x")
                c_y = self.mfitter.getPeakProperty("y")
                status = self.mfitter.getPeakProperty("status")
                new_status = iaUtilsC.runningIfHasNeighbors(status, c_x, c_y,
                                                            numpy.ascontiguousarray(new_peaks["x"]),
                                                            numpy.ascontiguousarray(new_peaks["y"]),
                                                            self.neighborhood)
                self.mfitter.setPeakStatus(new_status)
            self.mfitter.newPeaks(new_peaks, peaks_type)
            if not self.no_fitting:
                self.mfitter.doFit()
                self.mfitter.removeErrorPeaks()
            status = self.mfitter.getPeakProperty("status")
            px = self.mfitter.getPeakProperty("x")
            py = self.mfitter.getPeakProperty("y")
            n_proximity = iaUtilsC.markDimmerPeaks(px, py, self.mfitter.getPeakProperty("height"), status,
                                                   self.sigma, self.neighborhood)
            n_significance = iaUtilsC.markLowSignificancePeaks(px, py,
                                                               self.mfitter.getPeakProperty("significance"),
                                                               status, self.minimum_significance,
                                                               self.neighborhood)
            if (n_proximity + n_significance) > 0:
                self.mfitter.setPeakStatus(status)
                self.mfitter.removeErrorPeaks()
                self.mfitter.incProximityCounter(n_proximity)
                self.mfitter.incSignificanceCounter(n_significance)
            if (self.mfitter.getUnconverged() > 0) and (not self.no_fitting):
                self.mfitter.doFit()
                self.mfitter.removeErrorPeaks()
        return self.mfitter.getFitImage()

    def getPeakProperty(self, pname):
        return self.mfitter.getPeakProperty(pname)

    def newBackground(self, new_background):
        self.mfitter.newBackground(new_background)

    def newImage(self, new_image):
        if not self.mfitter.isInitialized():
            self.mfitter.initializeC(new_image)
        self.mfitter.newImage(new_image)

    def removeRunningPeaks(self):
        if not self.no_fitting:
            self.mfitter.removeRunningPeaks()

    def rescaleZ(self, z):
        return self.mfitter.rescaleZ(z)


class PeakFinderFitter(object):
    """fitting.py:832-935."""
    unconverged_dist = 5.0

    def __init__(self, peak_finder=None, peak_fitter=None, properties=None, **kwds):
        super(PeakFinderFitter, self).__init__(**kwds)
        self.peak_finder = peak_finder
        self.peak_fitter = peak_fitter
        self.properties = properties
        assert ("x" in self.properties), "'x' is a required property."
        assert ("y" in self.properties), "'y' is a required property."

    def analyzeImage(self, movie_reader):
        """As the reference: movie_reader.getFrame() (photo-electrons) and
        movie_reader.getBackground() (an estimate or None)."""
        bg = movie_reader.getBackground()
        return self.analyzeFrame(movie_reader.getFrame(), bg)

    def analyzeFrame(self, frame, bg_estimate=None):
        image = padArray(frame, self.peak_finder.margin)
        fit_peaks_image = numpy.zeros(image.shape)
        if bg_estimate is not None:
            bg_estimate = padArray(bg_estimate, self.peak_finder.margin)
        self.peak_finder.newImage(image)
        self.peak_fitter.newImage(image)
        for i in range(self.peak_finder.iterations):
            background = self.peak_finder.estimateBackground(fit_peaks_image, bg_estimate)
            [new_peaks, peaks_type, done] = self.peak_finder.findPeaks(fit_peaks_image)
            self.peak_fitter.newBackground(background)
            fit_peaks_image = self.peak_fitter.fitPeaks(new_peaks, peaks_type)
            if done:
                break
        self.peak_fitter.removeRunningPeaks()
        return self.getPeakProperties()

    def cleanUp(self):
        self.peak_finder.cleanUp()
        self.peak_fitter.cleanUp()

    def getPeakProperties(self):
        peaks = {}
        for pname in self.properties:
            peaks[pname] = self.peak_fitter.getPeakProperty(pname)
            if pname in ("x", "y"):
                peaks[pname] -= float(self.peak_finder.margin)
            elif pname == "z":
                peaks[pname] = self.peak_fitter.rescaleZ(peaks[pname])
        return peaks


def initFindAndFit(parameters, precision=32):
    """Finder + fitter for the MLE Gaussian models ('2dfixed', '2d', '3d';
    'Z' takes wx_params / wy_params / min_z / max_z from the parameters).
    A sCMOS camera_calibration file sets the camera variance and RQE as in
    daostorm_3d/find_peaks.py:31-40."""
    from .analysis_io import loadCMOSCalibration
    p = _Params(parameters)
    fmodel = p.getAttr("model")
    emodel = p.getAttr("fit_error_model", "MLE")
    if emodel != "MLE":
        raise dao_fit_c.MultiFitterException("only the MLE error model is implemented by this engine")
    finder = PeakFinderGaussian(parameters)
    rqe = variance = None
    if p.hasAttr("camera_calibration"):
        [offset, variance, gain, rqe] = loadCMOSCalibration(p.getAttr("camera_calibration"))
        variance = variance / (gain * gain)
        variance = finder.setVariance(variance)
        rqe = finder.padArray(rqe)
    kwds = {"roi_size": finder.getROISize(), "rqe": rqe, "scmos_cal": variance, "precision": precision}
    if fmodel in ("2d", "3d"):
        if p.hasAttr("sigma_range"):
            kwds["sigma_range"] = p.getAttr("sigma_range")
        else:
            sigma = p.getAttr("sigma")
            kwds["sigma_range"] = [0.5 * sigma, 5.0 * sigma]
    if fmodel == "2dfixed":
        mfitter = dao_fit_c.MultiFitter2DFixed(**kwds)
    elif fmodel == "2d":
        mfitter = dao_fit_c.MultiFitter2D(**kwds)
    elif fmodel == "3d":
        mfitter = dao_fit_c.MultiFitter3D(**kwds)
    elif fmodel == "Z":
        mfitter = dao_fit_c.MultiFitterZ(wx_params=p.getAttr("wx_params"), wy_params=p.getAttr("wy_params"),
                                         min_z=p.getAttr("min_z"), max_z=p.getAttr("max_z"), **kwds)
    else:
        raise dao_fit_c.MultiFitterException("unknown model '%s'" % fmodel)
    fitter = PeakFitter(mfitter=mfitter, parameters=parameters)
    properties = ["background", "error", "height", "iterations", "significance", "sum", "x", "y"]
    if fmodel in ("2dfixed", "2d"):
        properties.append("xsigma")
    elif fmodel == "3d":
        properties += ["xsigma", "ysigma"]
    elif fmodel == "Z":
        properties += ["xsigma", "ysigma", "z"]
    return PeakFinderFitter(peak_finder=finder, peak_fitter=fitter, properties=properties)
