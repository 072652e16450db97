"""
The find / fit loop of 3D-DAOSTORM and sCMOS analysis on the GPU: the
reference's PeakFitter, PeakFinderFitter (sa_library/fitting.py:674-935)
and initFindAndFit (daostorm_3d/find_peaks.py:16-135) over this package's
GPU finder (fitting.PeakFinderGaussian), culling (ia_utilities_c) and
fitter (dao_fit_c).  Same control flow as the reference: per frame, up to
`iterations` passes of background estimate -> new peaks -> fit -> culling,
then the unconverged peaks are removed.

BatchFindFit runs the same loop for n frames at once: frames, backgrounds,
new peaks, fit images and the fits stay on the GPU across passes, the fits
of all frames run in one batched sweep loop, and only the per-frame peak
lists that the culling reads travel to the host.
"""
import numpy

from . import dao_fit_c, engine
from . import ia_utilities_c as iaUtilsC
from .fitting import BatchPeakFinder, PeakFinderGaussian, _Params, padArray

RUNNING, CONVERGED, ERROR = 0, 1, 2


class PeakFitter(object):
    """fitting.py:674-823."""

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


class PeakFitterArbitraryPSF(PeakFitter):
    """fitting.py:826-834: the neighbourhood is half the PSF size + 1."""

    def __init__(self, **kwds):
        super(PeakFitterArbitraryPSF, self).__init__(**kwds)
        self.neighborhood = int(0.5 * self.mfitter.getSize()) + 1


class PeakFinderFitter(object):
    """fitting.py:837-935."""
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


def initFindAndFitSpline(parameters, spline_fn=None, precision=32):
    """Spliner's finder + fitter (spliner/find_peaks_std.py:52-135): the
    arbitrary-PSF finder with the spline as its PSF object, the cubic spline
    fitter (MLE), properties with z in microns.  spline_fn defaults to the
    parameters' "spline" file."""
    from . import cubic_fit_c
    from .analysis_io import loadCMOSCalibration
    from .fitting import PeakFinderArbitraryPSF
    p = _Params(parameters)
    if p.getAttr("fit_error_model", "MLE") != "MLE":
        raise dao_fit_c.MultiFitterException("only the MLE error model is implemented by this engine")
    if spline_fn is None:
        spline_fn = cubic_fit_c.SplinePSF(spline_data=p.getAttr("spline"))
    finder = PeakFinderArbitraryPSF(parameters=parameters, psf_object=spline_fn)
    rqe = variance = None
    if p.hasAttr("camera_calibration"):
        [offset, variance, gain, rqe] = loadCMOSCalibration(p.getAttr("camera_calibration"))
        variance = finder.setVariance(variance / (gain * gain))
        rqe = finder.padArray(rqe)
    cls = cubic_fit_c.CSpline3DFit if spline_fn.getType() == "3D" else cubic_fit_c.CSpline2DFit
    mfitter = cls(spline_fn=spline_fn, rqe=rqe, scmos_cal=variance, precision=precision)
    fitter = PeakFitterArbitraryPSF(mfitter=mfitter, parameters=parameters)
    properties = ["background", "error", "height", "iterations", "significance", "sum", "x", "y", "z"]
    return PeakFinderFitter(peak_finder=finder, peak_fitter=fitter, properties=properties)


class BatchFindFit(object):
    """PeakFinderFitter.analyzeImage for n_frames frames of one shape at
    once (Gaussian models, MLE).  Frames that a pass leaves without new
    peaks are not refitted, as the reference's per-frame loop stops there;
    the loop ends when every frame is done or after `iterations` passes."""

    def __init__(self, parameters, shape, n_frames, precision=32, max_iterations=2000):
        import torch
        self.torch = torch
        p = _Params(parameters)
        self.model = p.getAttr("model")
        self.n_frames = int(n_frames)
        # the finder's ROI and margin (fitting.py:376-386)
        roi = p.getAttr("roi_size", -1)
        if roi == -1:
            roi = int(8.0 * p.getAttr("sigma"))
            if self.model != "2dfixed":
                roi = int(1.5 * roi)
        self.margin = int(roi / 2 + 2)
        self.shape = tuple(shape)
        self.pshape = (self.shape[0] + 2 * self.margin, self.shape[1] + 2 * self.margin)
        self.finder = BatchPeakFinder(parameters, self.pshape, self.n_frames)
        sigma = p.getAttr("sigma")
        kw = dict(roi_size=roi, precision=precision)
        if self.model in ("2d", "3d"):
            kw["sigma_range"] = p.getAttr("sigma_range") if p.hasAttr("sigma_range") else [0.5 * sigma, 5.0 * sigma]
        if self.model == "Z":
            kw.update(wx_params=p.getAttr("wx_params"), wy_params=p.getAttr("wy_params"),
                      min_z=p.getAttr("min_z"), max_z=p.getAttr("max_z"))
        self.fitter = engine.BatchFitter(self.model, self.pshape, self.n_frames, **kw)
        self.sigma = sigma
        self.neighborhood = sigma * PeakFinderFitter.unconverged_dist
        self.threshold = p.getAttr("threshold")
        self.max_iterations = max_iterations
        self.d_fit = torch.zeros(self.n_frames * self.pshape[0] * self.pshape[1], dtype=torch.float64,
                                 device="cuda")
        self.passes = 0

    def _frames_of(self, a):
        edges = numpy.concatenate([[0], numpy.cumsum(self.fitter.counts())])
        return [numpy.ascontiguousarray(a[edges[f]:edges[f + 1]]) for f in range(self.n_frames)], edges

    def analyze(self, frames):
        """frames: (n_frames, ny, nx) photo-electrons.  Returns one dict of
        peak properties per frame (x, y without the margin)."""
        f = self.finder
        fit = self.fitter
        padded = numpy.ascontiguousarray(numpy.stack([padArray(im, self.margin) for im in frames]))
        f.newImages(padded)
        # a new frame set: drop the previous analysis's peaks (mFitNewImage
        # starts every frame empty, multi_fit.c:1407)
        fit.reset()
        fit.ensure_frames(1)
        fit.load_images(padded)
        self.d_fit.zero_()
        self.torch.cuda.synchronize()
        done = numpy.zeros(self.n_frames, dtype=bool)
        for it in range(f.iterations):
            self.passes = it + 1
            first = it == 0
            f.estimateBackground(None if first else self.d_fit)
            counting_down = f.cur_threshold > f.threshold
            counts, _ = f.findPeaks(None if first else self.d_fit)
            fit.load_backgrounds(self.fitter.clib.saFinderBackgroundDevice(f.fh), on_device=True, dtype_bits=64)
            active = (counts > 0) & ~done
            if active.any():
                self._fit_pass(active, counts)
            fit.fit_images_device(self.d_fit.data_ptr())
            if not counting_down:
                done |= counts == 0
            if done.all():
                break
        fit.remove(RUNNING)
        props = ["background", "error", "height", "iterations", "significance", "sum", "x", "y", "xsigma",
                 "ysigma", "status"]
        vals = {}
        for pname in props:
            if pname == "significance":
                v = fit.prop("fg_sum") / numpy.sqrt(fit.prop("bg_sum"))
            else:
                v = fit.prop(pname)
            vals[pname] = v
        per, _ = zip(*[self._frames_of(vals[p]) for p in props])
        out = []
        for fr in range(self.n_frames):
            d = {p: per[k][fr] for k, p in enumerate(props)}
            d["x"] = d["x"] - float(self.margin)
            d["y"] = d["y"] - float(self.margin)
            out.append(d)
        return out

    def _fit_pass(self, active, counts):
        """PeakFitter.fitPeaks (fitting.py:701-782) for the active frames."""
        fit = self.fitter
        nfit = fit.counts()
        new = self.finder.peaks()
        if (nfit[active] > 0).any():
            status = fit.prop("status")
            xs, edges = self._frames_of(fit.prop("x"))
            ys, _ = self._frames_of(fit.prop("y"))
            for fr in numpy.nonzero(active & (nfit > 0))[0]:
                st = numpy.ascontiguousarray(status[edges[fr]:edges[fr + 1]])
                iaUtilsC.runningIfHasNeighbors(st, xs[fr], ys[fr], numpy.ascontiguousarray(new[fr]["x"]),
                                               numpy.ascontiguousarray(new[fr]["y"]), self.neighborhood)
                status[edges[fr]:edges[fr + 1]] = st
            fit.set_status(status)
        # new peaks of inactive frames are not added (counts 0 there)
        add = numpy.where(active, counts, 0).astype(numpy.int32)
        fit.reserve(int((nfit + add).max()) + 1)
        if (add != counts).any():
            rows = numpy.concatenate([numpy.stack([new[fr]["x"], new[fr]["y"], new[fr]["z"], new[fr]["sigma"]], axis=1)
                                      for fr in range(self.n_frames) if add[fr] > 0] or [numpy.zeros((0, 4))])
            self.fitter.clib.saNewPeaksBatch(fit.h, numpy.ascontiguousarray(rows), add, self.n_frames, b"finder")
        else:
            fit.load_peaks_device(self.fitter.clib.saFinderPeaksDevice(self.finder.fh), add, "finder")
        fit.fit_frames(active, self.max_iterations)
        fit.remove(ERROR)
        status = fit.prop("status")
        xs, edges = self._frames_of(fit.prop("x"))
        ys, _ = self._frames_of(fit.prop("y"))
        hs, _ = self._frames_of(fit.prop("height"))
        sig = fit.prop("fg_sum") / numpy.sqrt(fit.prop("bg_sum"))
        ss, _ = self._frames_of(sig)
        changed = False
        for fr in numpy.nonzero(active)[0]:
            st = numpy.ascontiguousarray(status[edges[fr]:edges[fr + 1]])
            n_p = iaUtilsC.markDimmerPeaks(xs[fr], ys[fr], hs[fr], st, self.sigma, self.neighborhood)
            n_s = iaUtilsC.markLowSignificancePeaks(xs[fr], ys[fr], ss[fr], st, self.threshold, self.neighborhood)
            if n_p + n_s > 0:
                status[edges[fr]:edges[fr + 1]] = st
                changed = True
        if changed:
            fit.set_status(status)
            fit.remove(ERROR)
        status = fit.prop("status")
        sts, _ = self._frames_of(status)
        again = numpy.array([active[fr] and bool((sts[fr] == RUNNING).any()) for fr in range(self.n_frames)])
        if again.any():
            fit.fit_frames(again, self.max_iterations)
            fit.remove(ERROR)

    def cleanUp(self):
        self.finder.cleanUp()
        self.fitter.close()
