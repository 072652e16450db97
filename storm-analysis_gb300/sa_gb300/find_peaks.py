"""
The find / fit loop of 3D-DAOSTORM, sCMOS and Spliner analysis, over this
package's GPU finder (fitting.PeakFinderGaussian / PeakFinderArbitraryPSF /
BatchPeakFinder), culling (ia_utilities_c) and fitter (dao_fit_c,
cubic_fit_c, engine.BatchFitter).

Design.  A frame's analysis is a sequence of finder passes; each pass that
found new peaks runs one *fit pass* over the frame's fitted peaks.  The fit
pass is written once (`fit_pass`) for a set of frames and a mask of the
frames it applies to, over a small "frame set" interface:

    FitterFrames   one MultiFitter per frame (the reference's one-frame
                   objects: dao_fit_c / cubic_fit_c, or anything with the
                   same methods);
    BatchFrames    one engine.BatchFitter holding every frame on the GPU.

`FindFitLoop` drives host-side finders and a FitterFrames set; with one
frame it is the reference's per-frame analysis (initFindAndFit(...)
.analyzeImage / analyzeFrame, the entry points std_analysis calls,
sa_utilities/std_analysis.py:84-105).  `BatchFindFit` drives the batched
finder and a BatchFrames set: frames, backgrounds, new peaks, fit images
and peak records stay on the GPU across passes, and only the per-frame peak
lists that the culling reads travel to the host.

What a fit pass does (the reference's PeakFitter.fitPeaks,
sa_library/fitting.py:701-782, whose order decides the results): peaks near
a new peak go back to RUNNING; the new peaks are added; the frame is fitted
and its ERROR peaks dropped; dimmer neighbours and low-significance peaks are
marked ERROR and dropped; a frame that still has RUNNING peaks is fitted
again.
"""
import numpy

from . import dao_fit_c, engine
from . import ia_utilities_c as iaUtilsC
from .fitting import BatchPeakFinder, PeakFinderGaussian, _Params, padArray

RUNNING, CONVERGED, ERROR = 0, 1, 2

# Radius of "near a new peak", in units of the PSF sigma (fitting.py:839).
UNCONVERGED_DIST = 5.0


class GpuCulling(object):
    """The three culling steps of a fit pass on the GPU (ia_utilities_c).
    Each works on one frame's arrays; statuses are edited in place."""

    @staticmethod
    def wake(status, x, y, new_x, new_y, radius):
        return iaUtilsC.runningIfHasNeighbors(status, x, y, numpy.ascontiguousarray(new_x),
                                              numpy.ascontiguousarray(new_y), radius)

    @staticmethod
    def dimmer(x, y, height, status, sigma, radius):
        return iaUtilsC.markDimmerPeaks(x, y, height, status, sigma, radius)

    @staticmethod
    def faint(x, y, significance, status, threshold, radius):
        return iaUtilsC.markLowSignificancePeaks(x, y, significance, status, threshold, radius)


# ---------------------------------------------------------------------------
# frame sets
# ---------------------------------------------------------------------------

class FitterFrames(object):
    """A frame set of MultiFitter objects, one per frame."""

    def __init__(self, fitters, max_iterations=2000):
        self.fitters = list(fitters)
        self.max_iterations = max_iterations

    def __len__(self):
        return len(self.fitters)

    def nfit(self):
        return numpy.array([f.getNFit() for f in self.fitters])

    def column(self, k, name):
        return self.fitters[k].getPeakProperty(name)

    def set_status(self, statuses, frames):
        for k in frames:
            self.fitters[k].setPeakStatus(statuses[k])

    def add(self, new_peaks, peaks_type, frames):
        for k in frames:
            self.fitters[k].newPeaks(new_peaks[k], peaks_type)

    def fit(self, frames):
        for k in frames:
            self.fitters[k].doFit(self.max_iterations)

    def drop(self, status, frames):
        for k in frames:
            if status == ERROR:
                self.fitters[k].removeErrorPeaks()
            else:
                self.fitters[k].removeRunningPeaks()

    def running(self, frames):
        return [k for k in frames if self.fitters[k].getUnconverged() > 0]

    def count_culled(self, k, n_dimmer, n_faint):
        f = self.fitters[k]
        if hasattr(f, "incProximityCounter"):
            f.incProximityCounter(n_dimmer)
            f.incSignificanceCounter(n_faint)


class BatchFrames(object):
    """A frame set that is one engine.BatchFitter: per-frame columns are
    slices of the batch's property arrays (read once per pass and name)."""

    def __init__(self, fitter, max_iterations=2000):
        self.fitter = fitter
        self.max_iterations = max_iterations
        self._cache = {}

    def __len__(self):
        return self.fitter.n_frames

    def _invalidate(self):
        self._cache = {}

    def nfit(self):
        if "_n" not in self._cache:
            self._cache["_n"] = self.fitter.counts()
        return self._cache["_n"]

    def _edges(self):
        return numpy.concatenate([[0], numpy.cumsum(self.nfit())])

    def _all(self, name):
        if name not in self._cache:
            if name == "significance":
                v = self.fitter.prop("fg_sum") / numpy.sqrt(self.fitter.prop("bg_sum"))
            else:
                v = self.fitter.prop(name)
            self._cache[name] = v
        return self._cache[name]

    def column(self, k, name):
        e = self._edges()
        return numpy.ascontiguousarray(self._all(name)[e[k]:e[k + 1]])

    def set_status(self, statuses, frames):
        full = self._all("status").copy()
        e = self._edges()
        for k in frames:
            full[e[k]:e[k + 1]] = statuses[k]
        self.fitter.set_status(full)
        self._invalidate()

    def add(self, new_peaks, peaks_type, frames, device_rows=None):
        counts = numpy.zeros(len(self), dtype=numpy.int32)
        for k in frames:
            counts[k] = new_peaks[k]["x"].size
        self.fitter.reserve(int((self.nfit() + counts).max()) + 1)
        if device_rows is not None:
            # every frame's finder rows are used: the device hand-off
            self.fitter.load_peaks_device(device_rows, counts, peaks_type)
        else:
            rows = [numpy.stack([new_peaks[k][c] for c in ("x", "y", "z", "sigma")], axis=1)
                    for k in range(len(self)) if counts[k] > 0]
            rows = numpy.ascontiguousarray(numpy.concatenate(rows) if rows else numpy.zeros((0, 4)))
            self.fitter.clib.saNewPeaksBatch(self.fitter.h, rows, counts, len(self), peaks_type.encode())
        self._invalidate()

    def fit(self, frames):
        mask = numpy.zeros(len(self), dtype=bool)
        mask[list(frames)] = True
        self.fitter.fit_frames(mask, self.max_iterations)
        self._invalidate()

    def drop(self, status, frames):
        # ERROR / RUNNING peaks only exist in the frames being worked on
        self.fitter.remove(status)
        self._invalidate()

    def running(self, frames):
        st = self._all("status")
        e = self._edges()
        return [k for k in frames if (st[e[k]:e[k + 1]] == RUNNING).any()]

    def count_culled(self, k, n_dimmer, n_faint):
        pass


# ---------------------------------------------------------------------------
# one fit pass over a set of frames
# ---------------------------------------------------------------------------

def fit_pass(fs, frames, new_peaks, peaks_type, sigma, threshold, neighborhood, culling=GpuCulling,
             fitting=True, add_kw=None):
    """One pass of PeakFitter.fitPeaks (sa_library/fitting.py:701-782) for
    the frames listed in `frames`, each of which has new peaks
    (new_peaks[k], a dict of x, y, ...).  fs is a frame set."""
    frames = [int(k) for k in frames]
    if not frames:
        return
    nfit = fs.nfit()
    # 1. a fitted peak near a new one must be refitted
    woken = [k for k in frames if nfit[k] > 0]
    if woken:
        st = {}
        for k in woken:
            s = numpy.ascontiguousarray(fs.column(k, "status"), dtype=numpy.int32)
            st[k] = culling.wake(s, fs.column(k, "x"), fs.column(k, "y"), new_peaks[k]["x"], new_peaks[k]["y"],
                                 neighborhood)
        fs.set_status(st, woken)
    # 2. add and fit
    fs.add(new_peaks, peaks_type, frames, **(add_kw or {}))
    if fitting:
        fs.fit(frames)
        fs.drop(ERROR, frames)
    # 3. culling: dimmer neighbours, then low significance
    culled, st = [], {}
    for k in frames:
        s = numpy.ascontiguousarray(fs.column(k, "status"), dtype=numpy.int32)
        x, y = fs.column(k, "x"), fs.column(k, "y")
        n_dim = culling.dimmer(x, y, fs.column(k, "height"), s, sigma, neighborhood)
        n_sig = culling.faint(x, y, fs.column(k, "significance"), s, threshold, neighborhood)
        if n_dim + n_sig > 0:
            st[k] = s
            culled.append(k)
            fs.count_culled(k, n_dim, n_sig)
    if culled:
        fs.set_status(st, culled)
        fs.drop(ERROR, culled)
    # 4. refit the frames whose culling left peaks RUNNING
    if fitting:
        again = fs.running(frames)
        if again:
            fs.fit(again)
            fs.drop(ERROR, again)


# ---------------------------------------------------------------------------
# host-driven loop (the reference's per-frame analysis)
# ---------------------------------------------------------------------------

class FindFitLoop(object):
    """Find / fit analysis of frames one at a time with a host-side finder
    and a MultiFitter (PeakFinderFitter.analyzeImage, fitting.py:867-935).

    finder      PeakFinderGaussian / PeakFinderArbitraryPSF (or an object
                with their methods)
    mfitter     the frame's MultiFitter
    properties  the peak properties analyzeImage returns
    neighborhood  radius (pixels) of the culling's neighbour queries
    """

    def __init__(self, finder, mfitter, properties, neighborhood, sigma, threshold, no_fitting=False,
                 culling=GpuCulling):
        assert "x" in properties and "y" in properties, "'x' and 'y' are required properties."
        self.peak_finder = finder
        self.mfitter = mfitter
        self.properties = list(properties)
        self.neighborhood = neighborhood
        self.sigma = sigma
        self.threshold = threshold
        self.no_fitting = bool(no_fitting)
        self.culling = culling
        self.frames = FitterFrames([mfitter])

    def analyzeImage(self, movie_reader):
        """movie_reader.getFrame() (photo-electrons) and getBackground()."""
        return self.analyzeFrame(movie_reader.getFrame(), movie_reader.getBackground())

    def analyzeFrame(self, frame, bg_estimate=None):
        margin = self.peak_finder.margin
        image = padArray(frame, margin)
        if bg_estimate is not None:
            bg_estimate = padArray(bg_estimate, margin)
        if not self.mfitter.isInitialized():
            self.mfitter.initializeC(image)
        self.peak_finder.newImage(image)
        self.mfitter.newImage(image)
        fit_image = numpy.zeros(image.shape)
        for _ in range(self.peak_finder.iterations):
            background = self.peak_finder.estimateBackground(fit_image, bg_estimate)
            new_peaks, peaks_type, done = self.peak_finder.findPeaks(fit_image)
            self.mfitter.newBackground(background)
            if new_peaks["x"].size > 0:
                fit_pass(self.frames, [0], [new_peaks], peaks_type, self.sigma, self.threshold,
                         self.neighborhood, culling=self.culling, fitting=not self.no_fitting)
            fit_image = self.mfitter.getFitImage()
            if done:
                break
        if not self.no_fitting:
            self.mfitter.removeRunningPeaks()
        return self.getPeakProperties()

    def getPeakProperties(self):
        out = {}
        margin = float(self.peak_finder.margin)
        for name in self.properties:
            v = self.mfitter.getPeakProperty(name)
            if name in ("x", "y"):
                v = v - margin
            elif name == "z":
                v = self.mfitter.rescaleZ(v)
            out[name] = v
        return out

    def cleanUp(self, verbose=False):
        self.peak_finder.cleanUp()
        self.mfitter.cleanup(verbose=verbose)


def _camera(finder, parameters):
    """sCMOS calibration of the analysis, padded like the frames: (rqe,
    variance / gain^2) or (None, None) (daostorm_3d/find_peaks.py:31-40)."""
    from .analysis_io import loadCMOSCalibration
    p = _Params(parameters)
    if not p.hasAttr("camera_calibration"):
        return None, None
    offset, variance, gain, rqe = loadCMOSCalibration(p.getAttr("camera_calibration"))
    variance = finder.setVariance(variance / (gain * gain))
    return finder.padArray(rqe), variance


_GAUSSIAN_FITTERS = {"2dfixed": dao_fit_c.MultiFitter2DFixed, "2d": dao_fit_c.MultiFitter2D,
                     "3d": dao_fit_c.MultiFitter3D, "Z": dao_fit_c.MultiFitterZ}

_GAUSSIAN_PROPS = {"2dfixed": ["xsigma"], "2d": ["xsigma"], "3d": ["xsigma", "ysigma"],
                   "Z": ["xsigma", "ysigma", "z"]}


def _check_mle(p):
    if p.getAttr("fit_error_model", "MLE") != "MLE":
        raise dao_fit_c.MultiFitterException("only the MLE error model is implemented by this engine")


def _sigma_range(p):
    if p.hasAttr("sigma_range"):
        return p.getAttr("sigma_range")
    s = p.getAttr("sigma")
    return [0.5 * s, 5.0 * s]


def initFindAndFit(parameters, precision=32):
    """3D-DAOSTORM / sCMOS analysis of one frame at a time
    (daostorm_3d/find_peaks.py:16-135): the Gaussian finder and the MLE
    Gaussian fitter of the parameters' model ('2dfixed', '2d', '3d', 'Z';
    'Z' reads wx_params / wy_params / min_z / max_z)."""
    p = _Params(parameters)
    _check_mle(p)
    model = p.getAttr("model")
    if model not in _GAUSSIAN_FITTERS:
        raise dao_fit_c.MultiFitterException("unknown model '%s'" % model)
    finder = PeakFinderGaussian(parameters)
    rqe, variance = _camera(finder, parameters)
    kw = dict(roi_size=finder.getROISize(), rqe=rqe, scmos_cal=variance, precision=precision)
    if model in ("2d", "3d"):
        kw["sigma_range"] = _sigma_range(p)
    if model == "Z":
        kw.update(wx_params=p.getAttr("wx_params"), wy_params=p.getAttr("wy_params"), min_z=p.getAttr("min_z"),
                  max_z=p.getAttr("max_z"))
    mfitter = _GAUSSIAN_FITTERS[model](**kw)
    props = ["background", "error", "height", "iterations", "significance", "sum", "x", "y"] + _GAUSSIAN_PROPS[model]
    sigma = p.getAttr("sigma")
    return FindFitLoop(finder, mfitter, props, sigma * UNCONVERGED_DIST, sigma, p.getAttr("threshold"),
                       no_fitting=p.getAttr("no_fitting", 0))


def initFindAndFitSpline(parameters, spline_fn=None, precision=32):
    """Spliner's analysis (spliner/find_peaks_std.py:52-135): the
    arbitrary-PSF finder with the spline as its PSF object and the cubic
    spline fitter (MLE); z comes back in microns.  The culling's neighbour
    radius is half the spline's size plus one pixel (fitting.py:826-834).
    spline_fn defaults to the parameters' "spline" file."""
    from . import cubic_fit_c
    from .fitting import PeakFinderArbitraryPSF
    p = _Params(parameters)
    _check_mle(p)
    if spline_fn is None:
        spline_fn = cubic_fit_c.SplinePSF(spline_data=p.getAttr("spline"))
    finder = PeakFinderArbitraryPSF(parameters=parameters, psf_object=spline_fn)
    rqe, variance = _camera(finder, parameters)
    cls = cubic_fit_c.CSpline3DFit if spline_fn.getType() == "3D" else cubic_fit_c.CSpline2DFit
    mfitter = cls(spline_fn=spline_fn, rqe=rqe, scmos_cal=variance, precision=precision)
    props = ["background", "error", "height", "iterations", "significance", "sum", "x", "y", "z"]
    return FindFitLoop(finder, mfitter, props, int(0.5 * mfitter.getSize()) + 1, p.getAttr("sigma"),
                       p.getAttr("threshold"), no_fitting=p.getAttr("no_fitting", 0))


# ---------------------------------------------------------------------------
# batched loop: n frames at once, state on the GPU
# ---------------------------------------------------------------------------

class BatchFindFit(object):
    """FindFitLoop.analyzeFrame for n_frames frames of one shape at once
    (Gaussian models, MLE).  All frames advance pass by pass together: a
    frame whose pass found no new peaks is not refitted (the per-frame loop
    skips the fit pass there), and a frame that is done keeps taking finder
    passes, which change nothing, until every frame is done or after
    `iterations` passes."""

    def __init__(self, parameters, shape, n_frames, precision=32, max_iterations=2000):
        import torch
        self.torch = torch
        p = _Params(parameters)
        self.model = p.getAttr("model")
        self.n_frames = int(n_frames)
        # the finder's ROI decides the margin (fitting.py:376-386)
        roi = p.getAttr("roi_size", -1)
        if roi == -1:
            roi = int(8.0 * p.getAttr("sigma"))
            if self.model != "2dfixed":
                roi = int(1.5 * roi)
        self.margin = int(roi / 2 + 2)
        self.shape = tuple(shape)
        self.pshape = (self.shape[0] + 2 * self.margin, self.shape[1] + 2 * self.margin)
        self.finder = BatchPeakFinder(parameters, self.pshape, self.n_frames)
        kw = dict(roi_size=roi, precision=precision)
        if self.model in ("2d", "3d"):
            kw["sigma_range"] = _sigma_range(p)
        if self.model == "Z":
            kw.update(wx_params=p.getAttr("wx_params"), wy_params=p.getAttr("wy_params"),
                      min_z=p.getAttr("min_z"), max_z=p.getAttr("max_z"))
        self.fitter = engine.BatchFitter(self.model, self.pshape, self.n_frames, **kw)
        self.frames = BatchFrames(self.fitter, max_iterations)
        self.sigma = p.getAttr("sigma")
        self.neighborhood = self.sigma * UNCONVERGED_DIST
        self.threshold = p.getAttr("threshold")
        self.d_fit = torch.zeros(self.n_frames * self.pshape[0] * self.pshape[1], dtype=torch.float64,
                                 device="cuda")
        self.passes = 0

    def analyze(self, frames):
        """frames: (n_frames, ny, nx) photo-electrons.  Returns one dict of
        peak properties per frame (x, y without the margin)."""
        f, fit = self.finder, self.fitter
        padded = numpy.ascontiguousarray(numpy.stack([padArray(im, self.margin) for im in frames]))
        f.newImages(padded)
        # a new frame set: every frame starts empty (mFitNewImage, multi_fit.c:1407)
        fit.reset()
        fit.ensure_frames(1)
        fit.load_images(padded)
        self.d_fit.zero_()
        self.torch.cuda.synchronize()
        done = numpy.zeros(self.n_frames, dtype=bool)
        for it in range(f.iterations):
            self.passes = it + 1
            fit_images = None if it == 0 else self.d_fit
            f.estimateBackground(fit_images)
            counting_down = f.cur_threshold > f.threshold
            counts, _ = f.findPeaks(fit_images)
            fit.load_backgrounds(self.fitter.clib.saFinderBackgroundDevice(f.fh), on_device=True, dtype_bits=64)
            active = numpy.nonzero((counts > 0) & ~done)[0]
            if active.size:
                new = f.peaks()
                # rows of frames that are done stay on the host path (they are skipped)
                every = active.size == int((counts > 0).sum())
                add_kw = {"device_rows": self.fitter.clib.saFinderPeaksDevice(f.fh)} if every else None
                fit_pass(self.frames, active, new, "finder", self.sigma, self.threshold, self.neighborhood,
                         add_kw=add_kw)
            fit.fit_images_device(self.d_fit.data_ptr())
            if not counting_down:
                done |= counts == 0
            if done.all():
                break
        fit.remove(RUNNING)
        self.frames._invalidate()
        props = ["background", "error", "height", "iterations", "significance", "sum", "x", "y", "xsigma",
                 "ysigma", "status"]
        out = []
        for k in range(self.n_frames):
            d = {name: self.frames.column(k, name) for name in props}
            d["x"] = d["x"] - float(self.margin)
            d["y"] = d["y"] - float(self.margin)
            out.append(d)
        return out

    def cleanUp(self):
        self.finder.cleanUp()
        self.fitter.close()
