"""
The peak-finding half of storm-analysis's find/fit loop on the GPU.

PeakFinderGaussian mirrors the reference's class of the same name
(sa_library/fitting.py:185-501: newImage, estimateBackground, findPeaks,
peakFinder, padArray, setVariance, getROISize, cleanUp) for one frame at a
time with host arrays; every step runs in libsa_cuda.so (saFinder*,
include/sa_finder.h).  BatchPeakFinder does the same for n frames of one
size at once with the frames, backgrounds and found peaks resident on the
GPU, and hands them to a BatchFitter without a host round trip.

gaussianPSF, padArray and peakMask give the finder's host-side set-up
(the filters' PSF, the mirror padding and the area-of-interest mask of
sa_library/fitting.py:38-46, :112-132 and :134-176).
"""
import ctypes

import numpy

from . import loadclib
from .matched_filter_c import MatchedFilter


class FittingException(Exception):
    pass


class _Params(object):
    """The reference's parameters object (getAttr / hasAttr) or a dict."""

    def __init__(self, parameters):
        self.p = parameters

    def hasAttr(self, name):
        if isinstance(self.p, dict):
            return name in self.p and self.p[name] is not None
        return self.p.hasAttr(name)

    def getAttr(self, name, default=None):
        if isinstance(self.p, dict):
            v = self.p.get(name, default)
            return default if v is None else v
        if default is None:
            return self.p.getAttr(name)
        return self.p.getAttr(name, default)


def gaussianPSF(shape, sigma):
    """A unit-sum Gaussian centred at (shape[0]/2, shape[1]/2), drawn as the
    reference's drawGaussians draws it at resolution 1
    (simulator/draw_gaussians.c:24-80): exp(-(dx^2 + dy^2)/(2 sigma^2)) on
    the pixels within int(5 sigma) of the centre's integer part."""
    rows, cols = int(shape[0]), int(shape[1])
    px, py = 0.5 * rows, 0.5 * cols
    aw = max(int(5.0 * sigma), 1)
    sg = 1.0 / (2.0 * sigma * sigma)
    psf = numpy.zeros((rows, cols))
    r0, r1 = max(int(px) - aw, 0), min(int(px) + aw + 1, rows)
    c0, c1 = max(int(py) - aw, 0), min(int(py) + aw + 1, cols)
    dj = numpy.arange(r0, r1, dtype=numpy.float64)[:, None] - px
    dk = numpy.arange(c0, c1, dtype=numpy.float64)[None, :] - py
    psf[r0:r1, c0:c1] = numpy.exp(-1.0 * (dj * dj * sg + dk * dk * sg))
    return psf / numpy.sum(psf)


def padArray(ori_array, pad_size):
    """The frame with pad_size pixels of mirror padding on every side, as
    float64: the border pixel is repeated (numpy's "symmetric" mode), which
    is the padding the reference's finder and fitter see
    (sa_library/fitting.py:112-132).  pad_size must not exceed the frame's
    size; pad_size <= 0 returns the frame unchanged."""
    if pad_size <= 0:
        return ori_array
    return numpy.pad(numpy.asarray(ori_array, dtype=numpy.float64), int(pad_size), mode="symmetric")


_AOI_CIRCLE = ("x_center", "y_center", "aoi_radius")


def peakMask(shape, parameters, margin):
    """The finder's area-of-interest mask on padded frames of this shape: 1
    where peaks may be found, 0 elsewhere (sa_library/fitting.py:134-176).
    Parameters are in unpadded pixels.  Two forms:

    circle  x_center, y_center, aoi_radius (all three once any is given): a
            pixel (column c, row r) is out when (c - xc)^2 + (r - yc)^2 >
            aoi_radius^2; both coordinates run over shape[0] values, so the
            circle form needs square frames;
    box     any of x_start, x_stop (columns) and y_start, y_stop (rows):
            columns before x_start and from x_stop up to, but not including,
            the last column are out (rows likewise)."""
    p = _Params(parameters)
    mask = numpy.ones(shape)
    given = [k for k in _AOI_CIRCLE if p.hasAttr(k)]
    if given:
        missing = [k for k in _AOI_CIRCLE if k not in given]
        if missing:
            raise AssertionError("%s must be specified for a circular AOI." % missing[0])
        r = float(p.getAttr("aoi_radius"))
        n = shape[0]
        dc = numpy.arange(n, dtype=numpy.float64) - (p.getAttr("x_center") + margin)
        dr = numpy.arange(n, dtype=numpy.float64) - (p.getAttr("y_center") + margin)
        mask[(dc[None, :] * dc[None, :] + dr[:, None] * dr[:, None]) > r * r] = 0
        return mask
    lo = {k: p.getAttr(k) + margin for k in ("x_start", "y_start") if p.hasAttr(k)}
    hi = {k: p.getAttr(k) + margin for k in ("x_stop", "y_stop") if p.hasAttr(k)}
    if "x_start" in lo:
        mask[:, :lo["x_start"]] = 0.0
    if "x_stop" in hi:
        mask[:, hi["x_stop"]:-1] = 0.0
    if "y_start" in lo:
        mask[:lo["y_start"], :] = 0.0
    if "y_stop" in hi:
        mask[hi["y_stop"]:-1, :] = 0.0
    return mask


def _ptr(a):
    """ctypes pointer of a C-contiguous float64 numpy array, an integer
    device address, or None."""
    if a is None:
        return None, 0
    if isinstance(a, int):
        return ctypes.c_void_p(a), 1
    if hasattr(a, "data_ptr"):   # a CUDA tensor
        return ctypes.c_void_p(a.data_ptr()), 1
    a = numpy.ascontiguousarray(a, dtype=numpy.float64)
    return a, 0


class _FinderCore(object):
    """Shared state of the one-frame and the batched finder."""

    def __init__(self, parameters):
        self.parameters = _Params(parameters)
        p = self.parameters
        self.clib = loadclib.load()
        self.find_max_radius = p.getAttr("find_max_radius")
        self.iterations = p.getAttr("iterations")
        self.sigma = p.getAttr("sigma")
        self.threshold = p.getAttr("threshold")
        if p.getAttr("roi_size", -1) != -1:
            self.roi_size = p.getAttr("roi_size")
        else:
            self.roi_size = int(8.0 * self.sigma)
            if p.getAttr("model", None) != "2dfixed":
                self.roi_size = int(1.5 * self.roi_size)
        self.margin = int(self.roi_size / 2 + 2)
        self.z_value = p.getAttr("z_value", 0.0)
        if p.hasAttr("peak_locations"):
            raise FittingException("peak_locations files are not read by the GPU finder")
        self.bg_filter = self.fg_mfilter = self.fg_vfilter = None
        self.camera_variance = None
        self.peak_mask = None
        self.fh = None
        self.pf_iterations = 0
        self.cur_threshold = None
        self.shape = None

    def _setup(self, shape):
        """Filters, mask and finder handle for frames of this shape
        (newImage, fitting.py:304-339 and :424-442)."""
        if self.fh is not None:
            if tuple(shape) != self.shape:
                raise FittingException("frame shape changed from %s to %s" % (self.shape, tuple(shape)))
            return
        self.shape = tuple(shape)
        p = self.parameters
        self.peak_mask = peakMask(shape, p.p, self.margin)
        self.bg_filter = MatchedFilter(gaussianPSF(shape, p.getAttr("background_sigma")), memoize=True,
                                       max_diff=1.0e-3)
        if p.hasAttr("foreground_sigma") and p.getAttr("foreground_sigma") > 0.0:
            fg_psf = gaussianPSF(shape, p.getAttr("foreground_sigma"))
            self.fg_mfilter = MatchedFilter(fg_psf, memoize=True, max_diff=1.0e-3)
            self.fg_vfilter = MatchedFilter(fg_psf * fg_psf, memoize=True, max_diff=1.0e-3)
        fm = self.fg_mfilter.handle() if self.fg_mfilter else None
        fv = self.fg_vfilter.handle() if self.fg_vfilter else None
        self.fh = self.clib.saFinderCreate(shape[0], shape[1], self.bg_filter.handle(), fm, fv, self.margin,
                                           float(self.find_max_radius), float(self.threshold),
                                           float(self.z_value), float(self.sigma))
        if not self.fh:
            raise FittingException(loadclib.last_error())
        mask = numpy.ascontiguousarray(self.peak_mask, dtype=numpy.float64)
        if numpy.all(mask == 1.0):
            self.clib.saFinderSetMask(self.fh, None)
        else:
            self._ok(self.clib.saFinderSetMask(self.fh, mask.ctypes.data_as(ctypes.c_void_p)))
        if self.camera_variance is not None:
            self._upload_variance()

    def _ok(self, r):
        if r < 0:
            raise FittingException(loadclib.last_error())
        return r

    def _upload_variance(self):
        cv = numpy.ascontiguousarray(self.camera_variance, dtype=numpy.float64)
        self._ok(self.clib.saFinderSetVariance(self.fh, cv.ctypes.data_as(ctypes.c_void_p)))

    def _thresholds(self):
        if self.iterations > 4:
            self.cur_threshold = self.threshold + 4.0
        else:
            self.cur_threshold = self.threshold + float(self.iterations)

    def _after_find(self, total):
        """findPeaks' done flag (fitting.py:274-302)."""
        if self.cur_threshold > self.threshold:
            self.cur_threshold -= 1.0
            return False
        return total == 0

    def padArray(self, np_array):
        return padArray(np_array, self.margin)

    def setVariance(self, camera_variance):
        self.camera_variance = self.padArray(camera_variance)
        if self.fh is not None:
            self._upload_variance()
        return self.camera_variance

    def getROISize(self):
        return self.roi_size

    def kernel_launches(self):
        return int(self.clib.saFinderKernelLaunches(self.fh)) if self.fh else 0

    def cleanUp(self):
        if self.fh:
            self.clib.saFinderCleanup(self.fh)
        self.fh = None
        for f in (self.bg_filter, self.fg_mfilter, self.fg_vfilter):
            if f is not None:
                f.cleanup()
        self.bg_filter = self.fg_mfilter = self.fg_vfilter = None


class PeakFinderGaussian(_FinderCore):
    """One frame at a time, host arrays in and out, as the reference."""

    def newImage(self, new_image):
        self._setup(new_image.shape)
        self.image = numpy.ascontiguousarray(new_image, dtype=numpy.float64)
        self._thresholds()
        self._ok(self.clib.saFinderNewImages(self.fh, self.image.ctypes.data_as(ctypes.c_void_p), 1, 0))

    def estimateBackground(self, fit_peaks_image, bg_estimate=None):
        fit, _ = _ptr(fit_peaks_image)
        bge, _ = _ptr(bg_estimate)
        self._ok(self.clib.saFinderEstimateBackground(
            self.fh, None if fit is None else fit.ctypes.data_as(ctypes.c_void_p),
            None if bge is None else bge.ctypes.data_as(ctypes.c_void_p), 0))
        self.background = numpy.zeros(self.shape)
        self._ok(self.clib.saFinderGetArray(self.fh, 0, self.background))
        return self.background

    def peakFinder(self, fit_peaks_image):
        fit, _ = _ptr(fit_peaks_image)
        counts = numpy.zeros(1, dtype=numpy.int32)
        n = self._ok(self.clib.saFinderFindPeaks(
            self.fh, None if fit is None else fit.ctypes.data_as(ctypes.c_void_p), 0, counts))
        rows = numpy.zeros((max(n, 1), 4))
        self.clib.saFinderGetPeaks(self.fh, rows)
        rows = rows[:n]
        return {"x": numpy.ascontiguousarray(rows[:, 0]), "y": numpy.ascontiguousarray(rows[:, 1]),
                "z": numpy.ascontiguousarray(rows[:, 2]), "sigma": numpy.ascontiguousarray(rows[:, 3])}

    def findPeaks(self, fit_peaks_image):
        self.pf_iterations += 1
        new_peaks = self.peakFinder(fit_peaks_image)
        return [new_peaks, "finder", self._after_find(new_peaks["x"].size)]

    def significance(self):
        """The masked foreground / noise image of the last peakFinder."""
        out = numpy.zeros(self.shape)
        self._ok(self.clib.saFinderGetArray(self.fh, 1, out))
        return out


class BatchPeakFinder(_FinderCore):
    """n_frames padded frames of one shape at once, resident on the GPU.

        finder = BatchPeakFinder(params, (534, 534), 64)
        finder.newImages(frames)                 # (64, 534, 534) host array or device address
        finder.estimateBackground()              # zero fit image
        counts, done = finder.findPeaks()
        finder.handoff(batch_fitter)             # images, backgrounds, "finder" peaks, all on the GPU
    """

    def __init__(self, parameters, shape, n_frames):
        super(BatchPeakFinder, self).__init__(parameters)
        self.n_frames = int(n_frames)
        self._setup(tuple(shape))
        self.counts = numpy.zeros(self.n_frames, dtype=numpy.int32)
        self.total = 0

    def newImages(self, images):
        self._thresholds()
        ptr, dev = _ptr(images)
        if not dev:
            assert ptr.shape == (self.n_frames,) + self.shape, "expected %s frames" % ((self.n_frames,) + self.shape,)
            self._images = ptr
            ptr = ptr.ctypes.data_as(ctypes.c_void_p)
        self._ok(self.clib.saFinderNewImages(self.fh, ptr, self.n_frames, dev))

    def estimateBackground(self, fit_images=None, bg_estimate=None):
        fit, dev = _ptr(fit_images)
        bge, dev2 = _ptr(bg_estimate)
        if fit is not None and bge is not None and dev != dev2:
            raise FittingException("fit images and background estimate must both be on the host or the GPU")
        on_dev = dev if fit is not None else dev2
        c = lambda a, d: None if a is None else (a if d else a.ctypes.data_as(ctypes.c_void_p))
        self._ok(self.clib.saFinderEstimateBackground(self.fh, c(fit, dev), c(bge, dev2), on_dev))

    def findPeaks(self, fit_images=None):
        self.pf_iterations += 1
        fit, dev = _ptr(fit_images)
        arg = None if fit is None else (fit if dev else fit.ctypes.data_as(ctypes.c_void_p))
        self.total = self._ok(self.clib.saFinderFindPeaks(self.fh, arg, dev, self.counts))
        return self.counts.copy(), self._after_find(self.total)

    def peaks(self):
        """The found peaks as per-frame dicts of x, y, z, sigma."""
        rows = numpy.zeros((max(self.total, 1), 4))
        self.clib.saFinderGetPeaks(self.fh, rows)
        out, k = [], 0
        for n in self.counts:
            r = rows[k:k + n]
            out.append({"x": r[:, 0].copy(), "y": r[:, 1].copy(), "z": r[:, 2].copy(), "sigma": r[:, 3].copy()})
            k += n
        return out

    def background(self):
        out = numpy.zeros((self.n_frames,) + self.shape)
        self._ok(self.clib.saFinderGetArray(self.fh, 0, out))
        return out

    def significance(self):
        out = numpy.zeros((self.n_frames,) + self.shape)
        self._ok(self.clib.saFinderGetArray(self.fh, 1, out))
        return out

    def device_pointers(self):
        """Device addresses of (backgrounds, peak rows)."""
        return self.clib.saFinderBackgroundDevice(self.fh), self.clib.saFinderPeaksDevice(self.fh)

    def handoff(self, fitter, images_device=None):
        """Give a BatchFitter of the same shape and frame count this batch's
        background estimates and found peaks ("finder" rows) straight from
        device memory.  The images are loaded from images_device (a device
        address of n_frames float64 frames) when given, else from the host
        frames passed to newImages."""
        if fitter.n_frames != self.n_frames or tuple(fitter.shape) != self.shape:
            raise FittingException("fitter and finder disagree on frames or shape")
        fitter.ensure_frames(max(int(self.counts.max()) if self.counts.size else 1, 1))
        if images_device is not None:
            fitter.load_images(images_device, on_device=True, dtype_bits=64)
        else:
            fitter.load_images(self._images)
        fitter.load_backgrounds(self.clib.saFinderBackgroundDevice(self.fh), on_device=True, dtype_bits=64)
        fitter.load_peaks_device(self.clib.saFinderPeaksDevice(self.fh), self.counts, "finder")


class PeakFinderArbitraryPSF(_FinderCore):
    """The reference's PeakFinderArbitraryPSF (sa_library/fitting.py:504-672),
    the finder of Spliner / pupil-function / PSF-FFT analysis, on the GPU.
    psf_object is the reference's PSF object (getMargin, getScaledZ,
    isValidZ, getPSF(z, shape=..., normalize=False)); parameters may hold
    z_value, a list of z (um) at which foreground filters are made.  One
    frame at a time with host arrays; peaks come back as x, y, z."""

    def __init__(self, parameters=None, psf_object=None):
        self.parameters = _Params(parameters)
        p = self.parameters
        self.clib = loadclib.load()
        self.find_max_radius = p.getAttr("find_max_radius")
        self.iterations = p.getAttr("iterations")
        self.sigma = p.getAttr("sigma")
        self.threshold = p.getAttr("threshold")
        if p.hasAttr("peak_locations"):
            raise FittingException("peak_locations files are not read by the GPU finder")
        self.psf_object = psf_object
        self.margin = psf_object.getMargin()
        zv = p.getAttr("z_value", [0.0])
        self.fg_mfilter_zval = [z * 1.0e3 for z in (zv if numpy.ndim(zv) else [zv])]
        self.z_values = []
        for zval in self.fg_mfilter_zval:
            assert psf_object.isValidZ(zval)
            self.z_values.append(psf_object.getScaledZ(zval))
        self.bg_filter = None
        self.fg_mfilter, self.fg_vfilter = [], []
        self.camera_variance = None
        self.peak_mask = None
        self.fh = None
        self.pf_iterations = 0
        self.cur_threshold = None
        self.shape = None

    def _setup(self, shape):
        if self.fh is not None:
            if tuple(shape) != self.shape:
                raise FittingException("frame shape changed from %s to %s" % (self.shape, tuple(shape)))
            return
        self.shape = tuple(shape)
        p = self.parameters
        self.peak_mask = peakMask(shape, p.p, self.margin)
        self.bg_filter = MatchedFilter(gaussianPSF(shape, p.getAttr("background_sigma")), memoize=True,
                                       max_diff=1.0e-3)
        for zval in self.fg_mfilter_zval:
            psf = self.psf_object.getPSF(zval, shape=shape, normalize=False)
            psf_norm = psf / numpy.sum(psf)
            self.fg_mfilter.append(MatchedFilter(psf_norm, memoize=True, max_diff=1.0e-3))
            self.fg_vfilter.append(MatchedFilter(psf_norm * psf_norm, memoize=True, max_diff=1.0e-3))
        n = len(self.fg_mfilter)
        fms = (ctypes.c_void_p * n)(*[f.handle() for f in self.fg_mfilter])
        fvs = (ctypes.c_void_p * n)(*[f.handle() for f in self.fg_vfilter])
        zv = numpy.ascontiguousarray(self.z_values, dtype=numpy.float64)
        self.fh = self.clib.saFinderCreateArbitrary(shape[0], shape[1], self.bg_filter.handle(), n, fms, fvs, zv,
                                                    self.margin, float(self.find_max_radius),
                                                    float(self.threshold))
        if not self.fh:
            raise FittingException(loadclib.last_error())
        mask = numpy.ascontiguousarray(self.peak_mask, dtype=numpy.float64)
        if not numpy.all(mask == 1.0):
            self._ok(self.clib.saFinderSetMask(self.fh, mask.ctypes.data_as(ctypes.c_void_p)))
        if self.camera_variance is not None:
            self._upload_variance()

    def cleanUp(self):
        if self.fh:
            self.clib.saFinderCleanup(self.fh)
        self.fh = None
        for f in [self.bg_filter] + self.fg_mfilter + self.fg_vfilter:
            if f is not None:
                f.cleanup()
        self.bg_filter = None
        self.fg_mfilter, self.fg_vfilter = [], []

    newImage = PeakFinderGaussian.newImage
    estimateBackground = PeakFinderGaussian.estimateBackground

    def peakFinder(self, fit_peaks_image):
        fit, _ = _ptr(fit_peaks_image)
        counts = numpy.zeros(1, dtype=numpy.int32)
        n = self._ok(self.clib.saFinderFindPeaks(
            self.fh, None if fit is None else fit.ctypes.data_as(ctypes.c_void_p), 0, counts))
        rows = numpy.zeros((max(n, 1), 4))
        self.clib.saFinderGetPeaks(self.fh, rows)
        rows = rows[:n]
        return {"x": numpy.ascontiguousarray(rows[:, 0]), "y": numpy.ascontiguousarray(rows[:, 1]),
                "z": numpy.ascontiguousarray(rows[:, 2])}

    def findPeaks(self, fit_peaks_image):
        self.pf_iterations += 1
        new_peaks = self.peakFinder(fit_peaks_image)
        return [new_peaks, "finder", self._after_find(new_peaks["x"].size)]

    def significance(self):
        out = numpy.zeros((len(self.z_values),) + self.shape)
        self._ok(self.clib.saFinderGetArray(self.fh, 1, out))
        return out
