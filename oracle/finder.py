"""
CPU restatement of the reference's Gaussian peak finder: the matched
filter (FFT convolution), the local-maxima finder and the
PeakFinderGaussian.peakFinder pipeline that feeds the fitter "finder" peaks.

TEST INFRASTRUCTURE ONLY: the checker for the GPU finder in tests/ and the
timed CPU baseline in bench.py.  Product code never imports this module.

Followed, function by function:

  gaussian_psf        simulator/draw_gaussians.c:24-80 (resolution 1) drawn
                      at the image centre and normalised, as
                      sa_library/fitting.py:38-46 (gaussianPSF)
  recenter_psf        sa_library/recenter_psf.py:11-19
  MatchedFilter       sa_library/matched_filter.c:93-106 (convolve),
                      :118-150 (convolveMemo), :163-215 (initialize: PSF
                      transform scaled by 1/(x_size*y_size)); the FFTs are
                      numpy's, which the reference's own test takes as the
                      truth (test/test_matched_filter.py, test 5)
  calc_max_peaks      sa_library/ia_utilities.c:58-75
  find_local_maxima   sa_library/ia_utilities.c:105-160 and isLocalMaxima
                      :177-210, including the truncating int conversions of
                      the search box and of radius**2
  MaximaFinder        sa_library/ia_utilities_c.py:132-250 (margin + 1,
                      taken initialised to 1 - n_duplicates)
  mark_dimmer_peaks,  sa_library/ia_utilities.c:221-430 (the post-fit
  mark_low_significance_peaks, running_if_has_neighbors, nearest
                      culling; brute-force neighbour search with the
                      kd-tree's membership test)
  pad_array           sa_library/fitting.py:112-132
  peak_mask           sa_library/fitting.py:134-176
  PeakFinderGaussian  sa_library/fitting.py:185-501 (newImage,
                      estimateBackground, findPeaks, peakFinder)
  PeakFinderArbitraryPSF  sa_library/fitting.py:504-672

Pinned by tests/golden/g_finder.npz, made by tests/golden/make_golden_finder.py
from the reference's own ia_utilities.c and draw_gaussians.c compiled from
source.  The reference's matched_filter.c needs FFTW, which is not
installed, so its restatement here is pinned by the reference's own test
criterion (agreement with numpy's FFT convolution).
"""
import math

import numpy


def gaussian_psf(shape, sigma):
    """A unit-sum Gaussian of the given sigma centred at (shape/2), drawn as
    draw_gaussians.c draws it: exp(-(dx^2 + dy^2)/(2 sigma^2)) on the
    pixels within int(5 sigma) of the centre's integer part, zero beyond."""
    rows, cols = shape
    px, py = 0.5 * rows, 0.5 * cols
    aw = max(int(5.0 * sigma), 1)
    sg = 1.0 / (2.0 * sigma * sigma)
    img = numpy.zeros(shape)
    r0, r1 = max(int(px) - aw, 0), min(int(px) + aw + 1, rows)
    c0, c1 = max(int(py) - aw, 0), min(int(py) + aw + 1, cols)
    j = numpy.arange(r0, r1, dtype=numpy.float64)[:, None]
    k = numpy.arange(c0, c1, dtype=numpy.float64)[None, :]
    x = (j - px) * (j - px) * sg
    y = (k - py) * (k - py) * sg
    img[r0:r1, c0:c1] = numpy.exp(-1.0 * (x + y))
    return img / numpy.sum(img)


def recenter_psf(psf):
    out = numpy.roll(psf, int(psf.shape[0] / 2), axis=0)
    return numpy.roll(out, int(psf.shape[1] / 2), axis=1)


class MatchedFilter:
    """Circular convolution with a PSF through its 2D real FFT."""

    def __init__(self, psf, memoize=False, max_diff=0.1):
        rc = recenter_psf(numpy.asarray(psf, dtype=numpy.float64))
        self.shape = rc.shape
        self.psf_fft = numpy.fft.rfft2(rc)
        self.memoize = memoize
        self.max_diff = float(max_diff) if memoize else 0.0
        self.old_image = numpy.zeros(self.shape) if memoize else None
        # the transform's work array holds the recentred PSF after set-up
        self.last = rc.copy()

    def _convolve(self, image):
        self.last = numpy.fft.irfft2(numpy.fft.rfft2(image) * self.psf_fft, s=self.shape)
        return self.last.copy()

    def convolve(self, image):
        image = numpy.ascontiguousarray(image, dtype=numpy.float64)
        if not self.memoize:
            return self._convolve(image)
        if numpy.any(numpy.abs(image - self.old_image) > self.max_diff):
            self.old_image = image.copy()
            return self._convolve(image)
        return self.last.copy()


def calc_max_peaks(images, taken, margin, threshold):
    n = 0
    for img, tk in zip(images, taken):
        inner = (slice(margin, img.shape[0] - margin), slice(margin, img.shape[1] - margin))
        n += int(numpy.count_nonzero((img[inner] > threshold) & (tk[inner] < 1)))
    return n


def _trunc(v):
    return int(math.trunc(v))


def find_local_maxima(images, taken, margin, radius, threshold, z_range, z_values):
    """Local maxima above threshold not yet taken, in plane, row, column
    order; increments taken at each one found.  Returns x, y, z, h."""
    zsize = len(images)
    ysize, xsize = images[0].shape
    rr = _trunc(radius * radius)
    cr = math.ceil(radius)
    xs, ys, zs, hs = [], [], [], []
    for zi in range(zsize):
        sz = max(zi - z_range, 0)
        ez = min(zi + z_range, zsize - 1)
        img = images[zi]
        cand = (img > threshold) & (taken[zi] < 1)
        cand[:margin, :] = False
        cand[ysize - margin:, :] = False
        cand[:, :margin] = False
        cand[:, xsize - margin:] = False
        for yi, xi in zip(*numpy.nonzero(cand)):
            yi, xi = int(yi), int(xi)
            sy = max(_trunc(yi - radius), 0)
            ey = min(_trunc(yi + radius), ysize - 1)
            sx = max(_trunc(xi - cr), 0)
            ex = min(_trunc(xi + cr), xsize - 1)
            cur = img[yi, xi]
            is_max = True
            for zj in range(sz, ez + 1):
                other = images[zj]
                for yj in range(sy, ey + 1):
                    dy = (yj - yi) * (yj - yi)
                    for xj in range(sx, ex + 1):
                        dx = (xj - xi) * (xj - xi)
                        if dx + dy > rr:
                            continue
                        v = other[yj, xj]
                        if yj <= yi and xj <= xi:
                            if v > cur:
                                is_max = False
                        elif v >= cur:
                            is_max = False
                        if not is_max:
                            break
                    if not is_max:
                        break
                if not is_max:
                    break
            if is_max:
                taken[zi][yi, xi] += 1
                zs.append(z_values[zi])
                ys.append(float(yi))
                xs.append(float(xi))
                hs.append(cur)
    f = numpy.array
    return f(xs, dtype=float), f(ys, dtype=float), f(zs, dtype=float), f(hs, dtype=float)


class MaximaFinder:
    def __init__(self, margin, radius, threshold, z_values, n_duplicates=1, z_range=None):
        self.margin = int(margin + 1)
        self.radius = float(radius)
        self.threshold = float(threshold)
        self.z_values = list(z_values)
        self.z_range = len(self.z_values) if z_range is None else int(z_range)
        self.n_duplicates = n_duplicates
        self.taken = None

    def findMaxima(self, images, want_height=False):
        if self.taken is None:
            self.taken = [numpy.ones(images[0].shape, dtype=numpy.int32) - self.n_duplicates
                          for _ in images]
        x, y, z, h = find_local_maxima(images, self.taken, self.margin, self.radius,
                                       self.threshold, self.z_range, self.z_values)
        return [x, y, z, h] if want_height else [x, y, z]

    def resetTaken(self):
        if self.taken is not None:
            for t in self.taken:
                t[:, :] = 1 - self.n_duplicates


RUNNING, CONVERGED, ERROR = 0, 1, 2


def _within(x, y, qx, qy, r):
    """Indices within r of (qx, qy): dx*dx + dy*dy <= r*r, as
    kd_nearest_range tests it (dbscan/kdtree.c:262-293)."""
    dx = x - qx
    dy = y - qy
    return numpy.nonzero(dx * dx + dy * dy <= r * r)[0]


def mark_dimmer_peaks(x, y, h, status, r_removal, r_neighbors):
    """sa_library/ia_utilities.c:221-283, in the reference's peak order."""
    removed = 0
    for i in range(x.size):
        if status[i] == ERROR:
            continue
        nb = _within(x, y, x[i], y[i], r_removal)
        if nb.size < 2:
            continue
        if numpy.any(h[nb] > h[i]):
            removed += 1
            status[i] = ERROR
            for k in _within(x, y, x[i], y[i], r_neighbors):
                if status[k] == CONVERGED:
                    status[k] = RUNNING
    return removed


def mark_low_significance_peaks(x, y, sig, status, min_sig, r_neighbors):
    """sa_library/ia_utilities.c:292-340."""
    removed = 0
    for i in range(x.size):
        if status[i] == ERROR:
            continue
        if sig[i] > min_sig:
            continue
        status[i] = ERROR
        removed += 1
        for k in _within(x, y, x[i], y[i], r_neighbors):
            if status[k] == CONVERGED:
                status[k] = RUNNING
    return removed


def mark_dimmer_peaks_kd(x, y, h, status, r_removal, r_neighbors):
    """mark_dimmer_peaks with the neighbour lists from a kd-tree (scipy's
    cKDTree), as the reference's C builds one per call
    (sa_library/ia_utilities.c:221-283); same visiting order and status
    rules.  For the timed CPU baseline."""
    from scipy.spatial import cKDTree
    pts = numpy.stack([x, y], axis=1)
    tree = cKDTree(pts)
    near = tree.query_ball_point(pts, r_removal)
    removed = 0
    for i in range(x.size):
        if status[i] == ERROR or len(near[i]) < 2:
            continue
        if numpy.any(h[near[i]] > h[i]):
            removed += 1
            status[i] = ERROR
            for k in tree.query_ball_point(pts[i], r_neighbors):
                if status[k] == CONVERGED:
                    status[k] = RUNNING
    return removed


def mark_low_significance_peaks_kd(x, y, sig, status, min_sig, r_neighbors):
    """mark_low_significance_peaks with kd-tree neighbour queries
    (sa_library/ia_utilities.c:292-340).  For the timed CPU baseline."""
    from scipy.spatial import cKDTree
    pts = numpy.stack([x, y], axis=1)
    tree = cKDTree(pts)
    removed = 0
    for i in range(x.size):
        if status[i] == ERROR or sig[i] > min_sig:
            continue
        status[i] = ERROR
        removed += 1
        for k in tree.query_ball_point(pts[i], r_neighbors):
            if status[k] == CONVERGED:
                status[k] = RUNNING
    return removed


def running_if_has_neighbors(c_x, c_y, n_x, n_y, status, radius):
    """sa_library/ia_utilities.c:401-430."""
    for i in range(c_x.size):
        if status[i] == RUNNING or status[i] == ERROR:
            continue
        if _within(n_x, n_y, c_x[i], c_y[i], radius).size > 0:
            status[i] = RUNNING
    return status


def nearest(px, py, qx, qy, radius):
    """sa_library/ia_utilities.c:347-391: distance to and index of the
    nearest point within radius, -1 / -1 when there is none."""
    dist = numpy.full(qx.size, -1.0)
    index = numpy.full(qx.size, -1, dtype=numpy.int32)
    for i in range(qx.size):
        nb = _within(px, py, qx[i], qy[i], radius)
        if nb.size == 0:
            continue
        dx = px[nb] - qx[i]
        dy = py[nb] - qy[i]
        dd = dx * dx + dy * dy
        j = int(numpy.argmin(dd))
        if dd[j] < radius * radius + 0.1:
            dist[i] = math.sqrt(dd[j])
            index[i] = nb[j]
    return dist, index


def pad_array(a, pad):
    if pad <= 0:
        return a
    xs, ys = a.shape
    lg = numpy.ones((xs + 2 * pad, ys + 2 * pad))
    lg[pad:xs + pad, pad:ys + pad] = a.astype(numpy.float64)
    lg[0:pad, :] = numpy.flipud(lg[pad:2 * pad, :])
    lg[xs + pad:xs + 2 * pad, :] = numpy.flipud(lg[xs:xs + pad, :])
    lg[:, 0:pad] = numpy.fliplr(lg[:, pad:2 * pad])
    lg[:, ys + pad:ys + 2 * pad] = numpy.fliplr(lg[:, ys:ys + pad])
    return lg


def peak_mask(shape, p, margin):
    """The AOI mask, sa_library/fitting.py:134-176 (its circle uses shape[0]
    on both axes; its stop slices end at -1)."""
    mask = numpy.ones(shape)
    has = lambda k: p.get(k) is not None
    if has("x_center"):
        rr = p["aoi_radius"] ** 2
        xr = numpy.arange(mask.shape[0]) - (p["x_center"] + margin)
        yr = numpy.arange(mask.shape[0]) - (p["y_center"] + margin)
        xv, yv = numpy.meshgrid(xr, yr)
        mask[(xv * xv + yv * yv) > rr] = 0
    elif not has("y_center") and not has("aoi_radius"):
        if has("x_start"):
            mask[:, 0:p["x_start"] + margin] = 0.0
        if has("x_stop"):
            mask[:, p["x_stop"] + margin:-1] = 0.0
        if has("y_start"):
            mask[0:p["y_start"] + margin, :] = 0.0
        if has("y_stop"):
            mask[p["y_stop"] + margin:-1, :] = 0.0
    return mask


class PeakFinderGaussian:
    """The finder half of 3D-DAOSTORM / sCMOS analysis on padded frames.

    params: dict with background_sigma, find_max_radius, iterations, sigma,
    threshold, roi_size (or model), optional foreground_sigma, z_value."""

    def __init__(self, params):
        self.p = dict(params)
        self.find_max_radius = self.p["find_max_radius"]
        self.iterations = self.p["iterations"]
        self.sigma = self.p["sigma"]
        self.threshold = self.p["threshold"]
        if self.p.get("roi_size", -1) != -1:
            self.roi_size = self.p["roi_size"]
        else:
            self.roi_size = int(8.0 * self.sigma)
            if self.p.get("model") != "2dfixed":
                self.roi_size = int(1.5 * self.roi_size)
        self.margin = int(self.roi_size / 2 + 2)
        self.z_value = self.p.get("z_value", 0.0)
        self.mfinder = MaximaFinder(self.margin, self.find_max_radius, self.threshold, [self.z_value])
        self.bg_filter = self.fg_mfilter = self.fg_vfilter = None
        self.camera_variance = None
        self.peak_mask = None
        self.background = None
        self.pf_iterations = 0

    def padArray(self, a):
        return pad_array(a, self.margin)

    def setVariance(self, camera_variance):
        self.camera_variance = self.padArray(camera_variance)
        return self.camera_variance

    def newImage(self, new_image):
        self.image = numpy.copy(new_image)
        if self.iterations > 4:
            self.cur_threshold = self.threshold + 4.0
        else:
            self.cur_threshold = self.threshold + float(self.iterations)
        if self.peak_mask is None:
            self.peak_mask = peak_mask(new_image.shape, self.p, self.margin)
        if self.bg_filter is None:
            self.bg_filter = MatchedFilter(gaussian_psf(new_image.shape, self.p["background_sigma"]),
                                           memoize=True, max_diff=1.0e-3)
        self.mfinder.resetTaken()
        fs = self.p.get("foreground_sigma", 0.0)
        if self.fg_mfilter is None and fs > 0.0:
            psf = gaussian_psf(new_image.shape, fs)
            self.fg_mfilter = MatchedFilter(psf, memoize=True, max_diff=1.0e-3)
            self.fg_vfilter = MatchedFilter(psf * psf, memoize=True, max_diff=1.0e-3)

    def estimateBackground(self, fit_peaks_image, bg_estimate=None):
        if bg_estimate is not None:
            self.background = bg_estimate
        else:
            self.background = self.bg_filter.convolve(self.image - fit_peaks_image)
        return self.background

    def peakFinder(self, fit_peaks_image):
        bg_var = self.background + fit_peaks_image
        if self.camera_variance is not None:
            bg_var += self.camera_variance
        if self.fg_vfilter is not None:
            bg_var = self.fg_vfilter.convolve(bg_var)
        mask = bg_var <= 0.1
        if numpy.sum(mask) > 0:
            bg_var[mask] = 0.1
        bg_std = numpy.sqrt(bg_var)
        foreground = self.image - self.background - fit_peaks_image
        if self.fg_mfilter is not None:
            foreground = self.fg_mfilter.convolve(foreground)
        foreground = foreground / bg_std
        masked = foreground * self.peak_mask
        self.last_masked = masked
        x, y, z = self.mfinder.findMaxima([masked])
        return {"x": x, "y": y, "z": z, "sigma": numpy.ones(x.size) * self.sigma}

    def findPeaks(self, fit_peaks_image):
        self.pf_iterations += 1
        new_peaks = self.peakFinder(fit_peaks_image)
        if self.cur_threshold > self.threshold:
            self.cur_threshold -= 1.0
            return [new_peaks, "finder", False]
        return [new_peaks, "finder", new_peaks["x"].size == 0]


class PeakFinderArbitraryPSF(PeakFinderGaussian):
    """sa_library/fitting.py:504-672: per z plane a foreground filter (the
    PSF at that z, unit sum) and its square; the variance takes |fit|; the
    maxima are searched over all planes."""

    def __init__(self, params, psf_object):
        self.p = dict(params)
        self.find_max_radius = self.p["find_max_radius"]
        self.iterations = self.p["iterations"]
        self.sigma = self.p["sigma"]
        self.threshold = self.p["threshold"]
        self.psf_object = psf_object
        self.margin = psf_object.getMargin()
        self.fg_mfilter_zval = [z * 1.0e3 for z in self.p.get("z_value", [0.0])]
        self.z_values = [psf_object.getScaledZ(z) for z in self.fg_mfilter_zval]
        self.mfinder = MaximaFinder(self.margin, self.find_max_radius, self.threshold, self.z_values)
        self.bg_filter = None
        self.fg_mfilter, self.fg_vfilter = [], []
        self.camera_variance = None
        self.peak_mask = None
        self.background = None
        self.pf_iterations = 0

    def newImage(self, new_image):
        self.image = numpy.copy(new_image)
        if self.iterations > 4:
            self.cur_threshold = self.threshold + 4.0
        else:
            self.cur_threshold = self.threshold + float(self.iterations)
        if self.peak_mask is None:
            self.peak_mask = peak_mask(new_image.shape, self.p, self.margin)
        if self.bg_filter is None:
            self.bg_filter = MatchedFilter(gaussian_psf(new_image.shape, self.p["background_sigma"]),
                                           memoize=True, max_diff=1.0e-3)
        self.mfinder.resetTaken()
        if not self.fg_mfilter:
            for zval in self.fg_mfilter_zval:
                psf = self.psf_object.getPSF(zval, shape=new_image.shape, normalize=False)
                psf_norm = psf / numpy.sum(psf)
                self.fg_mfilter.append(MatchedFilter(psf_norm, memoize=True, max_diff=1.0e-3))
                self.fg_vfilter.append(MatchedFilter(psf_norm * psf_norm, memoize=True, max_diff=1.0e-3))

    def peakFinder(self, fit_peaks_image):
        bg_var = self.background + numpy.abs(fit_peaks_image)
        if self.camera_variance is not None:
            bg_var += self.camera_variance
        masked = []
        for fm, fv in zip(self.fg_mfilter, self.fg_vfilter):
            background = fv.convolve(bg_var)
            mask = background <= 0.1
            if numpy.sum(mask) > 0:
                background[mask] = 0.1
            bg_std = numpy.sqrt(background)
            foreground = self.image - self.background - fit_peaks_image
            foreground = fm.convolve(foreground)
            masked.append((foreground / bg_std) * self.peak_mask)
        self.last_masked = masked
        x, y, z = self.mfinder.findMaxima(masked)
        return {"x": x, "y": y, "z": z}
