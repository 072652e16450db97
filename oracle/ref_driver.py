"""
Drive the reference's own fitting C code, compiled from its sources by
``make -C oracle ref`` into oracle/_ref/, through ctypes.

TEST INFRASTRUCTURE ONLY, and only where the reference tree exists (it
does not travel to the GPU host).  Used to pin the oracle restatement and
to generate the golden fixtures under tests/golden/.

The argument types follow the reference's ctypes declarations
(sa_library/dao_fit_c.py:147-238, spliner/cubic_fit_c.py:21-98); only the
leading counter/size fields of its fitData struct are mirrored, to read
nfit (sa_library/dao_fit_c.py:22-77).
"""
import ctypes
import os

import numpy
from numpy.ctypeslib import ndpointer

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")


class _FitDataHead(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in
                ["n_dposv", "n_iterations", "n_lost", "n_margin", "n_neg_fi", "n_neg_height",
                 "n_non_converged", "n_non_decr", "fit_size_x", "fit_size_y", "image_size_x",
                 "image_size_y", "jac_size", "max_nfit", "nfit", "roi_n_index"]]


def available():
    return (os.path.exists(os.path.join(REF_DIR, "libdao_fit.so")) and
            os.path.exists(os.path.join(REF_DIR, "libcubic_fit.so")))


def _declare(lib, spline):
    f64 = ndpointer(dtype=numpy.float64, flags="C_CONTIGUOUS")
    i32 = ndpointer(dtype=numpy.int32, flags="C_CONTIGUOUS")
    vp = ctypes.c_void_p
    lib.mFitGetNError.argtypes = [vp]
    lib.mFitGetNError.restype = ctypes.c_int
    lib.mFitGetPeakPropertyDouble.argtypes = [vp, f64, ctypes.c_char_p]
    lib.mFitGetPeakPropertyInt.argtypes = [vp, i32, ctypes.c_char_p]
    lib.mFitGetUnconverged.argtypes = [vp]
    lib.mFitGetUnconverged.restype = ctypes.c_int
    lib.mFitIterateLM.argtypes = [vp]
    lib.mFitNewBackground.argtypes = [vp, f64]
    lib.mFitNewImage.argtypes = [vp, f64]
    lib.mFitGetFitImage.argtypes = [vp, f64]
    lib.mFitGetResidual.argtypes = [vp, f64]
    lib.mFitSetPeakStatus.argtypes = [vp, i32]
    lib.mFitRemoveErrorPeaks.argtypes = [vp]
    lib.mFitRemoveRunningPeaks.argtypes = [vp]
    if spline:
        lib.initSpline3D.argtypes = [f64, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        lib.initSpline3D.restype = vp
        lib.initSpline2D.argtypes = [f64, ctypes.c_int, ctypes.c_int]
        lib.initSpline2D.restype = vp
        lib.cfInitialize.argtypes = [vp, f64, f64, ctypes.c_double, ctypes.c_int, ctypes.c_int]
        lib.cfInitialize.restype = ctypes.POINTER(_FitDataHead)
        lib.cfInitialize2D.argtypes = [vp]
        lib.cfInitialize3D.argtypes = [vp]
        lib.cfNewPeaks.argtypes = [vp, f64, ctypes.c_char_p, ctypes.c_int]
        lib.cfCleanup.argtypes = [vp]
    else:
        lib.daoInitialize.argtypes = [f64, f64, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_int]
        lib.daoInitialize.restype = ctypes.POINTER(_FitDataHead)
        lib.daoInitialize2DFixed.argtypes = [vp]
        lib.daoInitialize2D.argtypes = [vp, ctypes.c_double, ctypes.c_double]
        lib.daoInitialize3D.argtypes = [vp, ctypes.c_double, ctypes.c_double]
        lib.daoInitializeZ.argtypes = [vp, f64, f64, ctypes.c_double, ctypes.c_double]
        lib.daoNewPeaks.argtypes = [vp, f64, ctypes.c_char_p, ctypes.c_int]
        lib.daoCleanup.argtypes = [vp]


class RefFitter(object):
    """The reference C fitter with the same method names as oracle.OracleFitter."""

    def __init__(self, model, shape, rqe=None, scmos_cal=None, roi_size=10, sigma_range=None,
                 wx_params=None, wy_params=None, min_z=None, max_z=None, spline=None,
                 tol=1.0e-6):
        self.spline = model.startswith("spline")
        name = "libcubic_fit.so" if self.spline else "libdao_fit.so"
        lib = ctypes.CDLL(os.path.join(REF_DIR, name), mode=ctypes.RTLD_LOCAL)
        _declare(lib, self.spline)
        self.lib = lib
        self.shape = tuple(shape)
        ny, nx = shape
        self.rqe = numpy.ascontiguousarray(numpy.ones(shape) if rqe is None else rqe, dtype=numpy.float64)
        self.scmos = numpy.ascontiguousarray(numpy.zeros(shape) if scmos_cal is None else scmos_cal,
                                             dtype=numpy.float64)
        if self.spline:
            coeff = numpy.ascontiguousarray(spline, dtype=numpy.float64)
            if coeff.ndim == 4:
                sp = lib.initSpline3D(coeff.ravel(), coeff.shape[0], coeff.shape[1], coeff.shape[2])
            else:
                sp = lib.initSpline2D(coeff.ravel(), coeff.shape[0], coeff.shape[1])
            self.mfit = lib.cfInitialize(sp, self.rqe, self.scmos, tol, nx, ny)
            if model == "spline3D":
                lib.cfInitialize3D(self.mfit)
            else:
                lib.cfInitialize2D(self.mfit)
        else:
            self.mfit = lib.daoInitialize(self.rqe, self.scmos, tol, nx, ny, roi_size)
            if model == "2dfixed":
                lib.daoInitialize2DFixed(self.mfit)
            elif model in ("2d", "3d"):
                wmax = 1.0 / (2.0 * sigma_range[0] * sigma_range[0])
                wmin = 1.0 / (2.0 * sigma_range[1] * sigma_range[1])
                if model == "2d":
                    lib.daoInitialize2D(self.mfit, wmin, wmax)
                else:
                    lib.daoInitialize3D(self.mfit, wmin, wmax)
            elif model == "Z":
                lib.daoInitializeZ(self.mfit, numpy.ascontiguousarray(wx_params, dtype=numpy.float64),
                                   numpy.ascontiguousarray(wy_params, dtype=numpy.float64),
                                   float(min_z), float(max_z))

    def cleanup(self, verbose=False):
        if self.mfit is not None:
            if self.spline:
                self.lib.cfCleanup(self.mfit)
            else:
                self.lib.daoCleanup(self.mfit)
            self.mfit = None

    def newImage(self, image):
        self.lib.mFitNewImage(self.mfit, numpy.ascontiguousarray(image, dtype=numpy.float64))

    def newBackground(self, bg):
        self.lib.mFitNewBackground(self.mfit, numpy.ascontiguousarray(bg, dtype=numpy.float64))

    def newPeaks(self, peaks, peaks_type):
        from oracle.oracle import format_peaks
        c = format_peaks(peaks, peaks_type, self.spline)
        fn = self.lib.cfNewPeaks if self.spline else self.lib.daoNewPeaks
        fn(self.mfit, c, ctypes.c_char_p(peaks_type.encode()), c.shape[0])

    def iterate(self):
        self.lib.mFitIterateLM(self.mfit)

    def doFit(self, max_iterations=2000):
        i = 0
        self.iterate()
        while self.getUnconverged() and (i < max_iterations):
            self.iterate()
            i += 1
        return i + 1

    def getUnconverged(self):
        return self.lib.mFitGetUnconverged(self.mfit)

    def getNError(self):
        return self.lib.mFitGetNError(self.mfit)

    def getNFit(self):
        return self.mfit.contents.nfit

    def getNFitMax(self):
        return self.mfit.contents.max_nfit

    def counters(self):
        c = self.mfit.contents
        return {n: getattr(c, n) for n in ["n_dposv", "n_iterations", "n_lost", "n_margin",
                                            "n_neg_fi", "n_neg_height", "n_non_converged",
                                            "n_non_decr"]}

    def getPeakProperty(self, name):
        n = self.getNFit()
        if name == "significance":
            return self.getPeakProperty("fg_sum") / numpy.sqrt(self.getPeakProperty("bg_sum"))
        if name in ("iterations", "status"):
            v = numpy.zeros(n, dtype=numpy.int32)
            self.lib.mFitGetPeakPropertyInt(self.mfit, v, ctypes.c_char_p(name.encode()))
            return v
        if name == "jacobian":
            v = numpy.zeros((n, self.mfit.contents.jac_size))
        else:
            v = numpy.zeros(n)
        self.lib.mFitGetPeakPropertyDouble(self.mfit, v, ctypes.c_char_p(name.encode()))
        return v

    def getFitImage(self):
        out = numpy.zeros(self.shape)
        self.lib.mFitGetFitImage(self.mfit, out)
        return out

    def getResidual(self):
        out = numpy.zeros(self.shape)
        self.lib.mFitGetResidual(self.mfit, out)
        return out

    def setPeakStatus(self, status):
        self.lib.mFitSetPeakStatus(self.mfit, numpy.ascontiguousarray(status, dtype=numpy.int32))

    def removeErrorPeaks(self):
        self.lib.mFitRemoveErrorPeaks(self.mfit)

    def removeRunningPeaks(self):
        self.lib.mFitRemoveRunningPeaks(self.mfit)


class _MPFitHead(ctypes.Structure):
    """The leading fields of the reference's mpFit (multi_plane/mp_fit.h:12-44),
    through the per-channel fitData pointers."""
    _fields_ = ([(n, ctypes.c_int) for n in ["im_size_x", "im_size_y", "independent_heights", "n_channels",
                                               "n_weights"]] +
                [(n, ctypes.c_double) for n in ["tolerance", "w_z_offset", "w_z_scale", "zmin", "zmax"]] +
                [(n, ctypes.POINTER(ctypes.c_double)) for n in ["xt_0toN", "yt_0toN", "xt_Nto0", "yt_Nto0", "w_bg",
                                                                 "w_h", "w_x", "w_y", "w_z", "heights"]] +
                [(n, ctypes.c_void_p) for n in ["jacobian", "w_jacobian", "hessian", "w_hessian"]] +
                [("fit_data", ctypes.POINTER(ctypes.POINTER(_FitDataHead)))])


def mp_available():
    return os.path.exists(os.path.join(REF_DIR, "libmp_fit_dao.so"))


class RefMPDaoFitter(object):
    """The reference's 2D Gaussian multi-plane fitter (mp_fit.c + mp_fit_dao.c)
    with the call sequence of multi_plane/mp_fit_dao_c.py MPFitDao2D:
    mpInitialize(tol * n_channels), mpDaoInitialize2DChannel per channel,
    mpSetTransforms, mpSetWeights (equal weights, z_size 2), mpDaoNewPeaks,
    mpIterateLM."""

    PROPS_D = ("x", "y", "height", "background", "xsigma", "ysigma", "error", "z")
    PROPS_I = ("status", "iterations")

    def __init__(self, shape, n_channels, rqe, variance, sigma_range, roi_size, transforms, tol=1.0e-6):
        lib = ctypes.CDLL(os.path.join(REF_DIR, "libmp_fit_dao.so"))
        _declare(lib, False)
        f64 = ndpointer(dtype=numpy.float64, flags="C_CONTIGUOUS")
        vp = ctypes.c_void_p
        lib.mpInitialize.argtypes = [ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        lib.mpInitialize.restype = ctypes.POINTER(_MPFitHead)
        lib.mpDaoInitialize2DChannel.argtypes = [vp, f64, f64, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                                 ctypes.c_int]
        lib.mpSetTransforms.argtypes = [vp, f64, f64, f64, f64]
        lib.mpSetWeights.argtypes = [vp, f64, f64, f64, f64, f64, ctypes.c_int]
        lib.mpSetWeightsIndexing.argtypes = [vp, ctypes.c_double, ctypes.c_double]
        lib.mpDaoNewPeaks.argtypes = [vp, f64, ctypes.c_char_p, ctypes.c_int]
        lib.mpIterateLM.argtypes = [vp]
        lib.mpCleanup.argtypes = [vp]
        self.lib = lib
        self.nc = n_channels
        ny, nx = shape
        self.mp = lib.mpInitialize(tol * n_channels, n_channels, 1, nx, ny)
        wmax = 1.0 / (2.0 * sigma_range[0] * sigma_range[0])
        wmin = 1.0 / (2.0 * sigma_range[1] * sigma_range[1])
        self._keep = []
        for c in range(n_channels):
            r = numpy.ascontiguousarray(rqe[c], dtype=numpy.float64)
            v = numpy.ascontiguousarray(variance[c], dtype=numpy.float64)
            self._keep += [r, v]
            lib.mpDaoInitialize2DChannel(self.mp, r, v, wmin, wmax, roi_size, c)
        lib.mpSetTransforms(self.mp, *[numpy.ascontiguousarray(t, dtype=numpy.float64) for t in transforms])
        w = numpy.ascontiguousarray(numpy.ones((2, n_channels)) / float(n_channels))
        lib.mpSetWeights(self.mp, w, w, w, w, w, 2)
        lib.mpSetWeightsIndexing(self.mp, 0.0, 0.0)

    def channel(self, c):
        return self.mp.contents.fit_data[c]

    def newImage(self, images):
        for c in range(self.nc):
            self.lib.mFitNewImage(self.channel(c), numpy.ascontiguousarray(images[c], dtype=numpy.float64))

    def newBackground(self, bgs):
        for c in range(self.nc):
            self.lib.mFitNewBackground(self.channel(c), numpy.ascontiguousarray(bgs[c], dtype=numpy.float64))

    def newPeaks(self, rows, ptype):
        rows = numpy.ascontiguousarray(rows, dtype=numpy.float64)
        self.lib.mpDaoNewPeaks(self.mp, rows, ptype.encode(), rows.shape[0])

    def iterate(self):
        self.lib.mpIterateLM(self.mp)

    def getUnconverged(self):
        return self.lib.mFitGetUnconverged(self.channel(0))

    def doFit(self, max_iterations=200):
        """MultiFitter.doFit (sa_library/dao_fit_c.py:332-356)."""
        self.iterate()
        i = 0
        while (self.getUnconverged() > 0) and (i < max_iterations):
            self.iterate()
            i += 1
        return i + 1

    def getPeakProperty(self, name, channel=0):
        ch = self.channel(channel)
        n = ch.contents.nfit
        if name in self.PROPS_I:
            out = numpy.zeros(n, dtype=numpy.int32)
            self.lib.mFitGetPeakPropertyInt(ch, out, name.encode())
        else:
            out = numpy.zeros(n, dtype=numpy.float64)
            self.lib.mFitGetPeakPropertyDouble(ch, out, name.encode())
        return out

    def counters(self, channel=0):
        h = self.channel(channel).contents
        return numpy.array([h.n_dposv, h.n_iterations, h.n_lost, h.n_margin, h.n_neg_fi, h.n_neg_height,
                            h.n_non_converged, h.n_non_decr], dtype=numpy.int64)

    def cleanup(self):
        if self.mp:
            self.lib.mpCleanup(self.mp)
            self.mp = None
