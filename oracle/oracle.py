"""
ctypes front end of the CPU FP64 oracle (oracle/sa_oracle.c).

TEST INFRASTRUCTURE ONLY: the checker for the GPU engine in tests/,
__graft_entry__.smoke() and the timed CPU baseline in bench.py.  Product
code never imports this module.

The class mirrors the reference's MultiFitter call surface
(sa_library/dao_fit_c.py:257-549, spliner/cubic_fit_c.py:105-215) so that a
parity test drives the oracle and the GPU engine with the same calls.
"""
import ctypes
import os
import subprocess

import numpy
from numpy.ctypeslib import ndpointer

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")

MODELS = {"2dfixed": 0, "2d": 1, "3d": 2, "Z": 3, "spline2D": 4, "spline3D": 5, "fft": 6, "pupil": 7}
PEAK_TYPES = {"finder": 0, "testing": 1, "text": 2, "hdf5": 2}
DPROPS = {"background": 0, "bg_sum": 1, "error": 2, "fg_sum": 3, "height": 4, "sum": 5,
          "x": 6, "xsigma": 7, "y": 8, "ysigma": 9, "z": 10, "jacobian": 11}
IPROPS = {"iterations": 0, "status": 1}
COUNTERS = ["n_dposv", "n_iterations", "n_lost", "n_margin", "n_neg_fi", "n_neg_height",
            "n_non_converged", "n_non_decr"]

_lib = None


def build():
    """Compile liboracle.so with the committed Makefile."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        build()
    lib = ctypes.cdll.LoadLibrary(LIB)
    f64 = ndpointer(dtype=numpy.float64, flags="C_CONTIGUOUS")
    i32 = ndpointer(dtype=numpy.int32, flags="C_CONTIGUOUS")
    i64 = ndpointer(dtype=numpy.int64, flags="C_CONTIGUOUS")
    vp = ctypes.c_void_p
    lib.oraCreate.restype = vp
    lib.oraCreate.argtypes = [ctypes.c_int, f64, f64, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                              ctypes.c_int, ctypes.c_double, ctypes.c_double, f64, f64,
                              ctypes.c_double, ctypes.c_double, f64, ctypes.c_int, ctypes.c_int,
                              ctypes.c_int]
    lib.oraDestroy.argtypes = [vp]
    lib.oraNewImage.argtypes = [vp, f64]
    lib.oraNewBackground.argtypes = [vp, f64]
    lib.oraNewPeaks.argtypes = [vp, f64, ctypes.c_int, ctypes.c_int]
    lib.oraIterate.argtypes = [vp]
    lib.oraDoFit.argtypes = [vp, ctypes.c_int]
    lib.oraDoFit.restype = ctypes.c_int
    for name in ["oraGetUnconverged", "oraGetNError", "oraGetNFit", "oraGetNFitMax",
                 "oraGetJacSize", "oraGetRoiN"]:
        getattr(lib, name).argtypes = [vp]
        getattr(lib, name).restype = ctypes.c_int
    lib.oraGetRoiIndex.argtypes = [vp, i32, i32]
    lib.oraGetOffset.argtypes = [vp, ctypes.c_int]
    lib.oraGetOffset.restype = ctypes.c_double
    lib.oraGetCounters.argtypes = [vp, i64]
    lib.oraGetPeakPropertyDouble.argtypes = [vp, f64, ctypes.c_int]
    lib.oraGetPeakPropertyInt.argtypes = [vp, i32, ctypes.c_int]
    lib.oraGetFitImage.argtypes = [vp, f64]
    lib.oraGetResidual.argtypes = [vp, f64]
    lib.oraSetPeakStatus.argtypes = [vp, i32]
    lib.oraRemoveErrorPeaks.argtypes = [vp]
    lib.oraRemoveRunningPeaks.argtypes = [vp]
    lib.oraSplineEval3D.argtypes = [f64, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int]
    lib.oraSplineEval3D.restype = ctypes.c_double
    lib.oraSolve.argtypes = [f64, f64, ctypes.c_int]
    lib.oraSolve.restype = ctypes.c_int
    lib.oraFFTEval.argtypes = [vp, ctypes.c_double, ctypes.c_double, ctypes.c_double, f64, f64, f64, f64]
    lib.oraPupilEval.argtypes = [vp, ctypes.c_double, ctypes.c_double, ctypes.c_double] + [f64] * 8
    lib.oraSetMinHeight.argtypes = [vp, ctypes.c_double]
    lib.oraMPCreate.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double]
    lib.oraMPCreate.restype = vp
    lib.oraMPDestroy.argtypes = [vp]
    lib.oraMPSetChannel.argtypes = [vp, ctypes.c_int, vp]
    lib.oraMPSetTransforms.argtypes = [vp, f64, f64, f64, f64]
    lib.oraMPSetWeights.argtypes = [vp, f64, f64, f64, f64, f64, ctypes.c_int]
    lib.oraMPSetWeightsIndexing.argtypes = [vp, ctypes.c_double, ctypes.c_double]
    lib.oraMPNewPeaks.argtypes = [vp, f64, ctypes.c_int, ctypes.c_int]
    lib.oraMPIterate.argtypes = [vp]
    lib.oraMPGetUnconverged.argtypes = [vp]
    lib.oraMPGetUnconverged.restype = ctypes.c_int
    _lib = lib
    return lib


def format_peaks(peaks, peaks_type, spline):
    """Column layout of dao_fit_c.py:80-144 (formatPeaksArbitraryPSF / GaussianPSF)."""
    if peaks_type in ("testing", "finder"):
        cols = ["x", "y", "z"] if spline else ["x", "y", "z", "sigma"]
    elif peaks_type in ("text", "hdf5"):
        cols = (["x", "y", "z", "background", "height"] if spline else
                ["x", "y", "z", "background", "height", "xsigma", "ysigma"])
    else:
        raise ValueError("Unknown peaks type '" + peaks_type + "'")
    return numpy.ascontiguousarray(numpy.stack([numpy.asarray(peaks[c], dtype=numpy.float64)
                                                for c in cols], axis=1))


class OracleFitter(object):
    """FP64 CPU fitter with the reference MultiFitter method names."""

    def __init__(self, model, shape, rqe=None, scmos_cal=None, roi_size=10, sigma_range=None,
                 wx_params=None, wy_params=None, min_z=None, max_z=None, spline=None,
                 tol=1.0e-6, psf=None, pupil=None):
        lib = load()
        self.lib = lib
        self.model = model
        self.spline = model.startswith("spline") or model in ("fft", "pupil")
        ny, nx = shape
        self.shape = (ny, nx)
        rqe = numpy.ones(shape) if rqe is None else rqe
        scmos_cal = numpy.zeros(shape) if scmos_cal is None else scmos_cal
        rqe = numpy.ascontiguousarray(rqe, dtype=numpy.float64)
        scmos_cal = numpy.ascontiguousarray(scmos_cal, dtype=numpy.float64)
        wmin = wmax = 0.0
        if sigma_range is not None:
            wmax = 1.0 / (2.0 * sigma_range[0] * sigma_range[0])
            wmin = 1.0 / (2.0 * sigma_range[1] * sigma_range[1])
        wx = numpy.ascontiguousarray(wx_params if wx_params is not None else numpy.zeros(5),
                                     dtype=numpy.float64)
        wy = numpy.ascontiguousarray(wy_params if wy_params is not None else numpy.zeros(5),
                                     dtype=numpy.float64)
        zmin = 0.0 if min_z is None else float(min_z)
        zmax = 0.0 if max_z is None else float(max_z)
        if model == "pupil":
            # pfnInitialize / pfnSetPF inputs: the geometry's kx, ky, kz and
            # the pupil function (pupil = (kx, ky, kz, pf)); the z clamp of
            # pfitSetZRange, open when not given
            kx, ky, kz, pf = pupil
            n = numpy.asarray(kx).shape[0]
            aij = numpy.concatenate([numpy.ascontiguousarray(a, dtype=numpy.float64).ravel()
                                     for a in (kx, ky, numpy.real(kz), numpy.real(pf), numpy.imag(pf))])
            sx, sy, sz = n, n, 0
            zmin = -1.0e300 if min_z is None else float(min_z)
            zmax = 1.0e300 if max_z is None else float(max_z)
        elif model == "fft":
            # the PSF's spectrum as pFTInitialize computes it (oracle/psf_fft.py)
            from . import psf_fft
            psf = numpy.ascontiguousarray(psf, dtype=numpy.float64)
            sz, sy, sx = psf.shape
            spec = psf_fft.PSFFFT(psf).psf_fft
            aij = numpy.ascontiguousarray(numpy.stack([spec.real, spec.imag], axis=-1)).ravel()
        elif self.spline:
            coeff = numpy.ascontiguousarray(spline, dtype=numpy.float64)
            sx, sy = coeff.shape[0], coeff.shape[1]
            sz = coeff.shape[2] if coeff.ndim == 4 else 0
            aij = coeff.ravel()
        else:
            aij = numpy.zeros(1)
            sx = sy = sz = 0
        self.h = lib.oraCreate(MODELS[model], rqe, scmos_cal, tol, nx, ny, roi_size, wmin, wmax,
                               wx, wy, zmin, zmax, numpy.ascontiguousarray(aij), sx, sy, sz)
        self.iterations = 0
        self.psf_shape = None if psf is None else numpy.asarray(psf).shape
        self.pupil_size = None if pupil is None else numpy.asarray(pupil[0]).shape[0]

    def cleanup(self, verbose=False):
        if self.h:
            self.lib.oraDestroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.cleanup()
        except Exception:
            pass

    def newImage(self, image):
        self.lib.oraNewImage(self.h, numpy.ascontiguousarray(image, dtype=numpy.float64))

    def newBackground(self, bg):
        self.lib.oraNewBackground(self.h, numpy.ascontiguousarray(bg, dtype=numpy.float64))

    def newPeaks(self, peaks, peaks_type):
        c = format_peaks(peaks, peaks_type, self.spline)
        self.lib.oraNewPeaks(self.h, c, PEAK_TYPES[peaks_type], c.shape[0])

    def iterate(self):
        self.lib.oraIterate(self.h)

    def doFit(self, max_iterations=2000):
        return self.lib.oraDoFit(self.h, max_iterations)

    def getUnconverged(self):
        return self.lib.oraGetUnconverged(self.h)

    def getNError(self):
        return self.lib.oraGetNError(self.h)

    def getNFit(self):
        return self.lib.oraGetNFit(self.h)

    def getNFitMax(self):
        return self.lib.oraGetNFitMax(self.h)

    def counters(self):
        out = numpy.zeros(8, dtype=numpy.int64)
        self.lib.oraGetCounters(self.h, out)
        return dict(zip(COUNTERS, out.tolist()))

    def roiIndex(self):
        n = self.lib.oraGetRoiN(self.h)
        rx = numpy.zeros(n, dtype=numpy.int32)
        ry = numpy.zeros(n, dtype=numpy.int32)
        self.lib.oraGetRoiIndex(self.h, rx, ry)
        return rx, ry

    def getPeakProperty(self, name):
        n = self.getNFit()
        if name == "significance":
            if n == 0:
                return numpy.zeros(0)
            return self.getPeakProperty("fg_sum") / numpy.sqrt(self.getPeakProperty("bg_sum"))
        if name in IPROPS:
            v = numpy.zeros(n, dtype=numpy.int32)
            self.lib.oraGetPeakPropertyInt(self.h, v, IPROPS[name])
            return v
        if name == "jacobian":
            v = numpy.zeros((n, self.lib.oraGetJacSize(self.h)), dtype=numpy.float64)
            self.lib.oraGetPeakPropertyDouble(self.h, v, DPROPS[name])
            return v
        v = numpy.zeros(n, dtype=numpy.float64)
        self.lib.oraGetPeakPropertyDouble(self.h, v, DPROPS[name])
        return v

    def getFitImage(self):
        out = numpy.zeros(self.shape)
        self.lib.oraGetFitImage(self.h, out)
        return out

    def getResidual(self):
        out = numpy.zeros(self.shape)
        self.lib.oraGetResidual(self.h, out)
        return out

    def setPeakStatus(self, status):
        self.lib.oraSetPeakStatus(self.h, numpy.ascontiguousarray(status, dtype=numpy.int32))

    def removeErrorPeaks(self):
        self.lib.oraRemoveErrorPeaks(self.h)

    def removeRunningPeaks(self):
        self.lib.oraRemoveRunningPeaks(self.h)


def fit_frames(workload, indices, max_iterations=200, props=("x", "y", "z", "height",
                                                               "background", "xsigma", "ysigma",
                                                               "status", "iterations", "error")):
    """Fit frames of a synthetic workload with the oracle; returns a list of property dicts."""
    kw = dict(workload["fitter"])
    model = kw.pop("model")
    spline = kw.pop("spline", None)
    shape = (workload["ny"], workload["nx"])
    fitter = OracleFitter(model, shape, rqe=workload["rqe"], scmos_cal=workload["scmos_cal"],
                          spline=(spline["coeff"] if spline is not None else None), **kw)
    results = []
    for f in indices:
        fitter.newImage(workload["images"][f])
        fitter.newBackground(workload["backgrounds"][f])
        fitter.newPeaks(workload["guesses"][f], "hdf5")
        fitter.doFit(max_iterations)
        results.append({p: fitter.getPeakProperty(p) for p in props})
    fitter.cleanup()
    return results


def pupil_eval(fitter, dx, dy, dz):
    """The pupil model's complex PSF and its x, y, z derivatives on the
    pupil grid (index [u, v], u along the pupil's first index) for a
    translation (dx, dy, dz): oraPupilEval."""
    n = fitter.pupil_size
    out = [numpy.zeros((n, n)) for _ in range(8)]
    fitter.lib.oraPupilEval(fitter.h, dx, dy, dz, *out)
    return [out[2 * i] + 1j * out[2 * i + 1] for i in range(4)]


def fft_eval(fitter, dx, dy, dz):
    """The FFT PSF model's PSF and x, y, z derivatives on the PSF grid for a
    translation, as the oracle's fitter evaluates them."""
    ny, nx = fitter.psf_shape[1], fitter.psf_shape[2]
    out = [numpy.zeros(ny * nx) for _ in range(4)]
    fitter.lib.oraFFTEval(fitter.h, dx, dy, dz, *out)
    return [o.reshape(ny, nx) for o in out]


class OracleMPFitter(object):
    """FP64 CPU multi-plane fitter (multi_plane/mp_fit.c with mp_fit_arb.c or
    mp_fit_dao.c): channels is a list of OracleFitter (one per plane, same
    image size, created with tol * n_channels as the reference's MPFit
    does); transforms = (xt_0toN, yt_0toN, xt_Nto0, yt_Nto0), 3 coefficients
    per channel; weights a dict of (z_size, n_channels) arrays "bg", "h",
    "x", "y", "z" (None: equal weights, z_size 2, offset 0 and scale 0)."""

    def __init__(self, channels, transforms, kind="arb", independent_heights=0, tol=1.0e-6, weights=None,
                 z_offset=0.0, z_scale=0.0):
        self.lib = load()
        self.channels = channels
        self.nc = len(channels)
        self.kind = kind
        self.h = self.lib.oraMPCreate(self.nc, int(independent_heights), 0 if kind == "arb" else 1,
                                      tol * self.nc)
        for c, ch in enumerate(channels):
            self.lib.oraMPSetChannel(self.h, c, ch.h)
        self.lib.oraMPSetTransforms(self.h, *[numpy.ascontiguousarray(t, dtype=numpy.float64) for t in transforms])
        if weights is None:
            w = numpy.ascontiguousarray(numpy.ones((2, self.nc)) / float(self.nc))
            weights = {k: w for k in ("bg", "h", "x", "y", "z")}
        ws = [numpy.ascontiguousarray(weights[k], dtype=numpy.float64) for k in ("bg", "h", "x", "y", "z")]
        self.lib.oraMPSetWeights(self.h, *ws, ws[0].shape[0])
        self.lib.oraMPSetWeightsIndexing(self.h, z_offset, z_scale)

    def newImage(self, images):
        for c, ch in enumerate(self.channels):
            ch.newImage(images[c])

    def newBackground(self, bgs):
        for c, ch in enumerate(self.channels):
            ch.newBackground(bgs[c])

    def newPeaks(self, peaks, peaks_type):
        rows = format_peaks(peaks, peaks_type, self.kind == "arb")
        self.lib.oraMPNewPeaks(self.h, rows, PEAK_TYPES[peaks_type], rows.shape[0])

    def iterate(self):
        self.lib.oraMPIterate(self.h)

    def getUnconverged(self):
        return self.lib.oraMPGetUnconverged(self.h)

    def doFit(self, max_iterations=200):
        """MultiFitter.doFit (sa_library/dao_fit_c.py:332-356)."""
        self.iterate()
        i = 0
        while (self.getUnconverged() > 0) and (i < max_iterations):
            self.iterate()
            i += 1
        return i + 1

    def getPeakProperty(self, name, channel=0):
        return self.channels[channel].getPeakProperty(name)

    def cleanup(self):
        if self.h:
            self.lib.oraMPDestroy(self.h)
            self.h = None
        for ch in self.channels:
            ch.cleanup()
