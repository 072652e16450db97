"""
Batched multi-frame fitting: many frames of one size and model in one
frame set on the GPU, all fitted by the same device-driven sweep loop.

    fitter = BatchFitter("3d", (512, 512), n_frames=64, roi_size=18,
                         sigma_range=[0.5, 4.0])
    fitter.load(images, backgrounds, peaks_per_frame, "hdf5")
    fitter.fit(max_iterations=200)
    res = fitter.results()          # dict of per-peak arrays + "frame"

Per frame the result is the reference's MultiFitter result for the same
frame (sa_library/dao_fit_c.py): peaks of different frames never interact,
and within a frame the engine keeps the reference's peak order.
"""
import ctypes

import numpy

from . import loadclib
from .dao_fit_c import MultiFitterException, formatPeaksArbitraryPSF, formatPeaksGaussianPSF

MODEL_INIT = {"2dfixed", "2d", "3d", "Z", "spline2D", "spline3D", "fft", "pupil"}

RESULT_PROPS = ("x", "y", "z", "height", "background", "xsigma", "ysigma", "error")


class BatchFitter(object):
    def __init__(self, model, shape, n_frames, roi_size=10, sigma_range=None, rqe=None,
                 scmos_cal=None, wx_params=None, wy_params=None, min_z=None, max_z=None,
                 spline=None, precision=32, peaks_capacity=None, tol=1.0e-6, dilation=None,
                 stream=None, psf_fft=None, pupil_fn=None):
        if model not in MODEL_INIT:
            raise MultiFitterException("unknown model '%s'" % model)
        self.clib = loadclib.load()
        self.model = model
        self.shape = tuple(shape)
        self.n_frames = int(n_frames)
        ny, nx = self.shape
        rqe = numpy.ones(self.shape) if rqe is None else rqe
        scmos_cal = numpy.zeros(self.shape) if scmos_cal is None else scmos_cal
        self.rqe = numpy.ascontiguousarray(rqe, dtype=numpy.float64)
        self.scmos_cal = numpy.ascontiguousarray(scmos_cal, dtype=numpy.float64)
        self.spline = spline
        lib = self.clib
        self.psf_fft = psf_fft
        self.pupil_fn = pupil_fn
        if model.startswith("spline"):
            sp = spline.getCPointer()
            self.h = lib.cfInitialize(sp, self.rqe, self.scmos_cal, tol, nx, ny)
        elif model == "fft":
            # psf_fft: a psf_fft_c.PSFFFT (or anything with getCPointer()); the
            # FFT PSF model runs in the FP64 engine
            self.h = lib.ftFitInitialize(psf_fft.getCPointer(), self.rqe, self.scmos_cal, tol, nx, ny)
        elif model == "pupil":
            # pupil_fn: a pupil_fn.PupilFunction (getCPointer(), getZMin(),
            # getZMax()); the pupil model runs in the FP64 engine
            self.h = lib.pfitInitialize(pupil_fn.getCPointer(), self.rqe, self.scmos_cal, tol, nx, ny)
            if self.h:
                lib.pfitSetZRange(self.h, pupil_fn.getZMin(), pupil_fn.getZMax())
        else:
            self.h = lib.daoInitialize(self.rqe, self.scmos_cal, tol, nx, ny, roi_size)
        if not self.h:
            raise MultiFitterException(loadclib.last_error())
        if lib.saSetPrecision(self.h, int(precision)) != 0:
            raise MultiFitterException(loadclib.last_error())
        if dilation is not None and lib.saSetDilation(self.h, int(dilation)) != 0:
            raise MultiFitterException(loadclib.last_error())
        if stream is not None:
            lib.saSetStream(self.h, ctypes.c_void_p(stream))
        if model in ("2d", "3d"):
            wmax = 1.0 / (2.0 * sigma_range[0] * sigma_range[0])
            wmin = 1.0 / (2.0 * sigma_range[1] * sigma_range[1])
            (lib.daoInitialize2D if model == "2d" else lib.daoInitialize3D)(self.h, wmin, wmax)
        elif model == "2dfixed":
            lib.daoInitialize2DFixed(self.h)
        elif model == "Z":
            lib.daoInitializeZ(self.h, numpy.ascontiguousarray(wx_params, dtype=numpy.float64),
                               numpy.ascontiguousarray(wy_params, dtype=numpy.float64),
                               float(min_z), float(max_z))
        elif model == "spline3D":
            lib.cfInitialize3D(self.h)
        elif model == "spline2D":
            lib.cfInitialize2D(self.h)
        self.capacity = None
        self._framed = False
        self.sweeps = 0
        if peaks_capacity:
            self.ensure_frames(int(peaks_capacity))

    def _ok(self, r, what):
        if r < 0:
            raise MultiFitterException(what + ": " + loadclib.last_error())
        return r

    def ensure_frames(self, capacity):
        if not self._framed or capacity > (self.capacity or 0):
            self.capacity = max(int(capacity), self.capacity or 0)
            self._ok(self.clib.saSetFrames(self.h, self.n_frames, self.capacity), "saSetFrames")
            self._framed = True

    def format(self, peaks, peaks_type):
        if self.model.startswith("spline") or self.model in ("fft", "pupil"):
            return formatPeaksArbitraryPSF(peaks, peaks_type)
        return formatPeaksGaussianPSF(peaks, peaks_type)

    def load_images(self, images, on_device=False, dtype_bits=None):
        """images: (F, ny, nx) host numpy array, or a device pointer (int) when on_device."""
        if on_device:
            return self._ok(self.clib.saNewImages(self.h, ctypes.c_void_p(images), self.n_frames,
                                                  dtype_bits, 1), "saNewImages")
        a = numpy.ascontiguousarray(images)
        bits = {numpy.dtype(numpy.float64): 64, numpy.dtype(numpy.float32): 32,
                numpy.dtype(numpy.uint16): 16}[a.dtype]
        return self._ok(self.clib.saNewImages(self.h, a.ctypes.data_as(ctypes.c_void_p), self.n_frames,
                                              bits, 0), "saNewImages")

    def load_backgrounds(self, bgs, on_device=False, dtype_bits=None):
        if on_device:
            return self._ok(self.clib.saNewBackgrounds(self.h, ctypes.c_void_p(bgs), self.n_frames,
                                                       dtype_bits, 1), "saNewBackgrounds")
        a = numpy.ascontiguousarray(bgs)
        bits = 64 if a.dtype == numpy.float64 else 32
        if a.dtype not in (numpy.float64, numpy.float32):
            a = a.astype(numpy.float64)
            bits = 64
        return self._ok(self.clib.saNewBackgrounds(self.h, a.ctypes.data_as(ctypes.c_void_p),
                                                   self.n_frames, bits, 0), "saNewBackgrounds")

    def load_peaks(self, peaks_per_frame, peaks_type):
        rows = [self.format(p, peaks_type) for p in peaks_per_frame]
        counts = numpy.array([r.shape[0] for r in rows], dtype=numpy.int32)
        self.ensure_frames(int(counts.max()) if counts.size else 1)
        allrows = numpy.ascontiguousarray(numpy.concatenate(rows, axis=0), dtype=numpy.float64)
        return self._ok(self.clib.saNewPeaksBatch(self.h, allrows, counts, self.n_frames,
                                                  ctypes.c_char_p(peaks_type.encode())), "saNewPeaksBatch")

    def load_peaks_device(self, d_rows, counts, peaks_type):
        """Peak rows already on the device (pointer), counts per frame (host)."""
        counts = numpy.ascontiguousarray(counts, dtype=numpy.int32)
        self.ensure_frames(int(counts.max()) if counts.size else 1)
        return self._ok(self.clib.saNewPeaksBatchDevice(self.h, ctypes.c_void_p(d_rows), counts,
                                                        self.n_frames,
                                                        ctypes.c_char_p(peaks_type.encode())),
                        "saNewPeaksBatchDevice")

    def reset(self):
        """Start over: the next load re-creates the frame set, dropping every
        frame's peaks (as mFitNewImage starts a frame empty)."""
        self._framed = False
        self.capacity = None

    def reserve(self, capacity_per_frame):
        """Grow each frame's peak storage, keeping its peaks."""
        if not self._framed:
            return self.ensure_frames(capacity_per_frame)
        if capacity_per_frame > (self.capacity or 0):
            self._ok(self.clib.saReservePeaksBatch(self.h, int(capacity_per_frame)), "saReservePeaksBatch")
            self.capacity = int(capacity_per_frame)

    def fit_frames(self, active, max_iterations=2000):
        """Fit only the frames with active[f] true."""
        a = numpy.ascontiguousarray(numpy.asarray(active, dtype=numpy.int32))
        return self._ok(self.clib.saDoFitBatchFrames(self.h, int(max_iterations), a), "saDoFitBatchFrames")

    def set_status(self, status):
        """Statuses of all frames' peaks (frames in order), as mFitSetPeakStatus."""
        st = numpy.ascontiguousarray(status, dtype=numpy.int32)
        return self._ok(self.clib.saSetPeakStatusBatch(self.h, st), "saSetPeakStatusBatch")

    def remove(self, status):
        """Drop every frame's peaks with this status (2 ERROR, 0 RUNNING)."""
        return self._ok(self.clib.saRemovePeaksBatch(self.h, int(status)), "saRemovePeaksBatch")

    def fit_images_device(self, d_out, residual=False):
        """Every frame's fit image into device memory d_out (address)."""
        return self._ok(self.clib.saGetFitImagesDevice(self.h, ctypes.c_void_p(d_out), 1 if residual else 0),
                        "saGetFitImagesDevice")

    def results_fast(self):
        """All results with one device-to-host copy: (values[n, 8], ints[n, 2]) with
        columns x, y, z, height, background, xsigma, ysigma, error / status, iterations."""
        n = int(self.counts().sum())
        vals = numpy.zeros((n, 8), dtype=numpy.float64)
        ints = numpy.zeros((n, 2), dtype=numpy.int32)
        if n:
            self._ok(self.clib.saGetResultsBatch(self.h, vals, ints), "saGetResultsBatch")
        return vals, ints

    def sweep_times(self, max_n=100000):
        """Per-launch sweep kernel times (ms) recorded while timing was on."""
        out = numpy.zeros(max_n, dtype=numpy.float32)
        n = self.clib.saGetSweepTimes(self.h, out, max_n)
        return out[:max(n, 0)]

    def kernel_launches(self):
        return int(self.clib.saGetKernelLaunches(self.h))

    def load(self, images, backgrounds, peaks_per_frame, peaks_type="hdf5"):
        counts = max(len(self.format(p, peaks_type)) for p in peaks_per_frame)
        self.ensure_frames(counts)
        self.load_images(images)
        self.load_backgrounds(backgrounds)
        self.load_peaks(peaks_per_frame, peaks_type)

    def fit(self, max_iterations=2000):
        self.sweeps = self._ok(self.clib.saDoFitBatch(self.h, int(max_iterations)), "saDoFitBatch")
        return self.sweeps

    def counts(self):
        c = numpy.zeros(self.n_frames, dtype=numpy.int32)
        self.clib.saGetNFitBatch(self.h, c)
        return c

    def prop(self, name):
        n = int(self.counts().sum())
        if name in ("status", "iterations"):
            v = numpy.zeros(n, dtype=numpy.int32)
            self._ok(self.clib.saGetPeakPropertyIntBatch(self.h, v, ctypes.c_char_p(name.encode())), name)
            return v
        v = numpy.zeros(n, dtype=numpy.float64)
        self._ok(self.clib.saGetPeakPropertyBatch(self.h, v, ctypes.c_char_p(name.encode())), name)
        return v

    def results(self, props=RESULT_PROPS):
        out = {p: self.prop(p) for p in props}
        out["status"] = self.prop("status")
        out["iterations"] = self.prop("iterations")
        out["frame"] = numpy.repeat(numpy.arange(self.n_frames), self.counts())
        return out

    def counters(self):
        out = numpy.zeros(9, dtype=numpy.int64)
        self.clib.saGetCounters(self.h, out)
        return out

    def sched_stats(self):
        out = numpy.zeros(2, dtype=numpy.int64)
        self.clib.saGetSchedStats(self.h, out)
        return {"reruns": int(out[0]), "barriers": int(out[1])}

    def set_timing(self, on):
        self.clib.saSetTiming(self.h, 1 if on else 0)

    def timing(self):
        ms = ctypes.c_double()
        n = ctypes.c_int64()
        t = ctypes.c_int64()
        self.clib.saGetTiming(self.h, ctypes.byref(ms), ctypes.byref(n), ctypes.byref(t))
        return ms.value, n.value, t.value

    def close(self):
        if self.h:
            if self.model.startswith("spline"):
                self.clib.cfCleanup(self.h)
            elif self.model == "fft":
                self.clib.ftFitCleanup(self.h)
            elif self.model == "pupil":
                self.clib.pfitCleanup(self.h)
            else:
                self.clib.daoCleanup(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
