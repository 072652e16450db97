"""
Spliner fitters backed by the GPU engine.

Class names and methods follow the reference's spliner/cubic_fit_c.py:105-215
(CSplineFit, CSpline2DFit, CSpline3DFit and the ALS/LS/FWLS variants).  The
``spline_fn`` argument is any object with the reference SplineToPSF
interface used by the fitter: getCPointer(), getSize(), rescaleZ(); the
SplinePSF class below provides it from coefficient arrays or from a
reference .spline pickle dict.
"""
import ctypes
import pickle

import numpy

from . import loadclib
from .dao_fit_c import MultiFitterArbitraryPSF, MultiFitterException


class SplinePSF(object):
    """Spline coefficients held by the engine library.

    coeff: (n, n, n, 64) for 3D or (n, n, 16) for 2D, index i*16+j*4+k
    multiplying dx^i dy^j dz^k (spliner/spline3D.py:72-102).  zmin/zmax in nm
    (spliner/spline_to_psf.py:140-210).
    """

    def __init__(self, coeff=None, zmin=-750.0, zmax=750.0, spline_data=None):
        if spline_data is not None:
            if isinstance(spline_data, str):
                with open(spline_data, "rb") as fp:
                    spline_data = pickle.load(fp)
            coeff = spline_data["coeff"]
            zmin = spline_data.get("zmin", zmin)
            zmax = spline_data.get("zmax", zmax)
        self.coeff = numpy.ascontiguousarray(coeff, dtype=numpy.float64)
        self.zmin = float(zmin)
        self.zmax = float(zmax)
        self.is3d = (self.coeff.ndim == 4)
        # spline size in cells (Spline.getSize, spliner/spline1D.py:35-36)
        self.spline_size = self.coeff.shape[0]
        self.clib = loadclib.load(require_device=False)
        self.c_spline = None

    def getCPointer(self):
        """A fresh engine-side spline; the fitter takes ownership (cfCleanup frees it)."""
        if self.is3d:
            return self.clib.initSpline3D(self.coeff.ravel(), self.coeff.shape[0], self.coeff.shape[1],
                                          self.coeff.shape[2])
        return self.clib.initSpline2D(self.coeff.ravel(), self.coeff.shape[0], self.coeff.shape[1])

    def getMargin(self):
        return int(self.getSize() / 2 + 2)

    def getZMin(self):
        return self.zmin

    def getZMax(self):
        return self.zmax

    def isValidZ(self, z):
        """fitting.py:996-1006: strictly inside the spline's z range (nm)."""
        return self.zmin < z < self.zmax

    def _f3d(self, z, y, x):
        """Spline3D.f (spliner/spline3D.py:150-163) for arrays of y, x at
        one z: cell by floor (the last knot belongs to the last cell),
        sum of coeff * dx^i dy^j dz^k; 0 outside [0, cells]."""
        n = self.spline_size

        def cell(v):
            v = numpy.asarray(v, dtype=numpy.float64)
            i = numpy.floor(v).astype(numpy.int64)
            d = v - numpy.floor(v)
            last = v == n
            i = numpy.where(last, n - 1, i)
            d = numpy.where(last, 1.0, d)
            bad = (v < 0.0) | (v > n)
            return numpy.clip(i, 0, n - 1), d, bad

        ix, dx, bx = cell(x)
        iy, dy, by = cell(y)
        iz, dz, bz = cell(numpy.full(numpy.shape(x), z))
        c = self.coeff[ix, iy, iz]                       # (..., 64)
        pw = lambda d: numpy.stack([numpy.ones_like(d), d, d * d, d * d * d], axis=-1)
        px, py, pz = pw(dx), pw(dy), pw(dz)
        mono = px[..., :, None, None] * py[..., None, :, None] * pz[..., None, None, :]
        val = numpy.sum(c * mono.reshape(mono.shape[:-3] + (64,)), axis=-1)
        return numpy.where(bx | by | bz, 0.0, val)

    def getPSF(self, z_value, shape=None, up_sample=1, normalize=True):
        """SplineToPSF3D.getPSF (spliner/spline_to_psf.py:162-200) with
        upsize (:49-73): the spline sampled at pixel centres around the
        middle, drawn into a `shape` array; z in nm."""
        assert isinstance(up_sample, int), "up_sample must be an integer."
        psf_size = up_sample * (self.spline_size - 1)
        off = 0.5 if psf_size % 2 == 0 else 1.0
        grid = numpy.arange(psf_size, dtype=numpy.float64) / float(up_sample) + off
        yy, xx = numpy.meshgrid(grid, grid, indexing="ij")
        if self.is3d:
            psf = self._f3d(self.getScaledZ(z_value), yy, xx)
        else:
            raise NotImplementedError("getPSF for 2D splines")
        if shape is not None:
            im_x, im_y = shape[0] * up_sample, shape[1] * up_sample
            if psf_size % 2 == 0:
                sx, sy = int(im_x / 2 - psf_size / 2), int(im_y / 2 - psf_size / 2)
            else:
                sx, sy = int(im_x / 2 - psf_size / 2) + 1, int(im_y / 2 - psf_size / 2) + 1
            big = numpy.zeros((im_x, im_y))
            big[sx:sx + psf_size, sy:sy + psf_size] = psf
            psf = big
        if normalize:
            psf = psf / numpy.sum(psf)
        return psf

    def getSize(self):
        return self.spline_size

    def getScaledZ(self, z_value):
        """spline_to_psf.py:202-203 (z in nm)."""
        if not self.is3d:
            return z_value * 0.0
        return float(self.spline_size) * (z_value - self.zmin) / (self.zmax - self.zmin)

    def getType(self):
        return "3D" if self.is3d else "2D"

    def rescaleZ(self, z_value):
        """spline_to_psf.py:208-210: spline units -> microns."""
        if not self.is3d:
            return z_value
        return 1.0e-3 * (z_value * (self.zmax - self.zmin) / self.spline_size + self.zmin)

    def cleanup(self):
        pass


class CSplineFit(MultiFitterArbitraryPSF):
    def __init__(self, spline_fn=None, **kwds):
        super(CSplineFit, self).__init__(**kwds)
        self.spline_fn = spline_fn

    def cleanup(self, spacing="  ", verbose=True):
        super(CSplineFit, self).cleanup(spacing=spacing, verbose=verbose)
        if self.mfit is not None:
            self.clib.cfCleanup(self.mfit)
            self.mfit = None
        self.c_spline = None

    def getSize(self):
        return self.spline_fn.getSize()

    def initializeC(self, image):
        super(CSplineFit, self).initializeC(image)
        self.mfit = self.clib.cfInitialize(self.spline_fn.getCPointer(), self.rqe, self.scmos_cal,
                                           self.default_tol, self.scmos_cal.shape[1],
                                           self.scmos_cal.shape[0])
        self._after_create("cfInitialize")

    def newPeaks(self, peaks, peaks_type):
        c_peaks = self.formatPeaks(peaks, peaks_type)
        self._clear_error()
        self.clib.cfNewPeaks(self.mfit, c_peaks, ctypes.c_char_p(peaks_type.encode()), c_peaks.shape[0])
        self._check("newPeaks")


class CSpline2DFit(CSplineFit):
    def initializeC(self, image):
        super(CSpline2DFit, self).initializeC(image)
        self.clib.cfInitialize2D(self.mfit)

    def rescaleZ(self, z):
        return z


class CSpline3DFit(CSplineFit):
    def initializeC(self, image):
        super(CSpline3DFit, self).initializeC(image)
        self.clib.cfInitialize3D(self.mfit)

    def rescaleZ(self, z):
        return self.spline_fn.rescaleZ(z)


class _UnsupportedSpline(CSplineFit):
    def initializeC(self, image):
        raise MultiFitterException(type(self).__name__ + ": only the MLE error model is implemented "
                                   "by the GPU engine")


class CSpline3DFitALS(_UnsupportedSpline):
    pass


class CSpline3DFitLS(_UnsupportedSpline):
    pass


class CSpline3DFitFWLS(_UnsupportedSpline):
    pass
