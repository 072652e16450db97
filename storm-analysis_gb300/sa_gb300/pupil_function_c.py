"""
The reference's pupil-function object (pupilfn/pupil_function_c.py
PupilFunction), backed by libsa_cuda.so's pupil_function.c interface
(pfnInitialize, pfnSetPF, pfnTranslate, pfnTranslateZ, pfnGetPSF*,
pfnSetPNEN and the dipole PSFs, pfnCleanup).  The object's C pointer is
what pupil_fit_c.CPupilFit hands to pfitInitialize.

The getXX functions return complex arrays; the intensity PSF is
psf * conj(psf) (or getPSFIntensity).
"""
import numpy

from . import loadclib


class PupilFunctionException(Exception):
    def __init__(self, message):
        Exception.__init__(self, message)


class PupilFunction(object):
    """geometry: an object with size, kx, ky, kz (pupil_math.Geometry), and
    optionally the six dipole patterns px_ex .. pz_ey."""

    def __init__(self, geometry=None, **kwds):
        super(PupilFunction, self).__init__(**kwds)
        self.size = geometry.size
        if self.size % 2 != 0:
            raise PupilFunctionException("Size must be an even number.")
        self.lib = loadclib.load(require_device=False)
        # kz is complex with a zero imaginary part; only its real part is used
        self.pfn = self.lib.pfnInitialize(numpy.ascontiguousarray(geometry.kx, dtype=numpy.float64),
                                          numpy.ascontiguousarray(geometry.ky, dtype=numpy.float64),
                                          numpy.ascontiguousarray(numpy.real(geometry.kz), dtype=numpy.float64),
                                          self.size)
        if not self.pfn:
            raise PupilFunctionException("pfnInitialize failed for size " + str(self.size))
        if hasattr(geometry, "px_ex"):
            self.lib.pfnSetPNEN(self.pfn, *[numpy.ascontiguousarray(getattr(geometry, a), dtype=numpy.float64)
                                            for a in ("px_ex", "px_ey", "py_ex", "py_ey", "pz_ex", "pz_ey")])

    def cleanup(self):
        if self.pfn:
            self.lib.pfnCleanup(self.pfn)
            self.pfn = None

    def getCPointer(self):
        return self.pfn

    def getXX(self, fn):
        r = numpy.zeros((self.size, self.size), dtype=numpy.float64)
        c = numpy.zeros((self.size, self.size), dtype=numpy.float64)
        fn(self.pfn, r, c)
        return r + 1j * c

    def getPSF(self):
        return self.getXX(self.lib.pfnGetPSF)

    def getPSFIntensity(self):
        psf = numpy.zeros((self.size, self.size), dtype=numpy.float64)
        self.lib.pfnGetPSFIntensity(self.pfn, psf)
        return psf

    def getPSFdx(self):
        return self.getXX(self.lib.pfnGetPSFdx)

    def getPSFdy(self):
        return self.getXX(self.lib.pfnGetPSFdy)

    def getPSFdz(self):
        return self.getXX(self.lib.pfnGetPSFdz)

    def getPXEX(self):
        return self.getXX(self.lib.pfnGetPXEX)

    def getPXEY(self):
        return self.getXX(self.lib.pfnGetPXEY)

    def getPYEX(self):
        return self.getXX(self.lib.pfnGetPYEX)

    def getPYEY(self):
        return self.getXX(self.lib.pfnGetPYEY)

    def getPZEX(self):
        return self.getXX(self.lib.pfnGetPZEX)

    def getPZEY(self):
        return self.getXX(self.lib.pfnGetPZEY)

    def setPF(self, pf):
        self.lib.pfnSetPF(self.pfn, numpy.ascontiguousarray(numpy.real(pf), dtype=numpy.float64),
                          numpy.ascontiguousarray(numpy.imag(pf), dtype=numpy.float64))

    def translate(self, dx, dy, dz):
        """dx, dy in pixels, dz in microns."""
        self.lib.pfnTranslate(self.pfn, dx, dy, dz)

    def translateZ(self, dz):
        self.lib.pfnTranslateZ(self.pfn, dz)
