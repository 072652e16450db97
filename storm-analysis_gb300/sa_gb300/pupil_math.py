"""
The pupil-function geometry the pupil model is built on: the translation
multipliers kx, ky, kz of a square pupil of `size` samples and the pupil
functions the reference's pupil-function files hold, with the conventions
of the reference's simulator/pupil_math.py (Geometry, GeometrySim,
createPlaneWave, applyNARestriction, changeFocus, translatePf, dx,
toRealSpace, intensity), which pupilfn/pupil_function.c is written to match.

Units are microns.  For a pupil of size N sampled at pixel size p:
  dk      = 1 / (N p)                       the frequency step
  x, y    = -N/2 .. N/2 - 1 along the first / second index
  kx, ky  = x / N, y / N                    translation multipliers (pixels)
  k       = dk sqrt(x^2 + y^2)
  kz      = sqrt((n / wavelength)^2 - k^2)  inside the NA (k <= NA / wavelength),
            0 outside                       the defocus multiplier
"""
import math

import numpy


class PupilMathException(Exception):
    pass


class Geometry(object):
    """size: pupil samples (even); pixel_size, wavelength in microns; imm_index:
    the immersion medium's index (larger than NA); NA: the objective's."""

    def __init__(self, size, pixel_size, wavelength, imm_index, NA):
        if size % 2 != 0:
            raise PupilMathException("PF size must be a multiple of 2!")
        if imm_index <= NA:
            raise PupilMathException("Immersion media index must be larger than objective NA!")
        self.size = int(size)
        self.pixel_size = float(pixel_size)
        self.wavelength = float(wavelength)
        self.imm_index = float(imm_index)
        self.NA = float(NA)
        self.k_max = self.NA / self.wavelength
        dk = 1.0 / (self.size * self.pixel_size)
        self.r_max = self.k_max / dk
        half = self.size / 2.0
        x, y = numpy.mgrid[-half:half, -half:half]
        self.kx = x / self.size
        self.ky = y / self.size
        kxp, kyp = dk * x, dk * y
        self.k = numpy.sqrt(kxp * kxp + kyp * kyp)
        t = self.imm_index / self.wavelength
        self.kz = numpy.sqrt((t * t - self.k * self.k).astype(numpy.complex128))
        self.r = self.k / self.k_max
        self.kz[self.r > 1.0] = 0.0
        self.n_pixels = int(numpy.sum(self.r <= 1))
        self.norm = math.sqrt(self.r.size)

    def applyNARestriction(self, pupil_fn):
        pupil_fn[self.r > 1.0] = 0.0
        return pupil_fn

    def changeFocus(self, pupil_fn, z_dist):
        return numpy.exp(1j * 2.0 * numpy.pi * self.kz * z_dist) * pupil_fn

    def createPlaneWave(self, n_photons):
        plane = numpy.sqrt(n_photons / self.n_pixels) * numpy.exp(1j * numpy.zeros(self.r.shape))
        return self.applyNARestriction(plane)

    def createFromPhase(self, n_photons, phase):
        """A pupil function of uniform amplitude and the given phase
        (radians, size x size) inside the NA."""
        pf = numpy.sqrt(n_photons / self.n_pixels) * numpy.exp(1j * numpy.asarray(phase))
        return self.applyNARestriction(pf)

    def dx(self, pupil_fn):
        return -1j * 2.0 * numpy.pi * self.kx * pupil_fn

    def translatePf(self, pupil_fn, dx, dy):
        return numpy.exp(-1j * 2.0 * numpy.pi * (self.kx * dx + self.ky * dy)) * pupil_fn


class GeometrySim(Geometry):
    """The simulations' geometry: half the camera pixel size (a more
    realistic PSF width without OTF scaling)."""

    def __init__(self, size, pixel_size, wavelength, imm_index, NA):
        super(GeometrySim, self).__init__(size, 0.5 * pixel_size, wavelength, imm_index, NA)


def intensity(x):
    return numpy.abs(x * numpy.conj(x))


def toRealSpace(pupil_fn):
    """The pupil function in real space: the inverse 2D DFT times the square
    root of the number of samples, centred."""
    return numpy.fft.ifftshift(math.sqrt(pupil_fn.size) * numpy.fft.ifft2(pupil_fn))
