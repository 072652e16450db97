"""
CPU restatement of the reference's pupil-function PSF model: the pupil
function library (pupilfn/pupil_function.c) that the pupil fitter
(pupilfn/pupil_fit.c) evaluates at every step.

TEST INFRASTRUCTURE ONLY: the checker for the GPU engine's pupil model in
tests/.  Product code never imports this module.

Followed, function by function:

  PupilFunction.__init__   pfnInitialize pupil_function.c:321-363 (kx, ky,
                           kz times 2 pi)
  set_pf                   pfnSetPF :370-410 (divided by the size, negated
                           where i + k is odd, so that the PSF comes out
                           centred)
  translate                pfnTranslate :448-506: x and y multipliers both
                           from kx's first column (cos, -sin of k d), the z
                           multiplier from kz over the pie slice of offsets
                           (a, b) from the centre with -dz, products in the
                           reference's order
  translate_z              pfnTranslateZ :515-556
  get_psf                  pfnGetPSF :80-98: FFTW's unnormalised backward
                           2D transform (numpy's ifft2 times size^2)
  get_psf_dx / dy / dz     pfnGetPSFdx / dy / dz :135-203 (times -i k before
                           the transform; dz negated)
  get_psf_intensity        pfnGetPSFIntensity :108-128
  fit_offsets              pfitInitialize pupil_fit.c:297-299 (xoff, yoff)

The reference's C needs FFTW, which is not installed, so pupil_function.c
cannot be built here.  This restatement is pinned against the reference's
own Python pupil math (simulator/pupil_math.py, which pupil_function.c is
written to match: test/test_pupilfn.py holds the two to numpy.allclose):
tests/golden/g_pupilfn.npz, made by tests/golden/make_golden_pupilfn.py.
"""
import numpy


class PupilFunction(object):
    """kx, ky, kz: (size, size) geometry arrays (simulator/pupil_math.py
    Geometry's kx, ky and the real part of kz); size even."""

    def __init__(self, kx, ky, kz, size):
        assert size % 2 == 0
        self.size = size
        self.kx = 2.0 * numpy.pi * numpy.asarray(kx, dtype=numpy.float64).reshape(size, size)
        self.ky = 2.0 * numpy.pi * numpy.asarray(ky, dtype=numpy.float64).reshape(size, size)
        self.kz = 2.0 * numpy.pi * numpy.asarray(kz, dtype=numpy.float64).reshape(size, size)
        self.pf = numpy.zeros((size, size), dtype=numpy.complex128)
        self.ws = self.pf.copy()

    def set_pf(self, pf):
        n = self.size
        i, k = numpy.mgrid[0:n, 0:n]
        sign = numpy.where((i + k) % 2 == 0, 1.0, -1.0)
        self.pf = numpy.asarray(pf, dtype=numpy.complex128) * sign * (1.0 / float(n))
        self.ws = self.pf.copy()

    def _z_multiplier(self, dz):
        n = self.size
        m = n // 2
        t = numpy.zeros((m + 1, m + 1), dtype=numpy.complex128)
        for i in range(m + 1):
            for j in range(i, m + 1):
                dd = -self.kz[m - i, m - j] * dz
                t[i, j] = numpy.cos(dd) - 1j * numpy.sin(dd)
                t[j, i] = t[i, j]
        a = numpy.abs(numpy.arange(n) - m)
        return t[a[:, None], a[None, :]]

    def translate(self, dx, dy, dz):
        kcol = self.kx[:, 0]
        sx = numpy.cos(kcol * dx) - 1j * numpy.sin(kcol * dx)
        sy = numpy.cos(kcol * dy) - 1j * numpy.sin(kcol * dy)
        self.ws = ((sx[:, None] * sy[None, :]) * self._z_multiplier(dz)) * self.pf

    def translate_z(self, dz):
        self.ws = self._z_multiplier(dz) * self.pf

    def _backward(self, a):
        return numpy.fft.ifft2(a) * float(self.size * self.size)

    def get_psf(self):
        return self._backward(self.ws)

    def get_psf_dx(self):
        return self._backward(-1j * self.kx * self.ws)

    def get_psf_dy(self):
        return self._backward(-1j * self.ky * self.ws)

    def get_psf_dz(self):
        return -self._backward(-1j * self.kz * self.ws)

    def get_psf_intensity(self):
        p = self.get_psf()
        return p.real * p.real + p.imag * p.imag


def fit_offsets(size):
    """(xoff, yoff) of pfitInitialize for a pupil function of this size."""
    return 0.5 * float(size), 0.5 * float(size)
