"""
CPU restatement of the reference's PSF-FFT model: the FFT-translated 3D PSF
(psf_fft/psf_fft.c) and what the FFT PSF fitter takes from it
(psf_fft/fft_fit.c).

TEST INFRASTRUCTURE ONLY: the checker for the GPU engine's PSF-FFT model in
tests/.  Product code never imports this module.

Followed, function by function:

  PSFFFT.__init__     pFTInitialize psf_fft.c:310-365: the r2c 3D transform
                      of psf / (z_size * y_size * x_size), x the fastest axis
  shift_vector        pFTCalcShiftVector psf_fft.c:43-60 (cos / sin of
                      -2 pi dx i / size; index size/2 keeps the positive sin,
                      the second assignment of the reference's loop)
  shift_derivative    pFTCalcShiftVectorDerivative psf_fft.c:70-84
  PSFFFT.translate    pFTTranslate psf_fft.c:372-420 (z shift with -dz, then
                      y, then x, complex products in that order)
  PSFFFT.get_psf      pFTGetPSF psf_fft.c:116-137: the c2r inverse (FFTW's
                      unnormalised backward transform; numpy's irfftn times
                      the number of points: complex inverses along z and y,
                      then c2r along x, the imaginary parts of the x DC and
                      Nyquist bins dropped) and its middle z plane
  PSFFFT.get_psf_dx,  pFTGetPSFdx / dy / dz :147-272: the spectrum times
  _dy, _dz            -i d(k) before the inverse; dz negated
  fit_psf_offsets     ftFitInitialize fft_fit.c:264-284 (xoff, yoff)
  z_range             ftFitZRangeCheck fft_fit.c:506-524

The reference's C needs FFTW, which is not installed, so psf_fft.c cannot
be built here.  This restatement is pinned against the reference's own
pure-Python version (psf_fft/psf_fft_py.py, "a Python version of the C
library for testing purposes") at the tolerance the reference's own test
holds the two to (test/test_psf_fft.py, tests 6-10: 1e-6):
tests/golden/g_psf_fft.npz, made by tests/golden/make_golden_psf_fft.py.
"""
import numpy


def shift_vector(dx, size):
    sr = numpy.empty(size)
    sc = numpy.empty(size)
    sr[0] = 1.0
    sc[0] = 0.0
    t1 = -numpy.pi * 2.0 * dx / float(size)
    for i in range(1, size // 2 + 1):
        t2 = t1 * float(i)
        tr, tc = numpy.cos(t2), numpy.sin(t2)
        sr[size - i] = tr
        sr[i] = tr
        sc[size - i] = -tc
        sc[i] = tc
    return sr + 1j * sc


def shift_derivative(size):
    sc = numpy.empty(size)
    sc[0] = 0.0
    t1 = -numpy.pi * 2.0 / float(size)
    for i in range(1, size // 2 + 1):
        t2 = t1 * float(i)
        sc[size - i] = t2
        sc[i] = -t2
    return sc


class PSFFFT(object):
    """psf: (z_size, y_size, x_size) float64, x the fastest axis."""

    def __init__(self, psf):
        psf = numpy.ascontiguousarray(psf, dtype=numpy.float64)
        self.z_size, self.y_size, self.x_size = psf.shape
        self.n = psf.size
        self.psf_fft = numpy.fft.rfftn(psf / float(self.n))
        self.ws = self.psf_fft.copy()

    def translate(self, dx, dy, dz):
        sx = shift_vector(dx, self.x_size)[: self.x_size // 2 + 1]
        sy = shift_vector(dy, self.y_size)
        sz = shift_vector(-dz, self.z_size)
        ws = self.psf_fft * sz[:, None, None]
        ws = ws * sy[None, :, None]
        self.ws = ws * sx[None, None, :]

    def _mid(self, spectrum):
        real = numpy.fft.irfftn(spectrum, s=(self.z_size, self.y_size, self.x_size), axes=(0, 1, 2)) * float(self.n)
        return real[self.z_size // 2]

    def get_psf(self):
        return self._mid(self.ws)

    def get_psf_dx(self):
        d = shift_derivative(self.x_size)[: self.x_size // 2 + 1]
        return self._mid(self.ws * (-1j) * d[None, None, :])

    def get_psf_dy(self):
        d = shift_derivative(self.y_size)
        return self._mid(self.ws * (-1j) * d[None, :, None])

    def get_psf_dz(self):
        d = shift_derivative(self.z_size)
        return -self._mid(self.ws * (-1j) * d[:, None, None])


def fit_psf_offsets(psf_shape):
    """(xoff, yoff) of ftFitInitialize for a PSF of (z, y, x) shape."""
    return 0.5 * float(psf_shape[2]) - 1.0, 0.5 * float(psf_shape[1]) - 1.0


def z_range(z, z_size):
    max_z = float(z_size) * 0.5 - 1.0e-12
    return min(max(z, -max_z), max_z)


def test_psf(z_size=17, size=20, seed=0):
    """An astigmatic 3D PSF stack on a (z_size, size, size) grid, smooth
    enough that its spectrum vanishes at the Nyquist frequencies, with a
    weak random ripple so that no symmetry hides a transposed axis."""
    rng = numpy.random.default_rng(seed)
    zz = numpy.linspace(-1.0, 1.0, z_size)[:, None, None]
    yy = (numpy.arange(size) - size / 2.0)[None, :, None]
    xx = (numpy.arange(size) - size / 2.0)[None, None, :]
    sx = 1.6 * (1.0 + 0.35 * zz + 0.2 * zz * zz)
    sy = 1.6 * (1.0 - 0.35 * zz + 0.2 * zz * zz)
    psf = numpy.exp(-xx * xx / (2 * sx * sx) - yy * yy / (2 * sy * sy))
    ripple = 1.0 + 0.02 * rng.standard_normal((z_size, 1, 1))
    psf = psf * ripple
    return psf / psf[z_size // 2].sum()
