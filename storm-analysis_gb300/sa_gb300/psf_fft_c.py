"""
The reference's PSF-FFT object (psf_fft/psf_fft_c.py), backed by
libsa_cuda.so's psf_fft.c interface (pFTInitialize, pFTTranslate,
pFTGetPSF, pFTGetPSFdx / dy / dz, pFTCleanup).  The object's C pointer is
what fft_fit_c.CFFTFit hands to ftFitInitialize.
"""
import numpy

from . import loadclib


class PSFFFTException(Exception):
    def __init__(self, message):
        Exception.__init__(self, message)


class PSFFFT(object):
    """psf: (z_size, y_size, x_size) array, x the fastest axis."""

    def __init__(self, psf=None, **kwds):
        super(PSFFFT, self).__init__(**kwds)
        self.psf_shape = psf.shape
        self.lib = loadclib.load(require_device=False)
        c_psf = numpy.ascontiguousarray(psf, dtype=numpy.float64)
        self.pfft = self.lib.pFTInitialize(c_psf, self.psf_shape[0], self.psf_shape[1], self.psf_shape[2])
        if not self.pfft:
            raise PSFFFTException("pFTInitialize failed for a PSF of shape " + str(self.psf_shape))

    def cleanup(self):
        if self.pfft:
            self.lib.pFTCleanup(self.pfft)
            self.pfft = None

    def getCPointer(self):
        return self.pfft

    def _plane(self, fn):
        out = numpy.zeros((self.psf_shape[1], self.psf_shape[2]), dtype=numpy.float64)
        fn(self.pfft, out)
        return out

    def getPSF(self):
        return self._plane(self.lib.pFTGetPSF)

    def getPSFdx(self):
        return self._plane(self.lib.pFTGetPSFdx)

    def getPSFdy(self):
        return self._plane(self.lib.pFTGetPSFdy)

    def getPSFdz(self):
        return self._plane(self.lib.pFTGetPSFdz)

    def translate(self, dx, dy, dz):
        """As the reference: dz in z pixel units, dx and dy reversed with
        respect to simulator.pupil_math."""
        self.lib.pFTTranslate(self.pfft, dx, dy, dz)


class PSFFnBase(object):
    """The PSF object of the reference's FFT PSF analysis (psf_fft/psf_fn.py
    PSFFnBase): psf_data is a dict of 'psf' (z, y, x; odd z size, square in
    x / y), 'pixel_size' and the z range 'zmin' / 'zmax' in nanometers
    (symmetric).  z in the fit is in z pixel units around the middle plane."""

    def __init__(self, psf_data=None, **kwds):
        super(PSFFnBase, self).__init__(**kwds)
        psf = numpy.ascontiguousarray(psf_data["psf"], dtype=numpy.float64)
        if psf.shape[0] % 2 != 1:
            raise PSFFFTException("Z size must be an odd number.")
        if psf.shape[1] != psf.shape[2]:
            raise PSFFFTException("X/Y size must be the same.")
        if psf_data["zmax"] != -psf_data["zmin"]:
            raise PSFFFTException("z range must be symmetric.")
        self.psf_fft_c = PSFFFT(psf)
        self.pixel_size = psf_data["pixel_size"]
        self.psf_shape = psf.shape
        self.zmax = psf_data["zmax"]
        self.zmin = psf_data["zmin"]
        nz1 = float(psf.shape[0]) - 1.0
        self.scale_gSZ = nz1 / (self.zmax - self.zmin)              # nm -> z pixels
        self.scale_rZ = 1.0e-3 * (self.zmax - self.zmin) / nz1      # z pixels -> um

    def cleanup(self):
        self.psf_fft_c.cleanup()

    def getCPointer(self):
        return self.psf_fft_c.getCPointer()

    def getMargin(self):
        return int((self.getSize() + 1) / 2 + 2)

    def getPixelSize(self):
        return self.pixel_size

    def getPSF(self, z_value, shape=None, normalize=False):
        """The PSF at z_value (nanometers), shifted by one pixel in x / y as
        the reference's (to line up with Spliner's PSF)."""
        self.psf_fft_c.translate(1.0, 1.0, self.getScaledZ(z_value))
        psf = self.psf_fft_c.getPSF()
        if shape is not None:
            n = psf.shape[0]
            sx, sy = int(shape[0] / 2.0 - n / 2.0), int(shape[1] / 2.0 - n / 2.0)
            big = numpy.zeros((shape[0], shape[1]))
            big[sx:sx + n, sy:sy + n] = psf
            psf = big
        if normalize:
            psf = psf / numpy.sum(psf)
        return psf

    def getScaledZ(self, z_value):
        return z_value * self.scale_gSZ

    def getSize(self):
        return self.psf_shape[1]

    def getZSize(self):
        return self.psf_shape[0]

    def rescaleZ(self, z_value):
        return z_value * self.scale_rZ


class PSFFn(PSFFnBase):
    """psf_fn.py PSFFn: the PSF data from a pickle file."""

    def __init__(self, psf_filename=None, **kwds):
        import pickle
        with open(psf_filename, "rb") as fp:
            psf_data = pickle.load(fp)
        super(PSFFn, self).__init__(psf_data=psf_data, **kwds)
