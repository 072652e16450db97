"""
The reference's FFT PSF fitter class (psf_fft/fft_fit_c.py CFFTFit) over
libsa_cuda.so: ftFitInitialize / ftFitNewPeaks / ftFitCleanup and the
shared mFit* calls.  The FFT PSF model runs in the engine's FP64 path.
"""
import ctypes

from .dao_fit_c import MultiFitterArbitraryPSF, MultiFitterException  # noqa: F401


class CFFTFit(MultiFitterArbitraryPSF):

    def __init__(self, psf_fn=None, **kwds):
        kwds.setdefault("precision", 64)
        super(CFFTFit, self).__init__(**kwds)
        self.psf_fn = psf_fn

    def cleanup(self, spacing="  ", verbose=True):
        super(CFFTFit, self).cleanup(spacing=spacing, verbose=verbose)
        if self.mfit is not None:
            self.clib.ftFitCleanup(self.mfit)
            self.mfit = None

    def getSize(self):
        return self.psf_fn.getSize()

    def initializeC(self, image):
        super(CFFTFit, self).initializeC(image)
        self.mfit = self.clib.ftFitInitialize(self.psf_fn.getCPointer(), self.rqe, self.scmos_cal,
                                              self.default_tol, self.scmos_cal.shape[1],
                                              self.scmos_cal.shape[0])
        self._after_create("ftFitInitialize")

    def newPeaks(self, peaks, peaks_type):
        c_peaks = self.formatPeaks(peaks, peaks_type)
        self._clear_error()
        self.clib.ftFitNewPeaks(self.mfit, c_peaks, ctypes.c_char_p(peaks_type.encode()), c_peaks.shape[0])
        self._check("newPeaks")

    def rescaleZ(self, z):
        return self.psf_fn.rescaleZ(z)
