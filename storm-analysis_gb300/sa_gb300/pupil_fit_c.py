"""
The reference's pupil-function fitter class (pupilfn/pupil_fit_c.py
CPupilFit) over libsa_cuda.so: pfitInitialize / pfitSetZRange /
pfitNewPeaks / pfitCleanup and the shared mFit* calls.  The pupil model
runs in the engine's FP64 path.

As the reference, initializeC passes the pupil function object's
getZMin() / getZMax() to pfitSetZRange unchanged (pupil_fit_c.py:115-117).
"""
import ctypes

from .dao_fit_c import MultiFitterArbitraryPSF, MultiFitterException  # noqa: F401


class CPupilFit(MultiFitterArbitraryPSF):

    def __init__(self, pupil_fn=None, **kwds):
        kwds.setdefault("precision", 64)
        super(CPupilFit, self).__init__(**kwds)
        self.pupil_fn = pupil_fn

    def cleanup(self, spacing="  ", verbose=True):
        super(CPupilFit, self).cleanup(spacing=spacing, verbose=verbose)
        if self.mfit is not None:
            self.clib.pfitCleanup(self.mfit)
            self.mfit = None
        self.pupil_fn = None

    def getSize(self):
        return self.pupil_fn.getSize()

    def initializeC(self, image):
        super(CPupilFit, self).initializeC(image)
        self.mfit = self.clib.pfitInitialize(self.pupil_fn.getCPointer(), self.rqe, self.scmos_cal,
                                             self.default_tol, self.scmos_cal.shape[1], self.scmos_cal.shape[0])
        self._after_create("pfitInitialize")
        self.clib.pfitSetZRange(self.mfit, self.pupil_fn.getZMin(), self.pupil_fn.getZMax())

    def newPeaks(self, peaks, peaks_type):
        c_peaks = self.formatPeaks(peaks, peaks_type)
        self._clear_error()
        self.clib.pfitNewPeaks(self.mfit, c_peaks, ctypes.c_char_p(peaks_type.encode()), c_peaks.shape[0])
        self._check("newPeaks")
