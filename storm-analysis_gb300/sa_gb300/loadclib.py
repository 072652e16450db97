"""
Load libsa_cuda.so, the GPU fitting engine, and declare its C ABI
(include/sa_cuda.h).

This is the only way the package reaches the engine.  There is no CPU
fallback: a missing library or a machine without a CUDA device raises.
"""
import ctypes
import os

import numpy
from numpy.ctypeslib import ndpointer

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsa_cuda.so")

_lib = None


class EngineUnavailable(RuntimeError):
    pass


class saMPFit(ctypes.Structure):
    pass


class saFitData(ctypes.Structure):
    """The handle's leading fields, laid out as the reference's fitData."""
    _fields_ = ([(n, ctypes.c_int) for n in
                 ["n_dposv", "n_iterations", "n_lost", "n_margin", "n_neg_fi", "n_neg_height",
                  "n_non_converged", "n_non_decr", "fit_size_x", "fit_size_y", "image_size_x",
                  "image_size_y", "jac_size", "max_nfit", "nfit", "roi_n_index"]] +
                [(n, ctypes.c_double) for n in ["minimum_height", "xoff", "yoff", "zoff", "tolerance"]] +
                [("bg_counts", ctypes.POINTER(ctypes.c_int)),
                 ("roi_x_index", ctypes.POINTER(ctypes.c_int)),
                 ("roi_y_index", ctypes.POINTER(ctypes.c_int)),
                 ("stale", ctypes.POINTER(ctypes.c_int))] +
                [(n, ctypes.POINTER(ctypes.c_double)) for n in
                 ["as_xi", "bg_data", "bg_estimate", "err_i", "f_data", "rqe", "scmos_term", "t_fi",
                  "x_data"]] +
                [("working_peak", ctypes.c_void_p), ("fit", ctypes.c_void_p), ("fit_model", ctypes.c_void_p),
                 ("fn_reserved", ctypes.c_void_p * 9), ("engine", ctypes.c_void_p)])


# The multi-plane handle's leading fields, laid out as the reference's mpFit
# (multi_plane/mp_fit.h:12-44; mp_fit_c.py mirrors them as mpFitData).
saMPFit._fields_ = ([(n, ctypes.c_int) for n in ["im_size_x", "im_size_y", "independent_heights", "n_channels",
                                                  "n_weights"]] +
                    [(n, ctypes.c_double) for n in ["tolerance", "w_z_offset", "w_z_scale", "zmin", "zmax"]] +
                    [(n, ctypes.POINTER(ctypes.c_double)) for n in ["xt_0toN", "yt_0toN", "xt_Nto0", "yt_Nto0",
                                                                     "w_bg", "w_h", "w_x", "w_y", "w_z", "heights"]] +
                    [(n, ctypes.c_void_p) for n in ["jacobian", "w_jacobian", "hessian", "w_hessian"]] +
                    [("fit_data", ctypes.POINTER(ctypes.POINTER(saFitData)))] +
                    [(n, ctypes.c_void_p) for n in ["fn_cleanup", "fn_newpeaks", "fn_peak_xi_yi", "fn_update",
                                                     "fn_zrange", "engine"]])


def last_error():
    lib = load(require_device=False)
    buf = ctypes.create_string_buffer(1024)
    lib.saGetLastError(buf, 1024)
    return buf.value.decode(errors="replace")


def load(require_device=True):
    """Return the loaded library (declaring argument types once)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise EngineUnavailable("libsa_cuda.so is not built; run "
                                    "'python -c \"import __graft_entry__ as g; g.build()\"'")
        lib = ctypes.cdll.LoadLibrary(LIB_PATH)
        _declare(lib)
        _lib = lib
    if require_device and _lib.saDeviceCount() < 1:
        raise EngineUnavailable("no CUDA device is visible; the GPU engine cannot run")
    return _lib


def _declare(lib):
    f64 = ndpointer(dtype=numpy.float64, flags="C_CONTIGUOUS")
    i32 = ndpointer(dtype=numpy.int32, flags="C_CONTIGUOUS")
    i64 = ndpointer(dtype=numpy.int64, flags="C_CONTIGUOUS")
    vp = ctypes.c_void_p
    hp = ctypes.POINTER(saFitData)
    ci, cd, cs = ctypes.c_int, ctypes.c_double, ctypes.c_char_p

    lib.daoInitialize.argtypes = [f64, f64, cd, ci, ci, ci]
    lib.daoInitialize.restype = hp
    lib.cfInitialize.argtypes = [vp, f64, f64, cd, ci, ci]
    lib.cfInitialize.restype = hp
    for name in ["daoInitialize2DFixed", "daoInitialize2DFixedALS", "daoInitialize2DFixedLS",
                 "daoInitialize2DFixedDWLS", "daoInitialize2DFixedFWLS", "cfInitialize2D",
                 "cfInitialize3D", "cfInitialize3DALS", "cfInitialize3DLS", "cfInitialize3DFWLS",
                 "daoCleanup", "cfCleanup", "mFitIterateLM", "mFitRemoveErrorPeaks",
                 "mFitRemoveRunningPeaks", "mFitAnscombeTransformImage"]:
        getattr(lib, name).argtypes = [hp]
        getattr(lib, name).restype = None
    for name in ["daoInitialize2D", "daoInitialize2DALS", "daoInitialize2DLS", "daoInitialize2DDWLS",
                 "daoInitialize2DFWLS", "daoInitialize3D"]:
        getattr(lib, name).argtypes = [hp, cd, cd]
        getattr(lib, name).restype = None
    lib.daoInitializeZ.argtypes = [hp, f64, f64, cd, cd]
    lib.daoInitializeZ.restype = None
    lib.daoNewPeaks.argtypes = [hp, f64, cs, ci]
    lib.daoNewPeaks.restype = None
    lib.cfNewPeaks.argtypes = [hp, f64, cs, ci]
    lib.cfNewPeaks.restype = None
    lib.initSpline2D.argtypes = [f64, ci, ci]
    lib.initSpline2D.restype = vp
    lib.initSpline3D.argtypes = [f64, ci, ci, ci]
    lib.initSpline3D.restype = vp
    lib.splineCleanup.argtypes = [vp]
    # the FFT PSF model (psf_fft.c / fft_fit.c names)
    lib.pFTInitialize.argtypes = [f64, ci, ci, ci]
    lib.pFTInitialize.restype = vp
    lib.pFTCleanup.argtypes = [vp]
    lib.pFTCleanup.restype = None
    lib.pFTTranslate.argtypes = [vp, cd, cd, cd]
    lib.pFTTranslate.restype = None
    for name in ["pFTGetPSF", "pFTGetPSFdx", "pFTGetPSFdy", "pFTGetPSFdz"]:
        getattr(lib, name).argtypes = [vp, f64]
        getattr(lib, name).restype = None
    for name in ["pFTGetXSize", "pFTGetYSize", "pFTGetZSize"]:
        getattr(lib, name).argtypes = [vp]
        getattr(lib, name).restype = ci
    lib.ftFitInitialize.argtypes = [vp, f64, f64, cd, ci, ci]
    lib.ftFitInitialize.restype = hp
    lib.ftFitNewPeaks.argtypes = [hp, f64, cs, ci]
    lib.ftFitNewPeaks.restype = None
    lib.ftFitCleanup.argtypes = [hp]
    lib.ftFitCleanup.restype = None
    # the pupil-function model (pupil_function.c / pupil_fit.c names)
    lib.pfnInitialize.argtypes = [f64, f64, f64, ci]
    lib.pfnInitialize.restype = vp
    lib.pfnCleanup.argtypes = [vp]
    lib.pfnCleanup.restype = None
    lib.pfnSetPF.argtypes = [vp, f64, f64]
    lib.pfnSetPF.restype = None
    lib.pfnSetPNEN.argtypes = [vp, f64, f64, f64, f64, f64, f64]
    lib.pfnSetPNEN.restype = None
    lib.pfnTranslate.argtypes = [vp, cd, cd, cd]
    lib.pfnTranslate.restype = None
    lib.pfnTranslateZ.argtypes = [vp, cd]
    lib.pfnTranslateZ.restype = None
    for name in ["pfnGetPSF", "pfnGetPSFdx", "pfnGetPSFdy", "pfnGetPSFdz", "pfnGetPXEX", "pfnGetPXEY",
                 "pfnGetPYEX", "pfnGetPYEY", "pfnGetPZEX", "pfnGetPZEY"]:
        getattr(lib, name).argtypes = [vp, f64, f64]
        getattr(lib, name).restype = None
    lib.pfnGetPSFIntensity.argtypes = [vp, f64]
    lib.pfnGetPSFIntensity.restype = None
    lib.pfnGetSize.argtypes = [vp]
    lib.pfnGetSize.restype = ci
    lib.pfitInitialize.argtypes = [vp, f64, f64, cd, ci, ci]
    lib.pfitInitialize.restype = hp
    lib.pfitNewPeaks.argtypes = [hp, f64, cs, ci]
    lib.pfitNewPeaks.restype = None
    lib.pfitSetZRange.argtypes = [hp, cd, cd]
    lib.pfitSetZRange.restype = None
    lib.pfitCleanup.argtypes = [hp]
    lib.pfitCleanup.restype = None
    # multi-plane fitting (mp_fit.c / mp_fit_arb.c / mp_fit_dao.c names)
    mpp = ctypes.POINTER(saMPFit)
    lib.mpInitialize.argtypes = [cd, ci, ci, ci, ci]
    lib.mpInitialize.restype = mpp
    lib.mpCleanup.argtypes = [mpp]
    lib.mpCleanup.restype = None
    lib.mpIterateLM.argtypes = [mpp]
    lib.mpIterateLM.restype = None
    lib.mpSetTransforms.argtypes = [mpp, f64, f64, f64, f64]
    lib.mpSetTransforms.restype = None
    lib.mpSetWeights.argtypes = [mpp, f64, f64, f64, f64, f64, ci]
    lib.mpSetWeights.restype = None
    lib.mpSetWeightsIndexing.argtypes = [mpp, cd, cd]
    lib.mpSetWeightsIndexing.restype = None
    lib.mpArbInitializePSFFFTChannel.argtypes = [mpp, vp, f64, f64, ci]
    lib.mpArbInitializePSFFFTChannel.restype = None
    lib.mpArbInitializePupilFnChannel.argtypes = [mpp, vp, f64, f64, cd, cd, ci]
    lib.mpArbInitializePupilFnChannel.restype = None
    lib.mpArbInitializeSplineChannel.argtypes = [mpp, vp, f64, f64, ci]
    lib.mpArbInitializeSplineChannel.restype = None
    lib.mpArbNewPeaks.argtypes = [mpp, f64, cs, ci]
    lib.mpArbNewPeaks.restype = None
    lib.mpDaoInitialize2DChannel.argtypes = [mpp, f64, f64, cd, cd, ci, ci]
    lib.mpDaoInitialize2DChannel.restype = None
    lib.mpDaoNewPeaks.argtypes = [mpp, f64, cs, ci]
    lib.mpDaoNewPeaks.restype = None
    lib.mpSetFrames.argtypes = [mpp, ci, ci]
    lib.mpSetFrames.restype = ci
    lib.mpNewPeaksBatch.argtypes = [mpp, f64, i32, cs]
    lib.mpNewPeaksBatch.restype = ci
    lib.mpDoFitBatch.argtypes = [mpp, ci]
    lib.mpDoFitBatch.restype = ci
    lib.mpSetTeams.argtypes = [mpp, ci]
    lib.mpSetTeams.restype = ci
    for name in ["getXSize", "getYSize", "getZSize"]:
        getattr(lib, name).argtypes = [vp]
        getattr(lib, name).restype = ci
    lib.mFitGetFitImage.argtypes = [hp, f64]
    lib.mFitGetResidual.argtypes = [hp, f64]
    lib.mFitGetNError.argtypes = [hp]
    lib.mFitGetNError.restype = ci
    lib.mFitGetUnconverged.argtypes = [hp]
    lib.mFitGetUnconverged.restype = ci
    lib.mFitGetPeakPropertyDouble.argtypes = [hp, f64, cs]
    lib.mFitGetPeakPropertyInt.argtypes = [hp, i32, cs]
    lib.mFitNewImage.argtypes = [hp, f64]
    lib.mFitNewBackground.argtypes = [hp, f64]
    lib.mFitSetPeakStatus.argtypes = [hp, i32]

    lib.saGetLastError.argtypes = [ctypes.c_char_p, ci]
    lib.saGetLastError.restype = ci
    lib.saClearLastError.argtypes = []
    lib.saClearLastError.restype = None
    lib.saDeviceCount.argtypes = []
    lib.saDeviceCount.restype = ci
    for name, args in [("saSetPrecision", [hp, ci]), ("saSetDilation", [hp, ci]),
                       ("saSetStream", [hp, vp]), ("saDoFit", [hp, ci]),
                       ("saGetCounters", [hp, i64]), ("saGetSchedStats", [hp, i64]),
                       ("saSetFrames", [hp, ci, ci]), ("saNewImages", [hp, vp, ci, ci, ci]),
                       ("saNewBackgrounds", [hp, vp, ci, ci, ci]),
                       ("saNewPeaksBatch", [hp, f64, i32, ci, cs]), ("saDoFitBatch", [hp, ci]),
                       ("saNewPeaksBatchDevice", [hp, vp, i32, ci, cs]),
                       ("saDoFitBatchFrames", [hp, ci, i32]), ("saSetPeakStatusBatch", [hp, i32]),
                       ("saRemovePeaksBatch", [hp, ci]), ("saReservePeaksBatch", [hp, ci]),
                       ("saGetFitImagesDevice", [hp, vp, ci]),
                       ("saGetNFitBatch", [hp, i32]), ("saGetPeakPropertyBatch", [hp, f64, cs]),
                       ("saGetPeakPropertyIntBatch", [hp, i32, cs]), ("saSetTiming", [hp, ci]),
                       ("saGetTiming", [hp, ctypes.POINTER(ctypes.c_double),
                                        ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)])]:
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = ci
    lib.saGetKernelLaunches.argtypes = [hp]
    lib.saGetKernelLaunches.restype = ctypes.c_int64
    lib.saGetResultsBatch.argtypes = [hp, f64, i32]
    lib.saGetResultsBatch.restype = ci
    lib.saSetDevice.argtypes = [ci]
    lib.saSetDevice.restype = ci
    lib.saGetSweepTimes.argtypes = [hp, ndpointer(dtype=numpy.float32, flags="C_CONTIGUOUS"), ci]
    lib.saGetSweepTimes.restype = ci
    lib.saGetFitImageNoAlloc.argtypes = [hp, ci, f64, ci]
    lib.saGetFitImageNoAlloc.restype = ci
    lib.saSolveDamped.argtypes = [f64, f64, ci, ci, ctypes.c_double, ci, f64, i32]
    lib.saSolveDamped.restype = ci
    lib.saSetSchedule.argtypes = [hp, ci, ci]
    lib.saSetSchedule.restype = ci
    lib.saGetSweepGrid.argtypes = [hp]
    lib.saGetSweepGrid.restype = ci
    lib.saSetTailPeaks.argtypes = [hp, ci]
    lib.saSetTailPeaks.restype = ci
    lib.saSetSweepCTAs.argtypes = [hp, ci]
    lib.saSetSweepCTAs.restype = ci
    lib.saSlotLoad.argtypes = [hp, ci, vp, vp, ci, f64, ci, cs, ci]
    lib.saSlotLoad.restype = ci
    lib.saSlotLaunch.argtypes = [hp, ci]
    lib.saSlotLaunch.restype = ci
    lib.saSlotPoll.argtypes = [hp, i32, i32]
    lib.saSlotPoll.restype = ci
    lib.saSlotReady.argtypes = [hp]
    lib.saSlotReady.restype = ci
    lib.saSlotResults.argtypes = [hp, ci, f64, i32]
    lib.saSlotResults.restype = ci

    # peak finder (include/sa_finder.h)
    i64r = ctypes.c_int64
    for name, args, res in [
            ("saFilterCreate", [f64, cd, ci, ci, ci], vp),
            ("saFilterAnalyze", [f64, ci, ci, i32, vp, vp], ci),
            ("saFilterConvolve", [vp, f64, f64], ci),
            ("saFilterConvolveMemo", [vp, f64, f64], ci),
            ("saFilterCleanup", [vp], None),
            ("saFilterConvolveDevice", [vp, vp, ci, ci, vp], ci),
            ("saFilterResultDevice", [vp], vp),
            ("saFilterInfo", [vp, i32], ci),
            ("saFilterSetStream", [vp, vp], ci),
            ("saCalcMaxPeaks", [vp], ci),
            ("saFindLocalMaxima", [vp, f64, f64, f64, f64], None),
            ("saMaximaCreate", [ci, ci, cd, cd, f64, ci, ci], vp),
            ("saMaximaFind", [vp, vp, ci, ci, ci, ci, i32, cd], ci),
            ("saMaximaPeaksDevice", [vp], vp),
            ("saMaximaGetPeaks", [vp, f64], ci),
            ("saMaximaResetTaken", [vp], ci),
            ("saMaximaGetTaken", [vp, i32], ci),
            ("saMaximaSetStream", [vp, vp], ci),
            ("saMaximaCleanup", [vp], None),
            ("saMarkDimmerPeaks", [f64, f64, f64, i32, cd, cd, ci], ci),
            ("saMarkLowSignificancePeaks", [f64, f64, f64, i32, cd, cd, ci], ci),
            ("saRunningIfHasNeighbors", [f64, f64, f64, f64, i32, cd, ci, ci], None),
            ("saCreateKDTree", [f64, f64, ci], vp),
            ("saFreeKDTree", [vp], None),
            ("saNearestKDTree", [vp, f64, f64, f64, i32, cd, ci], None),
            ("saIngestCreate", [ci, ci, ci, vp, vp, cd, cd, ci], vp),
            ("saIngestFrames", [vp, vp, ci, ci, ci, ci, vp], ci),
            ("saIngestResultDevice", [vp], vp),
            ("saIngestGetFrames", [vp, f64], ci),
            ("saIngestSetStream", [vp, vp], ci),
            ("saIngestKernelLaunches", [vp], i64r),
            ("saIngestCleanup", [vp], None),
            ("saFinderCreate", [ci, ci, vp, vp, vp, ci, cd, cd, cd, cd], vp),
            ("saFinderCreateArbitrary", [ci, ci, vp, ci, vp, vp, f64, ci, cd, cd], vp),
            ("saFinderSetVariance", [vp, vp], ci),
            ("saFinderSetMask", [vp, vp], ci),
            ("saFinderNewImages", [vp, vp, ci, ci], ci),
            ("saFinderEstimateBackground", [vp, vp, vp, ci], ci),
            ("saFinderFindPeaks", [vp, vp, ci, i32], ci),
            ("saFinderBackgroundDevice", [vp], vp),
            ("saFinderPeaksDevice", [vp], vp),
            ("saFinderGetPeaks", [vp, f64], ci),
            ("saFinderGetArray", [vp, ci, f64], ci),
            ("saFinderSetStream", [vp, vp], ci),
            ("saFinderKernelLaunches", [vp], i64r),
            ("saFinderCleanup", [vp], None)]:
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res


EXPORTS = ["daoInitialize", "daoInitialize2DFixed", "daoInitialize2D", "daoInitialize3D",
           "daoInitializeZ", "daoNewPeaks", "daoCleanup", "daoInitialize2DFixedALS",
           "daoInitialize2DFixedLS", "daoInitialize2DFixedDWLS", "daoInitialize2DFixedFWLS",
           "daoInitialize2DALS", "daoInitialize2DLS", "daoInitialize2DDWLS", "daoInitialize2DFWLS",
           "initSpline2D", "initSpline3D", "splineCleanup", "getXSize", "getYSize", "getZSize",
           "cfInitialize", "cfInitialize2D", "cfInitialize3D", "cfInitialize3DALS",
           "cfInitialize3DLS", "cfInitialize3DFWLS", "cfNewPeaks", "cfCleanup",
           "pFTInitialize", "pFTCleanup", "pFTTranslate", "pFTGetPSF", "pFTGetPSFdx", "pFTGetPSFdy",
           "pFTGetPSFdz", "pFTGetXSize", "pFTGetYSize", "pFTGetZSize", "ftFitInitialize", "ftFitNewPeaks",
           "ftFitCleanup",
           "pfnInitialize", "pfnCleanup", "pfnSetPF", "pfnSetPNEN", "pfnTranslate", "pfnTranslateZ",
           "pfnGetPSF", "pfnGetPSFdx", "pfnGetPSFdy", "pfnGetPSFdz", "pfnGetPSFIntensity", "pfnGetPXEX",
           "pfnGetPXEY", "pfnGetPYEX", "pfnGetPYEY", "pfnGetPZEX", "pfnGetPZEY", "pfnGetSize",
           "pfitInitialize", "pfitNewPeaks", "pfitSetZRange", "pfitCleanup",
           "mpInitialize", "mpCleanup", "mpIterateLM", "mpSetTransforms", "mpSetWeights", "mpSetWeightsIndexing",
           "mpArbInitializePSFFFTChannel", "mpArbInitializePupilFnChannel", "mpArbInitializeSplineChannel",
           "mpArbNewPeaks", "mpDaoInitialize2DChannel", "mpDaoNewPeaks", "mpSetFrames", "mpNewPeaksBatch",
           "mpDoFitBatch", "mpSetTeams",
           "mFitAnscombeTransformImage", "mFitGetFitImage", "mFitGetNError",
           "mFitGetPeakPropertyDouble", "mFitGetPeakPropertyInt", "mFitGetResidual",
           "mFitGetUnconverged", "mFitIterateLM", "mFitNewBackground", "mFitNewImage",
           "mFitRemoveErrorPeaks", "mFitRemoveRunningPeaks", "mFitSetPeakStatus",
           "saGetLastError", "saClearLastError", "saDeviceCount", "saSetPrecision", "saSetDilation", "saSetStream",
           "saDoFit", "saGetCounters", "saGetSchedStats", "saSetFrames", "saNewImages",
           "saNewBackgrounds", "saNewPeaksBatch", "saNewPeaksBatchDevice", "saDoFitBatch", "saGetNFitBatch",
           "saDoFitBatchFrames", "saSetPeakStatusBatch", "saRemovePeaksBatch", "saReservePeaksBatch",
           "saGetFitImagesDevice",
           "saGetPeakPropertyBatch", "saGetPeakPropertyIntBatch", "saSetTiming", "saGetTiming",
           "saGetKernelLaunches", "saGetResultsBatch", "saSetDevice", "saGetSweepTimes",
           "saGetFitImageNoAlloc", "saSlotLoad", "saSlotLaunch", "saSlotPoll", "saSlotReady", "saSlotResults",
           "saSetSweepCTAs", "saSolveDamped", "saSetSchedule", "saGetSweepGrid", "saSetTailPeaks"]

FINDER_EXPORTS = ["saFilterCreate", "saFilterAnalyze", "saFilterConvolve", "saFilterConvolveMemo", "saFilterCleanup",
                  "saFilterConvolveDevice", "saFilterResultDevice", "saFilterInfo", "saFilterSetStream",
                  "saCalcMaxPeaks", "saFindLocalMaxima", "saMaximaCreate", "saMaximaFind",
                  "saMaximaPeaksDevice", "saMaximaGetPeaks", "saMaximaResetTaken", "saMaximaGetTaken",
                  "saMaximaSetStream", "saMaximaCleanup", "saMarkDimmerPeaks", "saMarkLowSignificancePeaks",
                  "saRunningIfHasNeighbors", "saCreateKDTree", "saFreeKDTree", "saNearestKDTree",
                  "saIngestCreate", "saIngestFrames",
                  "saIngestResultDevice", "saIngestGetFrames", "saIngestSetStream", "saIngestKernelLaunches",
                  "saIngestCleanup", "saFinderCreate", "saFinderCreateArbitrary", "saFinderSetVariance",
                  "saFinderSetMask", "saFinderNewImages", "saFinderEstimateBackground",
                  "saFinderFindPeaks", "saFinderBackgroundDevice", "saFinderPeaksDevice",
                  "saFinderGetPeaks", "saFinderGetArray", "saFinderSetStream", "saFinderKernelLaunches",
                  "saFinderCleanup"]

# libsa_matched_filter.so: the reference's matched-filter names
MATCHED_FILTER_EXPORTS = ["cleanup", "convolve", "convolveMemo", "initialize"]
MF_LIB_PATH = os.path.join(HERE, "libsa_matched_filter.so")

# libsa_ia_utilities.so: the reference's image-analysis utility names
IA_UTILITIES_EXPORTS = ["calcMaxPeaks", "createKDTree", "findLocalMaxima", "freeKDTree", "markDimmerPeaks",
                        "markLowSignificancePeaks", "nearestKDTree", "runningIfHasNeighbors"]
IA_LIB_PATH = os.path.join(HERE, "libsa_ia_utilities.so")
