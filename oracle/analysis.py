"""
CPU restatement of the reference's find / fit loop for one frame:
PeakFitter.fitPeaks and PeakFinderFitter.analyzeImage
(sa_library/fitting.py:701-782, :867-896, :910-925) over the oracle's
fitter (oracle/oracle.py), peak finder and culling (oracle/finder.py), for
3D-DAOSTORM (Gaussian finder and fitter) and Spliner (arbitrary-PSF finder,
cubic spline fitter).

TEST INFRASTRUCTURE ONLY: the checker of sa_gb300.find_peaks in tests/.
Product code never imports this module.
"""
import numpy

from oracle import finder as F
from oracle.oracle import OracleFitter

UNCONVERGED_DIST = 5.0


def analyze_frame(params, frame, sigma_range, model="3d", max_iterations=2000, psf_object=None, spline=None):
    """Found and fitted peaks of one frame (x, y without the margin).  With
    psf_object and spline (the coefficients) the frame is analysed as
    Spliner does: the arbitrary-PSF finder, the cubic spline fitter and the
    neighbourhood int(spline size / 2) + 1 (fitting.py:826-834)."""
    sigma = params["sigma"]
    if psf_object is not None:
        finder = F.PeakFinderArbitraryPSF(params, psf_object)
        margin = finder.margin
        image = F.pad_array(frame, margin)
        mf = OracleFitter("spline3D", image.shape, spline=spline)
        neighborhood = int(0.5 * psf_object.getSize()) + 1
    else:
        finder = F.PeakFinderGaussian(params)
        margin = finder.margin
        image = F.pad_array(frame, margin)
        mf = OracleFitter(model, image.shape, roi_size=finder.roi_size, sigma_range=sigma_range)
        neighborhood = sigma * UNCONVERGED_DIST
    fit_image = numpy.zeros(image.shape)
    finder.newImage(image)
    mf.newImage(image)
    for _ in range(finder.iterations):
        background = finder.estimateBackground(fit_image)
        new_peaks, peaks_type, done = finder.findPeaks(fit_image)
        mf.newBackground(background)
        if new_peaks["x"].size > 0:
            if mf.getNFit() > 0:
                status = mf.getPeakProperty("status")
                F.running_if_has_neighbors(mf.getPeakProperty("x"), mf.getPeakProperty("y"), new_peaks["x"],
                                           new_peaks["y"], status, neighborhood)
                mf.setPeakStatus(status)
            mf.newPeaks(new_peaks, peaks_type)
            mf.doFit(max_iterations)
            mf.removeErrorPeaks()
            status = mf.getPeakProperty("status")
            px = mf.getPeakProperty("x")
            py = mf.getPeakProperty("y")
            n_p = F.mark_dimmer_peaks(px, py, mf.getPeakProperty("height"), status, sigma, neighborhood)
            n_s = F.mark_low_significance_peaks(px, py, mf.getPeakProperty("significance"), status,
                                                params["threshold"], neighborhood)
            if n_p + n_s > 0:
                mf.setPeakStatus(status)
                mf.removeErrorPeaks()
            if mf.getUnconverged() > 0:
                mf.doFit(max_iterations)
                mf.removeErrorPeaks()
        fit_image = mf.getFitImage()
        if done:
            break
    mf.removeRunningPeaks()
    names = ("x", "y", "z", "height", "background", "significance", "status") if psf_object is not None else \
        ("x", "y", "height", "background", "xsigma", "ysigma", "significance", "status")
    out = {p: mf.getPeakProperty(p) for p in names}
    out["x"] = out["x"] - float(margin)
    out["y"] = out["y"] - float(margin)
    mf.cleanup()
    return out
