"""The control flow of the batched find / fit loop (sa_gb300.find_peaks.
BatchFindFit), replayed on the CPU with the oracle's finder, fitter and
culling: all frames advance pass by pass together; a frame whose pass
found no new peaks is not refitted, and a frame that is done keeps taking
finder passes until every frame is done.  The claim the batched loop rests
on -- that those extra finder passes change nothing -- is checked here:
every frame ends exactly as the reference's one-frame loop ends it."""
import numpy

from oracle import analysis
from oracle import finder as F
from oracle.oracle import OracleFitter

PARAMS = dict(background_sigma=8.0, foreground_sigma=1.0, find_max_radius=5, iterations=20, sigma=1.5,
              threshold=6.0, roi_size=18, model="3d")


def batched_replay(frames, sigma_range=(0.75, 7.5)):
    n = len(frames)
    finders = [F.PeakFinderGaussian(PARAMS) for _ in range(n)]
    margin = finders[0].margin
    images = [F.pad_array(f, margin) for f in frames]
    fitters = [OracleFitter("3d", images[0].shape, roi_size=18, sigma_range=list(sigma_range)) for _ in range(n)]
    fits = [numpy.zeros(images[0].shape) for _ in range(n)]
    for k in range(n):
        finders[k].newImage(images[k])
        fitters[k].newImage(images[k])
    nb = PARAMS["sigma"] * analysis.UNCONVERGED_DIST
    done = numpy.zeros(n, dtype=bool)
    for _ in range(finders[0].iterations):
        counting_down = finders[0].cur_threshold > finders[0].threshold
        news = []
        for k in range(n):
            bg = finders[k].estimateBackground(fits[k])
            news.append(finders[k].findPeaks(fits[k])[0])
            fitters[k].newBackground(bg)
        counts = numpy.array([p["x"].size for p in news])
        for k in numpy.nonzero((counts > 0) & ~done)[0]:
            mf, newp = fitters[k], news[k]
            if mf.getNFit() > 0:
                st = mf.getPeakProperty("status")
                F.running_if_has_neighbors(mf.getPeakProperty("x"), mf.getPeakProperty("y"), newp["x"], newp["y"],
                                           st, nb)
                mf.setPeakStatus(st)
            mf.newPeaks(newp, "finder")
            mf.doFit()
            mf.removeErrorPeaks()
            st = mf.getPeakProperty("status")
            px, py = mf.getPeakProperty("x"), mf.getPeakProperty("y")
            n_p = F.mark_dimmer_peaks(px, py, mf.getPeakProperty("height"), st, PARAMS["sigma"], nb)
            n_s = F.mark_low_significance_peaks(px, py, mf.getPeakProperty("significance"), st,
                                                PARAMS["threshold"], nb)
            if n_p + n_s > 0:
                mf.setPeakStatus(st)
                mf.removeErrorPeaks()
            if mf.getUnconverged() > 0:
                mf.doFit()
                mf.removeErrorPeaks()
        fits = [mf.getFitImage() for mf in fitters]
        if not counting_down:
            done |= counts == 0
        if done.all():
            break
    out = []
    for mf in fitters:
        mf.removeRunningPeaks()
        out.append({p: mf.getPeakProperty(p) for p in ("x", "y", "height")})
        mf.cleanup()
    return out


def test_batched_control_flow_equals_per_frame_loops():
    from sa_gb300 import synth
    wl = synth.make_workload(1, frames=3, nx=128, ny=128, seed=31)
    got = batched_replay(wl["images"])
    for k in range(3):
        ref = analysis.analyze_frame(PARAMS, wl["images"][k], [0.75, 7.5])
        assert got[k]["x"].size == ref["x"].size
        assert numpy.array_equal(got[k]["x"] - 11.0, ref["x"])
        assert numpy.array_equal(got[k]["height"], ref["height"])


class _OracleMultiFitter(object):
    """The oracle fitter behind the MultiFitter methods FindFitLoop calls
    (initializeC on the first image, doFit(max_iterations), rescaleZ)."""

    def __init__(self, model, **kw):
        self.model, self.kw, self.f = model, kw, None

    def isInitialized(self):
        return self.f is not None

    def initializeC(self, image):
        self.f = OracleFitter(self.model, image.shape, **self.kw)

    def rescaleZ(self, z):
        return z

    def cleanup(self, verbose=False):
        self.f.cleanup()

    def __getattr__(self, name):
        return getattr(self.f, name)


class _OracleCulling(object):
    """The oracle's culling loops with FindFitLoop's culling interface."""

    @staticmethod
    def wake(status, x, y, new_x, new_y, radius):
        return F.running_if_has_neighbors(x, y, new_x, new_y, status, radius)

    @staticmethod
    def dimmer(x, y, height, status, sigma, radius):
        return F.mark_dimmer_peaks(x, y, height, status, sigma, radius)

    @staticmethod
    def faint(x, y, significance, status, threshold, radius):
        return F.mark_low_significance_peaks(x, y, significance, status, threshold, radius)


def test_find_fit_loop_control_flow_equals_oracle_loop():
    """sa_gb300.find_peaks.FindFitLoop (the one-frame find / fit loop, its
    fit passes through find_peaks.fit_pass) driven with the oracle's finder,
    fitter and culling gives exactly the oracle's restatement of the
    reference loop (oracle/analysis.py): the loop's control flow is the
    reference's."""
    from sa_gb300 import find_peaks, synth
    wl = synth.make_workload(1, frames=2, nx=128, ny=128, seed=21)
    props = ["x", "y", "height", "background", "xsigma", "ysigma", "significance", "status"]
    for k in range(2):
        loop = find_peaks.FindFitLoop(F.PeakFinderGaussian(PARAMS),
                                      _OracleMultiFitter("3d", roi_size=18, sigma_range=[0.75, 7.5]), props,
                                      PARAMS["sigma"] * find_peaks.UNCONVERGED_DIST, PARAMS["sigma"],
                                      PARAMS["threshold"], culling=_OracleCulling)
        got = loop.analyzeFrame(wl["images"][k])
        loop.mfitter.cleanup()
        ref = analysis.analyze_frame(PARAMS, wl["images"][k], [0.75, 7.5])
        assert ref["x"].size > 100
        for p in props:
            assert numpy.array_equal(got[p], ref[p]), (k, p)


def test_fit_pass_over_frame_sets_equals_batched_replay():
    """find_peaks.fit_pass over a FitterFrames set of three oracle fitters,
    driven pass by pass as BatchFindFit drives its BatchFrames set (all
    frames in lockstep, only frames with new peaks and not done take a fit
    pass), ends every frame exactly as the reference's one-frame loop."""
    from sa_gb300 import find_peaks, synth
    wl = synth.make_workload(1, frames=3, nx=128, ny=128, seed=31)
    n = 3
    finders = [F.PeakFinderGaussian(PARAMS) for _ in range(n)]
    margin = finders[0].margin
    images = [F.pad_array(f, margin) for f in wl["images"]]
    fitters = [OracleFitter("3d", images[0].shape, roi_size=18, sigma_range=[0.75, 7.5]) for _ in range(n)]
    fs = find_peaks.FitterFrames(fitters)
    fits = [numpy.zeros(images[0].shape) for _ in range(n)]
    for k in range(n):
        finders[k].newImage(images[k])
        fitters[k].newImage(images[k])
    nb = PARAMS["sigma"] * find_peaks.UNCONVERGED_DIST
    done = numpy.zeros(n, dtype=bool)
    for _ in range(finders[0].iterations):
        counting_down = finders[0].cur_threshold > finders[0].threshold
        news = []
        for k in range(n):
            bg = finders[k].estimateBackground(fits[k])
            news.append(finders[k].findPeaks(fits[k])[0])
            fitters[k].newBackground(bg)
        counts = numpy.array([p["x"].size for p in news])
        find_peaks.fit_pass(fs, numpy.nonzero((counts > 0) & ~done)[0], news, "finder", PARAMS["sigma"],
                            PARAMS["threshold"], nb, culling=_OracleCulling)
        fits = [mf.getFitImage() for mf in fitters]
        if not counting_down:
            done |= counts == 0
        if done.all():
            break
    for k in range(n):
        fitters[k].removeRunningPeaks()
        ref = analysis.analyze_frame(PARAMS, wl["images"][k], [0.75, 7.5])
        for p in ("x", "y", "height"):
            got = fitters[k].getPeakProperty(p)
            if p in ("x", "y"):
                got = got - float(margin)
            assert numpy.array_equal(got, ref[p]), (k, p)
        fitters[k].cleanup()
