"""The tail of a fit (saSetTailPeaks): once every frame still fitting has
at most a few RUNNING peaks, their remaining sweeps run in one launch, each
frame's steps one after another in index order.  The results -- every
peak's parameters, status and iteration count, the counters and the sweep
count -- are the ones the per-sweep ticks give, with fewer launches."""
import numpy
import pytest

pytestmark = pytest.mark.gpu

CASES = [(1, 32, {}), (1, 64, {}), (2, 32, {}), (3, 32, dict(n_emitters=60))]


def fit_once(wl, precision, tail_peaks, max_iterations=2000):
    from sa_gb300 import cubic_fit_c, engine
    kw = dict(wl["fitter"])
    model = kw.pop("model")
    spl = kw.pop("spline", None)
    if spl is not None:
        kw["spline"] = cubic_fit_c.SplinePSF(coeff=spl["coeff"])
    fit = engine.BatchFitter(model, (wl["ny"], wl["nx"]), len(wl["images"]), rqe=wl["rqe"],
                             scmos_cal=wl["scmos_cal"], precision=precision, **kw)
    assert fit.clib.saSetTailPeaks(fit.h, tail_peaks) == 0
    fit.load(numpy.stack(wl["images"]), numpy.stack(wl["backgrounds"]), wl["guesses"], "hdf5")
    l0 = fit.kernel_launches()
    sweeps = fit.fit(max_iterations)
    out = fit.results()
    out["counters"] = fit.counters()
    out["sweeps"] = sweeps
    out["launches"] = fit.kernel_launches() - l0
    fit.close()
    return out


@pytest.mark.parametrize("cfg,precision,kw", CASES)
def test_tail_launch_gives_the_ticks_results(cfg, precision, kw):
    from sa_gb300 import synth
    wl = synth.make_workload(cfg, frames=2, nx=128, ny=128, seed=41, **kw)
    ticks = fit_once(wl, precision, 0)
    tail = fit_once(wl, precision, 4)
    for k in ("x", "y", "z", "height", "background", "status", "iterations", "counters"):
        assert numpy.array_equal(tail[k], ticks[k]), k
    assert tail["sweeps"] == ticks["sweeps"]
    assert tail["launches"] <= ticks["launches"]
