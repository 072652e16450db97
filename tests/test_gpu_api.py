"""Behaviour of the reference MultiFitter API on the GPU engine: the
scenarios of the reference's test/test_multifit.py (storage growth, ERROR
and RUNNING peak removal, initial height/background, status marking,
pre-specified peaks round trip, significance, RQE) plus batching."""
import numpy
import pytest

pytestmark = pytest.mark.gpu


def gauss_image(shape, peaks, bg):
    """Sum of h * exp(-((c-x)^2 + (r-y)^2)/(2 s^2)) over (x, y, h, s) plus bg."""
    ny, nx = shape
    img = numpy.full(shape, float(bg))
    r, c = numpy.mgrid[0:ny, 0:nx]
    for (x, y, h, s) in peaks:
        img += h * numpy.exp(-((c - x) ** 2 + (r - y) ** 2) / (2.0 * s * s))
    return img


def mf2d(**kw):
    from sa_gb300 import dao_fit_c
    return dao_fit_c.MultiFitter2D(sigma_range=[1.0, 2.0], **kw)


def test_storage_growth_in_units_of_500():
    image = numpy.ones((40, 40))
    m = mf2d()
    m.initializeC(image)
    m.newImage(image)
    m.newBackground(image)
    assert m.getNFit() == 0 and m.getNFitMax() == 0
    n = 1020
    peaks = {"x": numpy.full(n, 20.0), "y": numpy.full(n, 20.0), "z": numpy.zeros(n),
             "sigma": numpy.ones(n)}
    m.newPeaks(peaks, "testing")
    assert m.getNFit() == n and m.getNFitMax() == 1500
    peaks["sigma"][:] = 2.0
    m.newPeaks(peaks, "testing")
    assert m.getNFit() == 2 * n and m.getNFitMax() == 2500
    w = m.getPeakProperty("xsigma")
    assert abs(w[0] - 1.0) < 1e-6 and abs(w[n] - 2.0) < 1e-6
    m.cleanup(verbose=False)


def test_growth_compacts_error_peaks():
    image = numpy.ones((40, 40))
    m = mf2d()
    m.initializeC(image)
    m.newImage(image)
    m.newBackground(image)
    z5 = numpy.zeros(5)
    m.newPeaks({"x": z5, "y": z5, "z": z5, "sigma": numpy.ones(5)}, "testing")
    assert m.getNFit() == 5 and m.getNFitMax() == 500
    n = 500
    m.newPeaks({"x": numpy.full(n, 20.0), "y": numpy.full(n, 20.0), "z": numpy.zeros(n),
                "sigma": numpy.full(n, 2.0)}, "testing")
    assert m.getNFit() == n and m.getNFitMax() == 1000
    assert abs(m.getPeakProperty("xsigma")[0] - 2.0) < 1e-6
    m.cleanup(verbose=False)


def test_error_and_running_removal_and_status():
    image = numpy.ones((40, 40))
    m = mf2d()
    m.initializeC(image)
    m.newImage(image)
    m.newBackground(image)
    n = 5
    m.newPeaks({"x": numpy.full(n, 20.0), "y": numpy.full(n, 20.0), "z": numpy.zeros(n),
                "sigma": 0.1 * numpy.arange(n) + 1.0}, "testing")
    m.removeErrorPeaks()
    assert m.getNFit() == 5
    status = m.getPeakProperty("status")
    status[1] = 2
    status[3] = 2
    m.setPeakStatus(status)
    m.removeErrorPeaks()
    assert m.getNFit() == 3
    assert numpy.allclose(m.getPeakProperty("xsigma"), [1.0, 1.2, 1.4])
    status = m.getPeakProperty("status")
    status[:] = 1
    status[0] = 0
    m.setPeakStatus(status)
    m.removeRunningPeaks()
    assert m.getNFit() == 2
    assert numpy.allclose(m.getPeakProperty("xsigma"), [1.2, 1.4])
    m.cleanup(verbose=False)


def test_height_background_init_and_fit():
    height, sigma = 20.0, 1.5
    bgim = numpy.full((100, 120), 10.0)
    image = gauss_image((100, 120), [(50.0, 50.0, height, sigma), (54.0, 50.0, height, sigma)], 0.0) + bgim
    for prec in (64, 32):
        m = mf2d(precision=prec)
        m.initializeC(image)
        m.newImage(image)
        m.newBackground(bgim)
        peaks = {"x": numpy.array([50.0, 54.0]), "y": numpy.array([50.0, 50.0]),
                 "z": numpy.zeros(2), "sigma": numpy.array([sigma, sigma])}
        m.newPeaks(peaks, "finder")
        h = m.getPeakProperty("height")
        assert (numpy.abs(h - height) / height < 0.1).all()
        assert (numpy.abs(m.getPeakProperty("background") - 10.0) < 1e-6).all()
        m.doFit()
        assert (numpy.abs(m.getPeakProperty("x") - peaks["x"]) < 1e-2).all()
        assert (numpy.abs(m.getPeakProperty("y") - peaks["y"]) < 1e-2).all()
        assert (numpy.abs(m.getPeakProperty("xsigma") - sigma) / sigma < 0.02).all()
        m.cleanup(verbose=False)


def test_text_round_trip():
    image = numpy.ones((40, 40))
    m = mf2d()
    m.initializeC(image)
    m.newImage(image)
    m.newBackground(image)
    peaks = {"background": numpy.array([10.0, 20.0]), "height": numpy.array([11.0, 21.0]),
             "x": numpy.array([12.0, 22.0]), "xsigma": numpy.array([1.0, 2.0]),
             "y": numpy.array([14.0, 24.0]), "ysigma": numpy.array([3.0, 4.0]),
             "z": numpy.array([16.0, 26.0])}
    for ptype in ("text", "hdf5"):
        m.newImage(image)
        m.newPeaks(peaks, ptype)
        for p in peaks:
            assert numpy.allclose(m.getPeakProperty(p), peaks[p], atol=1e-6)
    m.cleanup(verbose=False)


def test_significance_and_rqe():
    sigma = 1.5
    bgim = numpy.full((100, 120), 10.0)
    image = gauss_image((100, 120), [(30.0, 50.0, 10.0, sigma), (50.0, 50.0, 20.0, sigma),
                                     (70.0, 50.0, 30.0, sigma)], 0.0) + bgim
    m = mf2d()
    m.initializeC(image)
    m.newImage(image)
    m.newBackground(bgim)
    m.newPeaks({"x": numpy.array([30.0, 50.0, 70.0]), "y": numpy.full(3, 50.0), "z": numpy.zeros(3),
                "sigma": numpy.full(3, sigma)}, "finder")
    sig = m.getPeakProperty("significance")
    assert numpy.allclose(sig / sig[0], [1, 2, 3])
    m.cleanup(verbose=False)
    # RQE (test_mfit_12)
    bgim = numpy.full((60, 120), 10.0)
    image = gauss_image((60, 120), [(30.0, 30.0, 10.0, sigma), (60.0, 30.0, 10.0, sigma),
                                    (90.0, 30.0, 10.0, sigma)], 0.0) + bgim
    rqe = numpy.ones_like(image)
    rqe[:, :60] = 0.7
    m = mf2d(rqe=rqe)
    m.initializeC(image)
    m.newImage(image)
    m.newBackground(bgim)
    m.newPeaks({"x": numpy.array([30.0, 60.0, 90.0]), "y": numpy.full(3, 30.0), "z": numpy.zeros(3),
                "sigma": numpy.full(3, sigma)}, "finder")
    sig = m.getPeakProperty("significance")
    assert numpy.allclose(sig / sig[0], numpy.ones(3))
    assert numpy.allclose(image, m.getFitImage() + bgim, atol=0.2)
    m.cleanup(verbose=False)


def test_batch_equals_single_frames():
    """Frames fitted together in one frame set give bit-identical results to
    the same frames fitted one at a time."""
    from sa_gb300 import engine, synth
    from gpu_helpers import concat, fit_workload_gpu
    wl = synth.make_workload(1, frames=3, nx=192, ny=192)
    single = concat(fit_workload_gpu(wl, [0, 1, 2], 32))
    kw = dict(wl["fitter"])
    kw.pop("model")
    b = engine.BatchFitter("3d", (192, 192), 3, **kw)
    b.load(numpy.stack(wl["images"]), numpy.stack(wl["backgrounds"]), wl["guesses"], "hdf5")
    b.fit(200)
    res = b.results()
    b.close()
    for p in ["x", "y", "height", "background", "status", "iterations", "error"]:
        assert numpy.array_equal(res[p], single[p]), p


def test_uniform_calibration_path_is_exact(monkeypatch):
    """With rqe 1 and no sCMOS term the FP32 write-back quantises a peak's
    background contribution once per step; the per-pixel form gives the
    same bits."""
    from sa_gb300 import engine, synth
    wl = synth.make_workload(1, frames=3, nx=192, ny=192)
    kw = dict(wl["fitter"])
    kw.pop("model")
    outs = []
    for fast in ("0", "1"):
        monkeypatch.setenv("SA_CUDA_CAL_FAST", fast)
        b = engine.BatchFitter("3d", (192, 192), 3, precision=32, **kw)
        b.load(numpy.stack(wl["images"]), numpy.stack(wl["backgrounds"]), wl["guesses"], "hdf5")
        sweeps = b.fit(200)
        outs.append((b.results(), sweeps))
        b.close()
    assert outs[0][1] == outs[1][1]
    for p in ["x", "y", "z", "height", "background", "status", "iterations", "error"]:
        assert numpy.array_equal(outs[0][0][p], outs[1][0][p]), p


def test_escape_rollback_path_is_exact():
    """With no footprint dilation almost every anchor move escapes; the
    rollback / barrier re-run must still reproduce the normal schedule."""
    from sa_gb300 import engine, synth
    wl = synth.make_workload(1, frames=2, nx=128, ny=128)
    kw = dict(wl["fitter"])
    kw.pop("model")
    outs = []
    for dil in (2, 0):
        b = engine.BatchFitter("3d", (128, 128), 2, dilation=dil, precision=64, **kw)
        b.load(numpy.stack(wl["images"]), numpy.stack(wl["backgrounds"]), wl["guesses"], "hdf5")
        b.fit(200)
        outs.append((b.results(), b.sched_stats()))
        b.close()
    assert outs[1][1]["reruns"] > 0
    for p in ["x", "y", "height", "status", "iterations"]:
        assert numpy.array_equal(outs[0][0][p], outs[1][0][p]), p
