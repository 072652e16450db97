"""The GPU peak finder against the CPU oracle (oracle/finder.py) and the
golden fixture of the reference's own local-maxima C:

  * matched filters (separable and 2D paths, even / odd / clamped sizes,
    memoisation, the reference-named libsa_matched_filter.so);
  * the local-maxima finder, bit-exact (peak lists and taken counts) on the
    reference's outputs, through the handle and the flmData entry points;
  * PeakFinderGaussian.peakFinder on synthetic 512 x 512 frames (with and
    without the foreground filter, camera variance and an AOI mask), and
    the batched finder with its device hand-off to the fitter.

Tolerances: convolutions agree with numpy's FFT convolution to 1e-12 of the
result's magnitude (the two sum in different orders); the found peak lists
are compared exactly.
"""
import ctypes
import os

import numpy
import pytest

from oracle import finder as F

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "g_finder.npz")
CONV_RTOL = 1e-12

PARAMS = dict(background_sigma=8.0, foreground_sigma=1.0, find_max_radius=5, iterations=20, sigma=1.5,
              threshold=6.0, roi_size=18)


def conv_close(got, ref):
    return numpy.abs(got - ref).max() <= CONV_RTOL * max(numpy.abs(ref).max(), 1.0)


@pytest.mark.parametrize("shape,sigma", [((80, 90), 1.0), ((41, 53), 2.0), ((41, 53), 8.0),
                                         ((534, 534), 8.0), ((75, 64), 1.5)])
def test_matched_filter_separable(shape, sigma):
    from sa_gb300 import matched_filter_c
    rng = numpy.random.default_rng(int(sigma * 10) + shape[0])
    psf = F.gaussian_psf(shape, sigma)
    g = matched_filter_c.MatchedFilter(psf)
    assert g.info()[0] == 2        # separable, double-float passes
    o = F.MatchedFilter(psf)
    for _ in range(2):
        img = rng.uniform(0.0, 200.0, shape)
        assert conv_close(g.convolve(img), o.convolve(img))
    g.cleanup()


def test_double_float_passes_match_fp64_passes(monkeypatch):
    """The default separable passes (double-float on the FP32 pipe) agree
    with the FP64 passes (SA_FINDER_FP64=1) to 1e-13 of the magnitude, on
    the background (81 taps) and PSF-squared filters."""
    from sa_gb300 import matched_filter_c
    rng = numpy.random.default_rng(12)
    for sigma, square in ((8.0, False), (1.0, True)):
        psf = F.gaussian_psf((534, 534), sigma)
        if square:
            psf = psf * psf
        g_ff = matched_filter_c.MatchedFilter(psf)
        monkeypatch.setenv("SA_FINDER_FP64", "1")
        g_64 = matched_filter_c.MatchedFilter(psf)
        monkeypatch.delenv("SA_FINDER_FP64")
        assert g_ff.info()[0] == 2 and g_64.info()[0] == 1
        img = rng.uniform(1.0, 5000.0, (534, 534))
        a, b = g_ff.convolve(img), g_64.convolve(img)
        assert numpy.abs(a - b).max() <= 1e-13 * numpy.abs(b).max()
        g_ff.cleanup()
        g_64.cleanup()


def test_matched_filter_psf_squared_and_2d_path():
    from sa_gb300 import matched_filter_c
    rng = numpy.random.default_rng(8)
    psf = F.gaussian_psf((64, 48), 1.0)
    sq = psf * psf
    g = matched_filter_c.MatchedFilter(sq)
    img = rng.uniform(0.0, 50.0, (64, 48))
    assert conv_close(g.convolve(img), F.MatchedFilter(sq).convolve(img))
    g.cleanup()
    # a PSF that is not rank 1: the direct 2D path, support straddling the wrap
    blob = numpy.zeros((37, 45))
    blob[14:23, 17:28] = rng.uniform(0.0, 1.0, (9, 11))
    g = matched_filter_c.MatchedFilter(blob)
    info = g.info()
    assert info[0] == 0 and info[1] == 9 and info[2] == 11
    for _ in range(2):
        img = rng.uniform(-5.0, 50.0, (37, 45))
        assert conv_close(g.convolve(img), F.MatchedFilter(blob).convolve(img))
    g.cleanup()


def test_matched_filter_memo_and_normalisation():
    """The reference's matched-filter tests: unit-sum PSF keeps the sum;
    memoisation returns the previous result while no pixel moved more than
    max_diff and recomputes after."""
    from sa_gb300 import matched_filter_c
    psf = F.gaussian_psf((80, 90), 1.0)
    g = matched_filter_c.MatchedFilter(psf)
    for i in range(1, 5):
        img = numpy.zeros((80, 90))
        img[40, 45] = float(i)
        assert abs(img.sum() - g.convolve(img).sum()) < 1e-6
    g.cleanup()
    psf = F.gaussian_psf((40, 50), 2.0)
    g = matched_filter_c.MatchedFilter(psf, memoize=True, max_diff=0.1)
    o = F.MatchedFilter(psf, memoize=True, max_diff=0.1)
    assert numpy.array_equal(g.convolve(numpy.zeros((40, 50))), o.convolve(numpy.zeros((40, 50))))
    seq = [1.0, 1.05, 1.1, 1.0, 1.0]
    prev = None
    for v in seq:
        img = numpy.zeros((40, 50))
        img[20, 25] = v
        r, ro = g.convolve(img), o.convolve(img)
        assert conv_close(r, ro)
        if prev is not None and v in (1.05,):
            assert numpy.abs(r - prev).max() < 1e-12
        prev = r
    g.cleanup()


def test_reference_named_matched_filter_library():
    """libsa_matched_filter.so answers the reference binding's calls
    (matched_filter_c.py:17-34): initialize / convolve / convolveMemo /
    cleanup with host arrays."""
    from numpy.ctypeslib import ndpointer
    from sa_gb300 import loadclib
    loadclib.load()
    mf = ctypes.CDLL(loadclib.MF_LIB_PATH)
    f64 = ndpointer(dtype=numpy.float64)
    mf.initialize.argtypes = [f64, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    mf.initialize.restype = ctypes.c_void_p
    mf.convolve.argtypes = [ctypes.c_void_p, f64, f64]
    mf.convolveMemo.argtypes = [ctypes.c_void_p, f64, f64]
    mf.cleanup.argtypes = [ctypes.c_void_p]
    psf = F.gaussian_psf((60, 70), 2.0)
    rc = numpy.ascontiguousarray(F.recenter_psf(psf))
    h = mf.initialize(rc, 1.0e-3, 60, 70, 1)
    img = numpy.random.default_rng(2).uniform(0, 10, (60, 70))
    out = numpy.zeros((60, 70))
    mf.convolve(h, img, out)
    assert conv_close(out, F.MatchedFilter(psf).convolve(img))
    out2 = numpy.zeros((60, 70))
    mf.convolveMemo(h, img, out2)
    assert conv_close(out2, out)
    mf.cleanup(h)


def _lm_cases(g):
    i = 0
    while "lm%d_images" % i in g:
        yield i
        i += 1


def test_local_maxima_match_reference_golden():
    """MaximaFinder on the GPU returns the reference's peaks and taken
    counts exactly, call after call (ties, planes, fractional radii)."""
    from sa_gb300 import ia_utilities_c
    g = numpy.load(GOLDEN)
    for i in _lm_cases(g):
        imgs = [numpy.ascontiguousarray(a) for a in g["lm%d_images" % i]]
        m, r, thr, zr, calls, nd = g["lm%d_params" % i]
        zv = list(g["lm%d_zvalues" % i])
        mx = ia_utilities_c.MaximaFinder(margin=int(m) - 1, n_duplicates=int(nd), radius=float(r),
                                         threshold=float(thr), z_range=int(zr), z_values=zv)
        for c in range(int(calls)):
            x, y, z, h = mx.findMaxima(imgs, want_height=True)
            got = numpy.stack([x, y, z, h]) if x.size else numpy.zeros((4, 0))
            assert numpy.array_equal(got, g["lm%d_c%d_xyzh" % (i, c)]), (i, c)
            assert numpy.array_equal(mx.getTaken(), g["lm%d_c%d_taken" % (i, c)]), (i, c)
        mx.resetTaken()
        assert numpy.all(mx.getTaken() == 1 - int(nd))
        mx.cleanup()


def test_flmdata_entry_points_match_reference_golden():
    """saCalcMaxPeaks / saFindLocalMaxima with the reference's flmData and
    host arrays (the calls ia_utilities_c.py:214-225 makes)."""
    from sa_gb300 import ia_utilities_c
    g = numpy.load(GOLDEN)
    for i in _lm_cases(g):
        imgs = [numpy.ascontiguousarray(a) for a in g["lm%d_images" % i]]
        m, r, thr, zr, calls, nd = g["lm%d_params" % i]
        zv = numpy.ascontiguousarray(g["lm%d_zvalues" % i], dtype=numpy.float64)
        taken = [numpy.ascontiguousarray(numpy.ones(imgs[0].shape, numpy.int32) - int(nd)) for _ in imgs]
        P = ctypes.c_void_p * len(imgs)
        c_img = P(*[a.ctypes.data for a in imgs])
        c_tk = P(*[t.ctypes.data for t in taken])
        flm = ia_utilities_c.FlmData(margin=int(m), n_peaks=0, z_range=int(zr), xsize=imgs[0].shape[1],
                                     ysize=imgs[0].shape[0], zsize=len(imgs), radius=float(r),
                                     threshold=float(thr), z_values=zv.ctypes.data,
                                     taken=ctypes.addressof(c_tk), images=ctypes.addressof(c_img))
        for c in range(int(calls)):
            n = ia_utilities_c.calc_max_peaks(flm)
            assert n == int(g["lm%d_c%d_max" % (i, c)])
            out = [numpy.zeros(n + 1) for _ in range(4)]
            flm.n_peaks = n + 1
            k = ia_utilities_c.find_local_maxima(flm, *out)
            z, y, x, h = (a[:k] for a in out)
            got = numpy.stack([x, y, z, h]) if k else numpy.zeros((4, 0))
            assert numpy.array_equal(got, g["lm%d_c%d_xyzh" % (i, c)]), (i, c)
            assert numpy.array_equal(numpy.stack(taken), g["lm%d_c%d_taken" % (i, c)]), (i, c)
    # the n_peaks cap: the first n_peaks maxima, taken advanced for those only
    imgs = [numpy.ascontiguousarray(a) for a in g["lm0_images"]]
    m, r, thr, zr, calls, nd = g["lm0_params"]
    full = g["lm0_c0_xyzh"]
    taken = [numpy.zeros(imgs[0].shape, numpy.int32)]
    c_img = (ctypes.c_void_p * 1)(imgs[0].ctypes.data)
    c_tk = (ctypes.c_void_p * 1)(taken[0].ctypes.data)
    zv = numpy.ascontiguousarray(g["lm0_zvalues"])
    flm = ia_utilities_c.FlmData(margin=int(m), n_peaks=10, z_range=int(zr), xsize=imgs[0].shape[1],
                                 ysize=imgs[0].shape[0], zsize=1, radius=float(r), threshold=float(thr),
                                 z_values=zv.ctypes.data, taken=ctypes.addressof(c_tk),
                                 images=ctypes.addressof(c_img))
    out = [numpy.zeros(10) for _ in range(4)]
    assert ia_utilities_c.find_local_maxima(flm, *out) == 10
    assert numpy.array_equal(out[2], full[0, :10]) and numpy.array_equal(out[1], full[1, :10])
    assert int(taken[0].sum()) == 10


def _frames(n, size=512, seed=3):
    from sa_gb300 import synth
    wl = synth.make_workload(1, frames=n, nx=size, ny=size, seed=seed)
    return wl


def _compare_finder(params, frames, camvar=None, fit_images=None, iterations=1):
    from sa_gb300 import fitting
    gf = fitting.PeakFinderGaussian(params)
    of = F.PeakFinderGaussian(params)
    if camvar is not None:
        gf.setVariance(camvar)
        of.setVariance(camvar)
    n_peaks = 0
    for k, img in enumerate(frames):
        img = gf.padArray(img)
        gf.newImage(img)
        of.newImage(img)
        fit = numpy.zeros(img.shape) if fit_images is None else gf.padArray(fit_images[k])
        for it in range(iterations):
            bg_g = gf.estimateBackground(fit)
            bg_o = of.estimateBackground(fit)
            assert conv_close(bg_g, bg_o)
            pg, tg, dg = gf.findPeaks(fit)
            po, to, do = of.findPeaks(fit)
            assert (tg, dg) == (to, do)
            for key in ("x", "y", "z", "sigma"):
                assert numpy.array_equal(pg[key], po[key]), (k, it, key)
            sg = gf.significance()
            assert conv_close(sg, of.last_masked)
            n_peaks += pg["x"].size
    launches = gf.kernel_launches()
    gf.cleanUp()
    assert n_peaks > 0
    return n_peaks, launches


def test_peak_finder_matches_oracle_512():
    wl = _frames(2)
    n, launches = _compare_finder(PARAMS, wl["images"], iterations=2)
    assert launches > 0


def test_peak_finder_variants():
    """No foreground filter; camera variance; an AOI box; a fit image."""
    wl = _frames(1, size=256, seed=5)
    p = dict(PARAMS)
    p.pop("foreground_sigma")
    _compare_finder(p, wl["images"])
    cam = numpy.random.default_rng(1).gamma(2.0, 2.0, size=(256, 256))
    _compare_finder(PARAMS, wl["images"], camvar=cam)
    p = dict(PARAMS, x_start=20, x_stop=200, y_start=30, y_stop=220)
    _compare_finder(p, wl["images"])
    fit = [0.5 * numpy.asarray(wl["images"][0]) - 10.0]
    _compare_finder(PARAMS, wl["images"], fit_images=fit, iterations=3)


def test_batch_finder_matches_single_frames_and_hands_off():
    """Four frames at once equal four single-frame runs; the device
    hand-off to BatchFitter fits the same as loading the peaks from the
    host."""
    from sa_gb300 import engine, fitting
    wl = _frames(4, size=256, seed=9)
    pad = fitting.PeakFinderGaussian(PARAMS).margin
    frames = numpy.stack([fitting.padArray(im, pad) for im in wl["images"]])
    bf = fitting.BatchPeakFinder(PARAMS, frames.shape[1:], 4)
    bf.newImages(frames)
    bf.estimateBackground()
    counts, done = bf.findPeaks()
    peaks = bf.peaks()
    bgs = bf.background()
    for k in range(4):
        of = F.PeakFinderGaussian(PARAMS)
        of.newImage(frames[k])
        bo = of.estimateBackground(numpy.zeros(frames[k].shape))
        po, _, _ = of.findPeaks(numpy.zeros(frames[k].shape))
        assert conv_close(bgs[k], bo)
        assert counts[k] == po["x"].size
        for key in ("x", "y", "z", "sigma"):
            assert numpy.array_equal(peaks[k][key], po[key])
    kw = dict(roi_size=18, sigma_range=[0.5, 4.0])
    a = engine.BatchFitter("3d", frames.shape[1:], 4, precision=64, **kw)
    bf.handoff(a)
    a.fit(200)
    ra = a.results()
    b = engine.BatchFitter("3d", frames.shape[1:], 4, precision=64, **kw)
    b.load(frames, bgs, peaks, "finder")
    b.fit(200)
    rb = b.results()
    for key in ("x", "y", "height", "status"):
        assert numpy.array_equal(ra[key], rb[key]), key
    a.close()
    b.close()
    bf.cleanUp()


def test_frame_ingest_matches_reference_readers(tmp_path):
    """FrameReaderStd / FrameReaderSCMOS on the GPU return the reference
    readers' frames bit for bit (golden fixture), and the fused mirror
    padding equals padArray; float inputs go through the same kernel."""
    import ctypes
    from sa_gb300 import analysis_io, loadclib
    from test_oracle_ingest import write_dax
    g = numpy.load(os.path.join(os.path.dirname(GOLDEN), "g_ingest.npz"))
    n, h, w = g["frames"].shape
    for tag, big in (("big", 1), ("little", 0)):
        path = str(tmp_path / ("m_%s.dax" % tag))
        write_dax(path, g["raw_" + tag], big)
        rd = analysis_io.FrameReaderStd(movie_file=path, camera_gain=2.5, camera_offset=100.0)
        for i in range(n):
            assert numpy.array_equal(rd.loadAFrame(i), g["std_" + tag][i])
        ptr = rd.loadFramesPadded(0, n, 7)
        out = numpy.zeros((n, h + 14, w + 14))
        ih = rd._handle(7)
        rd.clib.saIngestGetFrames(ih, out)
        assert ptr and numpy.array_equal(out, g["std_%s_pad7" % tag])
        rd.close()
    cal = str(tmp_path / "calib.npy")
    numpy.save(cal, numpy.array([g["offset"], g["variance"], g["gain"], g["rqe"], 2], dtype=object),
               allow_pickle=True)
    rd = analysis_io.FrameReaderSCMOS(movie_file=str(tmp_path / "m_big.dax"), calibration_file=cal)
    for i in range(n):
        assert numpy.array_equal(rd.loadAFrame(i), g["scmos_big"][i])
    rd.loadFramesPadded(0, n, 11)
    out = numpy.zeros((n, h + 22, w + 22))
    rd.clib.saIngestGetFrames(rd._handle(11), out)
    assert numpy.array_equal(out, g["scmos_big_pad11"])
    rd.close()
    # float32 / float64 frames: conversion and padding only
    lib = loadclib.load()
    f64 = g["frames"].astype(numpy.float64) * 1.25
    for arr, bits in ((f64.astype(numpy.float32), 32), (f64, 64)):
        ih = lib.saIngestCreate(h, w, 5, None, None, 3.0, 0.5, 1)
        a = numpy.ascontiguousarray(arr)
        assert lib.saIngestFrames(ih, a.ctypes.data_as(ctypes.c_void_p), n, bits, 0, 0, None) == 0
        out = numpy.zeros((n, h + 10, w + 10))
        lib.saIngestGetFrames(ih, out)
        exp = numpy.stack([F.pad_array(numpy.maximum((a[i].astype(numpy.float64) - 3.0) * 0.5, 1.0), 5)
                           for i in range(n)])
        assert numpy.array_equal(out, exp)
        lib.saIngestCleanup(ih)


def _cull_cases(g):
    i = 0
    while "cull%d_xyhs" % i in g:
        yield i
        i += 1


def test_culling_matches_reference_golden():
    """The post-fit culling on the GPU returns the reference's statuses,
    counts and nearest-neighbour answers exactly (sa_gb300.ia_utilities_c
    mirror of the reference's Python functions)."""
    from sa_gb300 import ia_utilities_c as U
    g = numpy.load(GOLDEN)
    for i in _cull_cases(g):
        x, y, h, sig = (numpy.ascontiguousarray(a) for a in g["cull%d_xyhs" % i])
        st = numpy.ascontiguousarray(g["cull%d_status" % i])
        r1, r2 = (float(v) for v in g["cull%d_r" % i])
        s1 = st.copy()
        assert U.markDimmerPeaks(x, y, h, s1, r1, r2) == int(g["cull%d_dimmer_n" % i])
        assert numpy.array_equal(s1, g["cull%d_dimmer" % i])
        s2 = st.copy()
        assert U.markLowSignificancePeaks(x, y, sig, s2, 6.0, r2) == int(g["cull%d_lowsig_n" % i])
        assert numpy.array_equal(s2, g["cull%d_lowsig" % i])
        nx, ny = (numpy.ascontiguousarray(a) for a in g["cull%d_new" % i])
        assert numpy.array_equal(U.runningIfHasNeighbors(st.copy(), x, y, nx, ny, r2), g["cull%d_running" % i])
        kd = U.KDTree(x=nx, y=ny)
        d, ix = kd.nearest(x, y, r2)
        kd.cleanup()
        assert numpy.array_equal(d, g["cull%d_nearest_d" % i])
        assert numpy.array_equal(ix, g["cull%d_nearest_i" % i])
    # empty and degenerate inputs
    e = numpy.zeros(0)
    es = numpy.zeros(0, dtype=numpy.int32)
    assert U.markDimmerPeaks(e, e, e, es, 1.0, 5.0) == 0
    one = numpy.array([5.0])
    s = numpy.array([1], dtype=numpy.int32)
    assert U.markDimmerPeaks(one, one, one, s, 1.0, 5.0) == 0 and s[0] == 1


def test_reference_named_ia_utilities_library():
    """libsa_ia_utilities.so answers the reference binding's calls
    (ia_utilities_c.py:16-87) under the reference's names."""
    from numpy.ctypeslib import ndpointer
    from sa_gb300 import loadclib
    loadclib.load()
    ia = ctypes.CDLL(loadclib.IA_LIB_PATH)
    f64 = ndpointer(dtype=numpy.float64)
    i32 = ndpointer(dtype=numpy.int32)
    ia.markDimmerPeaks.argtypes = [f64, f64, f64, i32, ctypes.c_double, ctypes.c_double, ctypes.c_int]
    ia.markDimmerPeaks.restype = ctypes.c_int
    ia.createKDTree.argtypes = [f64, f64, ctypes.c_int]
    ia.createKDTree.restype = ctypes.c_void_p
    ia.nearestKDTree.argtypes = [ctypes.c_void_p, f64, f64, f64, i32, ctypes.c_double, ctypes.c_int]
    ia.freeKDTree.argtypes = [ctypes.c_void_p]
    g = numpy.load(GOLDEN)
    x, y, h, sig = (numpy.ascontiguousarray(a) for a in g["cull0_xyhs"])
    st = numpy.ascontiguousarray(g["cull0_status"]).copy()
    r1, r2 = (float(v) for v in g["cull0_r"])
    assert ia.markDimmerPeaks(x, y, h, st, r1, r2, x.size) == int(g["cull0_dimmer_n"])
    assert numpy.array_equal(st, g["cull0_dimmer"])
    nx, ny = (numpy.ascontiguousarray(a) for a in g["cull0_new"])
    kd = ia.createKDTree(nx, ny, nx.size)
    d = numpy.zeros(x.size)
    ix = numpy.zeros(x.size, dtype=numpy.int32)
    ia.nearestKDTree(kd, x, y, d, ix, r2, x.size)
    ia.freeKDTree(kd)
    assert numpy.array_equal(d, g["cull0_nearest_d"]) and numpy.array_equal(ix, g["cull0_nearest_i"])


def test_find_fit_loop_matches_oracle():
    """The whole 3D-DAOSTORM frame analysis (PeakFinderFitter.analyzeImage:
    background, finder passes with the threshold count-down, fits, culling,
    removal of unconverged peaks) on the GPU equals the oracle's loop: the
    FP64 engine gives the same peaks to 1e-6 px; the FP32 engine the same
    count within 1 % and matched peaks within 1e-3 px."""
    from sa_gb300 import find_peaks, synth
    from oracle import analysis
    P = dict(PARAMS, model="3d")
    wl = synth.make_workload(1, frames=1, nx=128, ny=128, seed=21)
    ref = analysis.analyze_frame(P, wl["images"][0], [0.75, 7.5])
    assert ref["x"].size > 100
    ff = find_peaks.initFindAndFit(P, precision=64)
    got = ff.analyzeFrame(wl["images"][0])
    ff.cleanUp()
    assert got["x"].size == ref["x"].size
    assert numpy.abs(got["x"] - ref["x"]).max() < 1e-6 and numpy.abs(got["y"] - ref["y"]).max() < 1e-6
    assert numpy.abs(got["height"] / ref["height"] - 1.0).max() < 1e-6
    ff = find_peaks.initFindAndFit(P, precision=32)
    got = ff.analyzeFrame(wl["images"][0])
    ff.cleanUp()
    assert abs(got["x"].size - ref["x"].size) <= max(1, ref["x"].size // 100)
    d2 = (got["x"][:, None] - ref["x"][None, :]) ** 2 + (got["y"][:, None] - ref["y"][None, :]) ** 2
    near = numpy.sqrt(d2.min(axis=1))
    assert numpy.mean(near < 1e-3) >= 0.99


def test_batched_find_fit_loop_matches_single_frames_and_oracle():
    """BatchFindFit (three frames at once, fits and finder state on the GPU
    across passes) returns exactly what the one-frame GPU loop returns for
    each frame.  Against the oracle's loop the bar is statistical: the loop
    refits duplicate peaks (two finder peaks on one emitter), whose LM
    steps are ill-conditioned, so a 1e-15 difference in exp / log can end
    such a pair differently, and the neighbours refitted in later passes
    then part too (seed 31, frame 0: identical to 1e-9 through the first fit
    of pass 2, apart after its refit).  The bar: counts within 2 %, at least
    half of the oracle's peaks identical to 1e-3 px and 90 % within 0.5 px
    (the same emitters found)."""
    from sa_gb300 import find_peaks, synth
    from oracle import analysis
    P = dict(PARAMS, model="3d")
    wl = synth.make_workload(1, frames=3, nx=128, ny=128, seed=31)
    frames = numpy.stack(wl["images"])
    bf = find_peaks.BatchFindFit(P, frames.shape[1:], 3, precision=64)
    got = bf.analyze(frames)
    bf.cleanUp()
    for k in range(3):
        ff = find_peaks.initFindAndFit(P, precision=64)
        one = ff.analyzeFrame(frames[k])
        ff.cleanUp()
        for key in ("x", "y", "height", "background", "xsigma", "ysigma"):
            assert numpy.array_equal(got[k][key], one[key]), (k, key)
        ref = analysis.analyze_frame(P, frames[k], [0.75, 7.5])
        n, nr = got[k]["x"].size, ref["x"].size
        assert nr > 50 and abs(n - nr) <= max(2, nr // 50), (k, n, nr)
        d2 = (ref["x"][:, None] - got[k]["x"][None, :]) ** 2 + (ref["y"][:, None] - got[k]["y"][None, :]) ** 2
        near = numpy.sqrt(d2.min(axis=1))
        assert numpy.mean(near < 1e-3) >= 0.5 and numpy.mean(near < 0.5) >= 0.9, (k, numpy.mean(near < 1e-3))


class RotatedGaussianPSF(object):
    """A PSF object with the reference's interface (getMargin, isValidZ,
    getScaledZ, getPSF): an elliptical Gaussian rotated by 30 degrees whose
    widths change with z, cut to 17 x 17 pixels -- not separable, so the
    matched filters take the direct 2D path."""

    def getMargin(self):
        return 10

    def isValidZ(self, z):
        return -500.0 <= z <= 500.0

    def getScaledZ(self, z):
        return (z + 500.0) / 100.0

    def getPSF(self, z, shape=None, normalize=False):
        sx, sy = 1.2 + 0.002 * abs(z), 1.8 - 0.001 * z
        yy, xx = numpy.mgrid[0:shape[0], 0:shape[1]]
        dx, dy = xx - 0.5 * shape[1], yy - 0.5 * shape[0]
        c, s = numpy.cos(numpy.pi / 6), numpy.sin(numpy.pi / 6)
        u, v = c * dx + s * dy, -s * dx + c * dy
        psf = numpy.exp(-(u * u / (2 * sx * sx) + v * v / (2 * sy * sy)))
        psf[(numpy.abs(dx) > 8) | (numpy.abs(dy) > 8)] = 0.0
        return psf / psf.sum() if normalize else psf


def test_arbitrary_psf_finder_matches_oracle():
    """PeakFinderArbitraryPSF (three z planes, non-separable PSFs, |fit| in
    the variance, maxima over the planes) returns the oracle's peaks."""
    from sa_gb300 import fitting, matched_filter_c
    params = dict(PARAMS, z_value=[-0.2, 0.0, 0.2])
    params.pop("foreground_sigma")
    psf = RotatedGaussianPSF()
    wl = _frames(1, size=128, seed=17)
    gf = fitting.PeakFinderArbitraryPSF(params, psf)
    of = F.PeakFinderArbitraryPSF(params, psf)
    img = gf.padArray(wl["images"][0])
    fit = [numpy.zeros(img.shape), 0.3 * img - 20.0]
    total = 0
    for f in (gf, of):
        f.newImage(img)
    for k in range(2):
        bg_g = gf.estimateBackground(fit[k])
        bg_o = of.estimateBackground(fit[k])
        assert conv_close(bg_g, bg_o)
        pg, tg, dg = gf.findPeaks(fit[k])
        po, to, do = of.findPeaks(fit[k])
        assert dg == do
        for key in ("x", "y", "z"):
            assert numpy.array_equal(pg[key], po[key]), (k, key)
        sg = gf.significance()
        for z in range(3):
            assert conv_close(sg[z], of.last_masked[z])
        total += pg["x"].size
    assert gf.fg_mfilter[0].info()[0] == 0 and total > 10
    assert set(numpy.unique(pg["z"])) <= set(of.z_values)
    gf.cleanUp()


def test_spliner_find_fit_loop_matches_oracle():
    """Spliner's whole frame analysis (arbitrary-PSF finder on three z
    planes of the spline PSF, cubic spline fitter, culling with the PSF-size
    neighbourhood) on the GPU against the oracle's loop: same peak count
    within 2 and 90 % of the peaks within 1e-4 px (x, y) and 1e-3 (z)."""
    from sa_gb300 import cubic_fit_c, find_peaks, synth
    from oracle import analysis
    wl = synth.make_workload(3, frames=1, nx=128, ny=128, seed=5, n_emitters=60)
    sp = wl["spline"]
    spline = cubic_fit_c.SplinePSF(coeff=sp["coeff"], zmin=synth.SPLINE_ZMIN_NM, zmax=synth.SPLINE_ZMAX_NM)
    P = dict(background_sigma=8.0, find_max_radius=5, iterations=20, sigma=1.5, threshold=6.0,
             z_value=[-0.2, 0.0, 0.2])
    ref = analysis.analyze_frame(P, wl["images"][0], None, psf_object=spline, spline=sp["coeff"])
    ff = find_peaks.initFindAndFitSpline(P, spline_fn=spline, precision=64)
    got = ff.analyzeFrame(wl["images"][0])
    ff.cleanUp()
    assert ref["x"].size > 40 and abs(got["x"].size - ref["x"].size) <= 2
    d2 = (ref["x"][:, None] - got["x"][None, :]) ** 2 + (ref["y"][:, None] - got["y"][None, :]) ** 2
    j = d2.argmin(axis=1)
    near = numpy.sqrt(d2[numpy.arange(ref["x"].size), j])
    zr = numpy.array([spline.rescaleZ(z) for z in ref["z"]])
    ok = (near < 1e-4) & (numpy.abs(got["z"][j] - zr) < 1e-3)
    assert numpy.mean(ok) >= 0.9
