"""Multi-plane fitting (multi_plane/mp_fit.c with mp_fit_dao.c and
mp_fit_arb.c) on the GPU.

The 2D Gaussian multi-plane fitter is held to the reference's own compiled
C (tests/golden/g_mp_dao.npz, made by tests/golden/make_golden_mp.py from
mp_fit.c + mp_fit_dao.c): statuses, iterations and counters equal,
parameters within 1e-7.  The arbitrary-PSF multi-plane fitter (whose
reference C needs FFTW through the FFT and pupil fitters' headers) is held
to the oracle's restatement (oracle/sa_oracle.c oraMP*, itself pinned to
the same goldens by tests/test_mp_oracle_cpu.py) on two-plane pupil-
function, FFT-PSF and spline cases: statuses and iterations equal,
positions within 1e-7 px, z within 1e-7 (the model's units), heights and
backgrounds within 1e-7 relative."""
import os
import sys

import numpy
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "storm-analysis_gb300"))
GOLDEN = os.path.join(ROOT, "tests", "golden", "g_mp_dao.npz")
PROPS = ("x", "y", "height", "background", "xsigma", "ysigma", "error")


@pytest.mark.parametrize("n", ["a", "b"])
def test_mp_dao_matches_reference_goldens(n):
    from sa_gb300 import mp_fit_dao_c
    g = numpy.load(GOLDEN)
    imgs = g[n + "_images"]
    nc = imgs.shape[0]
    f = mp_fit_dao_c.MPFitDao2D(n_channels=nc, roi_size=10, sigma_range=(1.0, 3.0))
    for c in range(nc):
        f.initializeChannel(g[n + "_rqe"][c], g[n + "_variance"][c], c)
    f.setMapping(*list(g[n + "_maps"]))
    f.setWeights(verbose=False)
    f.newImage(list(imgs))
    f.newBackground(list(g[n + "_backgrounds"]))
    p = g[n + "_peaks"]
    f.newPeaks({"x": p[:, 0], "y": p[:, 1], "z": p[:, 2], "sigma": p[:, 3]}, "finder")
    f.doFit(200)
    try:
        for c in range(nc):
            key = "%s_c%d_" % (n, c)
            assert numpy.array_equal(f.getPeakProperty("status", c), g[key + "status"])
            assert numpy.array_equal(f.getPeakProperty("iterations", c), g[key + "iterations"])
            fd = f.mfit.contents.fit_data[c].contents
            ctr = [fd.n_dposv, fd.n_iterations, fd.n_lost, fd.n_margin, fd.n_neg_fi, fd.n_neg_height,
                   fd.n_non_converged, fd.n_non_decr]
            # doFit folded n_iterations into the Python counter (getIterations)
            ref = list(g[key + "counters"])
            assert ctr[0] == ref[0] and ctr[2:] == ref[2:]
            for prop in PROPS:
                a, b = f.getPeakProperty(prop, c), g[key + prop]
                assert numpy.abs(a - b).max() <= 1.0e-7 * max(1.0, numpy.abs(b).max()), prop
        assert f.iterations == sum(int(g["%s_c%d_counters" % (n, c)][1]) for c in range(nc))
    finally:
        f.cleanup(verbose=False)


# ---- arbitrary PSFs against the oracle ------------------------------------

def maps2(seed):
    rng = numpy.random.default_rng(seed)
    th, s = rng.uniform(-0.01, 0.01), 1.0 + rng.uniform(-0.003, 0.003)
    a = s * numpy.array([[numpy.cos(th), -numpy.sin(th)], [numpy.sin(th), numpy.cos(th)]])
    t = rng.uniform(-1.5, 1.5, 2)
    ai = numpy.linalg.inv(a)
    ti = -ai @ t
    return (numpy.array([0.0, 1.0, 0.0, t[0], a[0, 0], a[0, 1]]), numpy.array([0.0, 0.0, 1.0, t[1], a[1, 0], a[1, 1]]),
            numpy.array([0.0, 1.0, 0.0, ti[0], ai[0, 0], ai[0, 1]]),
            numpy.array([0.0, 0.0, 1.0, ti[1], ai[1, 0], ai[1, 1]]))


def oracle_channel(kind, obj, shape, rqe=None, scmos=None, tol=1.0e-6, zr=None):
    from oracle import oracle
    if kind == "pupil":
        return oracle.OracleFitter("pupil", shape, pupil=obj, rqe=rqe, scmos_cal=scmos, tol=tol,
                                   min_z=zr[0], max_z=zr[1])
    if kind == "fft":
        return oracle.OracleFitter("fft", shape, psf=obj, rqe=rqe, scmos_cal=scmos, tol=tol)
    return oracle.OracleFitter("spline3D", shape, spline=obj, rqe=rqe, scmos_cal=scmos, tol=tol)


def render(kind, obj, shape, rows, zr):
    """The channel's model image of peaks given as "text" rows (x, y, z,
    background 0, height), from the oracle's fit image."""
    f = oracle_channel(kind, obj, shape, zr=zr)
    f.newImage(numpy.ones(shape))
    f.newBackground(numpy.zeros(shape))
    f.newPeaks({"x": rows[:, 0], "y": rows[:, 1], "z": rows[:, 2], "background": rows[:, 3],
                "height": rows[:, 4]}, "text")
    img = f.getFitImage()
    f.cleanup()
    return img


def make_arb_case(kind, seed, n_peaks=10, shape=(96, 100), indep=0):
    from sa_gb300 import pupil_math, synth
    rng = numpy.random.default_rng(seed)
    maps = maps2(seed + 1)
    if kind == "pupil":
        pf_data = synth.pupil_function_data(size=20, seed=seed)
        geo = pupil_math.Geometry(20, pf_data["pixel_size"], 0.6, 1.5, 1.4)
        objs = []
        for c, dz in enumerate((0.0, 0.3)):
            pf = geo.changeFocus(pf_data["pf"], -dz)
            objs.append((geo.kx, geo.ky, numpy.real(geo.kz), pf))
        zs = rng.uniform(-0.3, 0.3, n_peaks)
        zr = (-0.6, 0.6)
        pos_margin = 12
    elif kind == "fft":
        from oracle import psf_fft as opf
        objs = [opf.test_psf(17, 20, seed=3), opf.test_psf(17, 20, seed=9)[:, ::-1, :].copy()]
        zs = rng.uniform(-3.0, 3.0, n_peaks)
        zr = None
        pos_margin = 12
    else:
        objs = [synth.make_spline(seed=3)["coeff"]] * 2
        size = objs[0].shape[0]
        zs = numpy.floor(rng.uniform(0.25 * size, 0.75 * size, n_peaks)) + rng.uniform(0.3, 0.6, n_peaks)
        zr = None
        pos_margin = 14
    # the test spline has small negative lobes: a background that keeps the
    # model positive
    bg = 80.0 if kind == "spline" else 15.0
    ny, nx = shape
    x = rng.uniform(pos_margin, nx - pos_margin, n_peaks)
    y = rng.uniform(pos_margin, ny - pos_margin, n_peaks)
    h = rng.uniform(2000.0, 8000.0, n_peaks)
    images = []
    for c in range(2):
        cx = maps[0][3 * c] + maps[0][3 * c + 1] * x + maps[0][3 * c + 2] * y
        cy = maps[1][3 * c] + maps[1][3 * c + 1] * x + maps[1][3 * c + 2] * y
        rows = numpy.stack([cx, cy, zs, numpy.zeros(n_peaks), h], axis=1)
        img = bg + render(kind, objs[c], shape, rows, zr)
        images.append(rng.poisson(numpy.clip(img, 0.0, None)).astype(numpy.float64))
    bgs = [numpy.full(shape, bg) for _ in range(2)]
    # spline z starts near the truth (the test spline's z response is not
    # monotonic far from it); the others at 70 % of it
    z0 = zs + rng.uniform(0.15, 0.35, n_peaks) if kind == "spline" else 0.7 * zs
    peaks = {"x": x + rng.normal(0.0, 0.3, n_peaks), "y": y + rng.normal(0.0, 0.3, n_peaks), "z": z0,
             "background": numpy.full(n_peaks, bg), "height": 0.8 * h}
    return objs, maps, images, bgs, peaks, zr


def gpu_psf_objects(kind, objs, zr):
    from sa_gb300 import cubic_fit_c, psf_fft_c, pupil_fn, pupil_function_c

    class Pupil(object):
        def __init__(self, arrays):
            class Geo(object):
                pass
            geo = Geo()
            geo.size = arrays[0].shape[0]
            geo.kx, geo.ky, geo.kz = arrays[0], arrays[1], arrays[2]
            self.c = pupil_function_c.PupilFunction(geometry=geo)
            self.c.setPF(arrays[3])

        def getCPointer(self):
            return self.c.getCPointer()

        def getSize(self):
            return self.c.size

        def getZMin(self):
            return zr[0] * 1.0e3

        def getZMax(self):
            return zr[1] * 1.0e3

        def cleanup(self):
            self.c.cleanup()

    if kind == "pupil":
        return [Pupil(o) for o in objs]
    if kind == "fft":
        return [psf_fft_c.PSFFnBase(psf_data={"psf": o, "pixel_size": 100.0, "zmin": -800.0, "zmax": 800.0})
                for o in objs]
    return [cubic_fit_c.SplinePSF(coeff=o) for o in objs]


ARB_CASES = [
    dict(kind="pupil", seed=1, indep=0, ptype="hdf5"),
    dict(kind="pupil", seed=2, indep=1, ptype="hdf5"),
    dict(kind="pupil", seed=3, indep=0, ptype="finder"),
    dict(kind="fft", seed=4, indep=0, ptype="hdf5"),
    dict(kind="spline", seed=5, indep=0, ptype="hdf5"),
    dict(kind="spline", seed=6, indep=1, ptype="finder"),
]


@pytest.mark.parametrize("case", ARB_CASES, ids=lambda c: "%s-seed%d-indep%d-%s" % (c["kind"], c["seed"],
                                                                                        c["indep"], c["ptype"]))
def test_mp_arb_matches_oracle(case):
    from oracle import oracle
    from sa_gb300 import mp_fit_arb_c
    kind, indep, ptype = case["kind"], case["indep"], case["ptype"]
    objs, maps, images, bgs, peaks, zr = make_arb_case(kind, case["seed"], indep=indep)
    shape = images[0].shape
    if ptype != "hdf5":
        # (spline z off the knots: at a knot the test spline's z gradient can
        # vanish, a singular Hessian whose solve fails or not by rounding)
        peaks = {"x": numpy.round(peaks["x"]), "y": numpy.round(peaks["y"]),
                 "z": numpy.full(peaks["x"].size, 0.0 if kind != "spline" else 0.5 * objs[0].shape[0] + 0.37)}
    # oracle
    chans = [oracle_channel(kind, o, shape, tol=1.0e-6 * 2, zr=zr) for o in objs]
    ref = oracle.OracleMPFitter(chans, maps, kind="arb", independent_heights=indep)
    ref.newImage(images)
    ref.newBackground(bgs)
    ref.newPeaks(peaks, ptype)
    # the test spline leaves some peaks oscillating (in the oracle as in a
    # single-plane fit of the same frames): compare their trajectories over
    # 20 sweeps
    max_it = 20 if kind == "spline" else 200
    ref.doFit(max_it)
    # GPU
    psfs = gpu_psf_objects(kind, objs, zr)
    cls = {"pupil": mp_fit_arb_c.MPPupilFnFit, "fft": mp_fit_arb_c.MPPSFFnFit, "spline": mp_fit_arb_c.MPSplineFit}
    gpu = cls[kind](independent_heights=indep, psf_objects=psfs)
    for c in range(2):
        gpu.initializeChannel(numpy.ones(shape), numpy.zeros(shape), c)
    gpu.setMapping(*maps)
    gpu.setWeights(None, verbose=False)
    gpu.newImage(images)
    gpu.newBackground(bgs)
    gpu.newPeaks(peaks, ptype)
    gpu.doFit(max_it)
    try:
        for c in range(2):
            st_ref, st_gpu = ref.getPeakProperty("status", c), gpu.getPeakProperty("status", c)
            assert numpy.array_equal(st_ref, st_gpu), c
            assert numpy.array_equal(ref.getPeakProperty("iterations", c), gpu.getPeakProperty("iterations", c))
            ok = st_ref != 2
            assert ok.sum() >= 3
            for prop in ("x", "y", "z"):
                a, b = ref.getPeakProperty(prop, c), gpu.getPeakProperty(prop, c)
                assert numpy.abs(a[ok] - b[ok]).max() < 1.0e-7, (c, prop)
            for prop in ("height", "background"):
                a, b = ref.getPeakProperty(prop, c), gpu.getPeakProperty(prop, c)
                assert (numpy.abs(a[ok] - b[ok]) / numpy.abs(a[ok])).max() < 1.0e-7, (c, prop)
            if not indep:
                hs = gpu.getPeakProperty("height", c)
                assert numpy.array_equal(hs, gpu.getPeakProperty("height", 0))
    finally:
        ref.cleanup()
        gpu.cleanup(verbose=False)
        for p in psfs:
            if hasattr(p, "cleanup"):
                p.cleanup()


@pytest.mark.parametrize("teams", [0, 1, 3])
def test_mp_batch_equals_single_frames(teams):
    """mpSetFrames / mpNewPeaksBatch / mpDoFitBatch on three frames give
    every frame's results bit for bit as the one-frame calls do (those step
    up to 8 groups of a frame at once), whatever number of groups the batch
    steps at once (mpSetTeams; 0 chooses it from the frame count)."""
    from sa_gb300 import mp_fit_dao_c, synth
    wls = [synth.multiplane_workload(nx=96, ny=104, n_emitters=25, seed=s) for s in (41, 42, 43)]
    shape = (wls[0]["ny"], wls[0]["nx"])
    nc = wls[0]["n_channels"]
    maps = wls[0]["maps"]

    def make():
        f = mp_fit_dao_c.MPFitDao2D(n_channels=nc, roi_size=10, sigma_range=(1.0, 3.0))
        for c in range(nc):
            f.initializeChannel(numpy.ones(shape), numpy.zeros(shape), c)
        f.setMapping(*maps)
        f.setWeights(verbose=False)
        return f

    single = []
    for wl in wls:
        f = make()
        f.newImage(wl["images"])
        f.newBackground(wl["backgrounds"])
        f.newPeaks(wl["peaks"], "finder")
        f.doFit(200)
        single.append([{k: f.getPeakProperty(k, c) for k in ("x", "y", "height", "background", "xsigma", "status",
                                                             "iterations")} for c in range(nc)])
        f.cleanup(verbose=False)
    f = make()
    assert f.clib.mpSetTeams(f.mfit, teams) == 0
    images = [numpy.stack([wl["images"][c] for wl in wls]) for c in range(nc)]
    bgs = [numpy.stack([wl["backgrounds"][c] for wl in wls]) for c in range(nc)]
    out, sweeps = f.fitBatch(images, bgs, [wl["peaks"] for wl in wls], "finder", max_iterations=200)
    f.cleanup(verbose=False)
    assert sweeps >= 1
    for c in range(nc):
        o = 0
        for fr, wl in enumerate(wls):
            n = single[fr][c]["x"].size
            for k in ("x", "y", "height", "background", "xsigma", "status", "iterations"):
                assert numpy.array_equal(out[c][k][o:o + n], single[fr][c][k]), (c, fr, k)
            o += n
