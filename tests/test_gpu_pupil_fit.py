"""The pupil-function fitter (pupilfn/pupil_fit.c) on the GPU against the
oracle.

The reference's pupil_fit.c and pupil_function.c need FFTW (not
installed), so the fits are compared with the oracle's FP64 restatement
(oracle/sa_oracle.c, its pupil-function evaluation pinned to the
reference's own Python pupil math by tests/test_pupilfn_cpu.py).  The same
images, backgrounds and starting peaks go to both; the engine runs the
pupil model in its FP64 path.  Bar: every status equal, iterations equal,
positions within 1e-7 px, z within 1e-7 um, height and background within
1e-7 relative; "testing" peaks, which start at height 1, are held to
>= 90 % equal statuses and >= 70 % of the peaks converged in both within
the spec bar."""
import os
import sys

import numpy
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "storm-analysis_gb300"))


def geometry_arrays(pf_data):
    from sa_gb300 import pupil_math
    cls = pupil_math.GeometrySim if pf_data["geo_sim_pf"] else pupil_math.Geometry
    n = pf_data["pf"].shape[0]
    geo = cls(n, pf_data["pixel_size"], pf_data["wavelength"], pf_data["immersion_index"],
              pf_data["numerical_aperture"])
    return geo.kx, geo.ky, numpy.real(geo.kz), pf_data["pf"]


def make_case(seed, n_peaks, shape=(100, 108), size=20, ptype="hdf5", background=10.0):
    """An image of n_peaks pupil-function emitters (the oracle's model,
    Poisson noise) and starting peaks: for "hdf5" perturbed truth, for
    "finder" / "testing" rounded positions at z = 0."""
    from oracle import oracle
    from sa_gb300 import synth
    pf_data = synth.pupil_function_data(size=size, seed=seed)
    arrays = geometry_arrays(pf_data)
    rng = numpy.random.default_rng(seed)
    ny, nx = shape
    ref = oracle.OracleFitter("pupil", shape, pupil=arrays)
    off = 0.5 * size
    img = numpy.full(shape, background)
    truth = []
    for _ in range(n_peaks):
        x, y, z = rng.uniform(size, nx - size), rng.uniform(size, ny - size), rng.uniform(-0.4, 0.4)
        h = rng.uniform(3000.0, 20000.0)
        px, py = x - off, y - off
        xi, yi = int(numpy.floor(px)), int(numpy.floor(py))
        p = oracle.pupil_eval(ref, px - xi, py - yi, z)[0]
        # the pupil's first index is the image's x
        img[yi:yi + size, xi:xi + size] += h * (p.real * p.real + p.imag * p.imag).T
        truth.append((x, y, z, h))
    ref.cleanup()
    truth = numpy.array(truth)
    img = rng.poisson(img).astype(numpy.float64)
    bg = numpy.full(shape, background)
    if ptype == "hdf5":
        peaks = {"x": truth[:, 0] + rng.normal(0, 0.3, n_peaks), "y": truth[:, 1] + rng.normal(0, 0.3, n_peaks),
                 "z": truth[:, 2] * 0.5, "background": numpy.full(n_peaks, background),
                 "height": truth[:, 3] * 0.8}
    else:
        peaks = {"x": numpy.round(truth[:, 0]), "y": numpy.round(truth[:, 1]), "z": numpy.zeros(n_peaks)}
    return pf_data, img, bg, peaks


def fit_both(pf_data, img, bg, peaks, ptype, max_iterations=200, rqe=None, scmos=None, precision=64,
             zrange=(-500.0, 500.0)):
    from oracle import oracle
    from sa_gb300 import pupil_fit_c, pupil_fn
    ref = oracle.OracleFitter("pupil", img.shape, pupil=geometry_arrays(pf_data), rqe=rqe, scmos_cal=scmos,
                              min_z=zrange[0], max_z=zrange[1])
    ref.newImage(img)
    ref.newBackground(bg)
    ref.newPeaks(peaks, ptype)
    ref.doFit(max_iterations)
    fn = pupil_fn.PupilFunction(pf_data=pf_data, zmin=zrange[0], zmax=zrange[1])
    gpu = pupil_fit_c.CPupilFit(pupil_fn=fn, rqe=rqe, scmos_cal=scmos, precision=precision)
    gpu.initializeC(img)
    gpu.newImage(img)
    gpu.newBackground(bg)
    gpu.newPeaks(peaks, ptype)
    gpu.doFit(max_iterations)
    out = {}
    for name in ("x", "y", "z", "height", "background", "status", "iterations"):
        out[name] = (ref.getPeakProperty(name), gpu.getPeakProperty(name))
    ref.cleanup()
    gpu.cleanup(verbose=False)
    fn.cleanup()
    return out


CASES = [
    dict(seed=1, n_peaks=12, ptype="hdf5"),
    dict(seed=2, n_peaks=30, ptype="hdf5"),
    dict(seed=3, n_peaks=16, ptype="finder"),
    dict(seed=4, n_peaks=16, ptype="testing"),
    # the diagnostics' 30-pixel pupil, sCMOS calibration and RQE
    dict(seed=5, n_peaks=16, ptype="hdf5", size=30, calibration=True),
    # a tight z range: pfitZRangeCheck clamps
    dict(seed=6, n_peaks=12, ptype="hdf5", zrange=(-0.1, 0.1)),
    # a handle asked for the FP32 engine runs the pupil model in FP64 all the same
    dict(seed=7, n_peaks=12, ptype="hdf5", precision=32),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: "seed%d-%s" % (c["seed"], c["ptype"]))
def test_pupil_fit_matches_oracle(case):
    case = dict(case)
    ptype = case["ptype"]
    calibration = case.pop("calibration", False)
    precision = case.pop("precision", 64)
    zrange = case.pop("zrange", (-500.0, 500.0))
    size = case.get("size", 20)
    shape = (100, 108) if size <= 20 else (130, 124)
    pf_data, img, bg, peaks = make_case(case["seed"], case["n_peaks"], shape=shape, size=size, ptype=ptype)
    rqe = scmos = None
    if calibration:
        rng = numpy.random.default_rng(case["seed"] + 100)
        rqe = rng.uniform(0.8, 1.2, img.shape)
        scmos = rng.uniform(0.5, 3.0, img.shape)
    out = fit_both(pf_data, img, bg, peaks, ptype, rqe=rqe, scmos=scmos, precision=precision, zrange=zrange)
    st_ref, st_gpu = out["status"]
    if ptype == "testing":
        # "testing" peaks start at height 1 and z 0, far from the solution:
        # the first steps are ill-conditioned, and the last-bit differences
        # of the two FP64 evaluations (sum orders, the device's and the host
        # library's sine and cosine) can send a peak to another local
        # minimum, as on the reference's own g_2d_testing golden.  Held to
        # >= 90 % equal statuses and >= 70 % of the peaks converged in both
        # within the spec bar.
        assert (st_ref == st_gpu).mean() >= 0.9
        both = (st_ref == 1) & (st_gpu == 1)
        within = both.copy()
        for name, tol in (("x", 1.0e-4), ("y", 1.0e-4), ("z", 1.0e-3)):
            a, b = out[name]
            within &= numpy.abs(a - b) < tol
        for name in ("height", "background"):
            a, b = out[name]
            within &= numpy.abs(a - b) < 1.0e-4 * numpy.abs(a)
        assert within.sum() >= 0.7 * both.sum()
        return
    assert numpy.array_equal(st_ref, st_gpu)
    assert numpy.array_equal(out["iterations"][0], out["iterations"][1])
    ok = st_ref != 2
    assert ok.sum() >= 5
    for name in ("x", "y", "z"):
        a, b = out[name]
        assert numpy.abs(a[ok] - b[ok]).max() < 1.0e-7, name
    if zrange[1] < 1.0:
        z = out["z"][1][st_gpu == 1]
        assert (z >= zrange[0]).all() and (z <= zrange[1]).all()
    for name in ("height", "background"):
        a, b = out[name]
        assert (numpy.abs(a[ok] - b[ok]) / numpy.abs(a[ok])).max() < 1.0e-7, name
