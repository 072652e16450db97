"""
Generate the golden fixtures in tests/golden/ by running the REFERENCE's
own fitting C code (compiled from its sources by ``make -C oracle ref``)
on small seeded synthetic inputs.

Run here, where the reference tree exists:

    make -C oracle ref
    python tests/golden/make_golden.py

Each fixture stores the exact inputs the reference consumed (images are
rounded to float32 and then fed as float64, so the stored values are the
consumed values) and the reference's outputs after doFit.  The CPU tests
check the oracle restatement against these files, which pins it on
machines where the reference is absent.
"""
import os
import sys

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "storm-analysis_gb300"))

from oracle import ref_driver  # noqa: E402
from sa_gb300 import synth  # noqa: E402

PROPS = ["x", "y", "z", "height", "background", "xsigma", "ysigma", "status", "iterations",
         "error", "significance", "sum"]


def f32(a):
    return numpy.asarray(a, dtype=numpy.float32).astype(numpy.float64)


def small_spline(knots, seed):
    rng = numpy.random.default_rng(1000 + seed)
    coef = rng.normal(0.0, 1.0, 6)
    half = (knots - 1) / 2.0
    a = numpy.arange(knots) - half
    zs = synth.SPLINE_ZMIN_NM + numpy.arange(knots) * (synth.SPLINE_ZMAX_NM - synth.SPLINE_ZMIN_NM) / (knots - 1)
    X, Y, Z = numpy.meshgrid(a, a, zs * 1.0e-3, indexing="ij")
    return synth.tricubic_coefficients(synth._aberrated_psf(X, Y, Z, coef))


def run_case(name, model, image, bg, peaks, ptype, kw, rqe=None, scmos=None, spline=None,
             max_it=200, sweeps_only=None, store_spline=True):
    shape = image.shape
    ref = ref_driver.RefFitter(model, shape, rqe=rqe, scmos_cal=scmos, spline=spline, **kw)
    ref.newImage(image)
    ref.newBackground(bg)
    ref.newPeaks(peaks, ptype)
    init = {p: ref.getPeakProperty(p) for p in ["height", "background", "error", "status"]}
    if sweeps_only is None:
        nsweeps = ref.doFit(max_it)
    else:
        for _ in range(sweeps_only):
            ref.iterate()
        nsweeps = sweeps_only
    out = {p: ref.getPeakProperty(p) for p in PROPS}
    fimg = ref.getFitImage()
    ctr = ref.counters()
    ref.cleanup()
    rec = dict(model=model, ptype=ptype, image=image.astype(numpy.float32), bg=bg.astype(numpy.float32),
               nsweeps=nsweeps, max_it=max_it, fit_sum=fimg.sum(), fit_sq=(fimg * fimg).sum(),
               counters=numpy.array([ctr[k] for k in ["n_dposv", "n_iterations", "n_lost", "n_margin",
                                                      "n_neg_fi", "n_neg_height", "n_non_converged",
                                                      "n_non_decr"]]))
    for k, v in kw.items():
        if v is not None:
            rec["kw_" + k] = numpy.asarray(v)
    for k, v in peaks.items():
        rec["in_" + k] = numpy.asarray(v)
    for k, v in init.items():
        rec["init_" + k] = v
    for k, v in out.items():
        rec["out_" + k] = v
    if rqe is not None:
        rec["rqe"] = rqe.astype(numpy.float32)
    if scmos is not None:
        rec["scmos"] = scmos.astype(numpy.float32)
    if spline is not None and store_spline:
        rec["spline"] = spline.astype(numpy.float32)
    numpy.savez_compressed(os.path.join(HERE, name + ".npz"), **rec)
    print(name, "peaks", out["x"].size, "status", numpy.bincount(out["status"], minlength=3),
          "sweeps", nsweeps)


def gaussian_case(name, cfg, model, n, size, seed, ptype="hdf5", rqe_var=False, kw_override=None):
    wl = synth.make_workload(cfg, frames=1, nx=size, ny=size, seed=seed, n_emitters=n)
    kw = dict(wl["fitter"])
    kw.pop("model")
    if kw_override:
        kw.update(kw_override)
    image = f32(wl["images"][0])
    bg = f32(wl["backgrounds"][0])
    scmos = f32(wl["scmos_cal"]) if cfg == 2 else None
    rqe = None
    if rqe_var:
        rqe = f32(numpy.random.default_rng(seed + 7).uniform(0.8, 1.2, image.shape))
    g = {k: f32(v) for k, v in wl["guesses"][0].items()}
    if ptype in ("finder", "testing"):
        g = {"x": g["x"], "y": g["y"], "z": g["z"], "sigma": g["xsigma"]}
    run_case(name, model, image, bg, g, ptype, kw, rqe=rqe, scmos=scmos)


SPLINE_SEED = 5


def spline_case(name, n, size, seed, knots=9, ptype="hdf5"):
    coeff = f32(small_spline(knots, SPLINE_SEED))
    sp_size = knots - 1
    rng = numpy.random.default_rng(seed)
    half = sp_size // 2
    margin = half + 2
    x = rng.uniform(margin, size - margin - 1, n)
    y = rng.uniform(margin, size - margin - 1, n)
    zs = rng.uniform(1.0, sp_size - 1.0, n)
    h = rng.uniform(1000.0, 4000.0, n)
    # Render with the spline itself via the oracle's point evaluator-free path:
    # evaluate the tricubic at pixel centres (spline coordinate u = col - x + half).
    img = numpy.full((size, size), 20.0)
    for i in range(n):
        cx, cy = int(round(x[i])), int(round(y[i]))
        for r in range(max(0, cy - half + 1), min(size, cy + half)):
            for c in range(max(0, cx - half + 1), min(size, cx + half)):
                u = c - x[i] + half
                v = r - y[i] + half
                if 0.0 <= u < sp_size and 0.0 <= v < sp_size:
                    iu, iv, iz = int(u), int(v), int(zs[i])
                    du, dv, dz = u - iu, v - iv, zs[i] - iz
                    cell = coeff[iu, iv, iz]
                    val = 0.0
                    for a in range(4):
                        for b in range(4):
                            for cc in range(4):
                                val += cell[a * 16 + b * 4 + cc] * du ** a * dv ** b * dz ** cc
                    img[r, c] += h[i] * val
    image = f32(numpy.maximum(rng.poisson(img).astype(numpy.float64), 1.0))
    bg = numpy.full((size, size), 20.0)
    g = {"x": f32(x + rng.normal(0, 0.3, n)), "y": f32(y + rng.normal(0, 0.3, n)),
         "z": f32(zs + rng.normal(0, 0.3, n)), "background": bg[0, :n].copy(),
         "height": f32(h * rng.uniform(0.8, 1.2, n))}
    if ptype in ("finder", "testing"):
        g = {"x": g["x"], "y": g["y"], "z": g["z"]}
    run_case(name, "spline3D", image, bg, g, ptype, {}, spline=coeff, store_spline=False)


def spline_points(name, knots=9, seed=SPLINE_SEED, n=200):
    """Point evaluations of the reference's spline code (test/test_spline.py analogue)."""
    import ctypes
    lib = ctypes.CDLL(os.path.join(ref_driver.REF_DIR, "libcubic_fit.so"))
    coeff = f32(small_spline(knots, seed))
    f64 = numpy.ctypeslib.ndpointer(dtype=numpy.float64, flags="C_CONTIGUOUS")
    lib.initSpline3D.argtypes = [f64, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    lib.initSpline3D.restype = ctypes.c_void_p
    sp = lib.initSpline3D(numpy.ascontiguousarray(coeff.ravel()), knots - 1, knots - 1, knots - 1)
    rng = numpy.random.default_rng(seed)
    pts = rng.uniform(1.0e-6, knots - 1 - 1.0e-6, (n, 3))
    vals = numpy.zeros((n, 4))
    for fi, fname in enumerate(["fSpline3D", "dxfSpline3D", "dyfSpline3D", "dzfSpline3D"]):
        fn = getattr(lib, fname)
        fn.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_double]
        fn.restype = ctypes.c_double
        for i in range(n):
            vals[i, fi] = fn(sp, pts[i, 0], pts[i, 1], pts[i, 2])
    # The spline cases above read their coefficients from this file.
    numpy.savez_compressed(os.path.join(HERE, name + ".npz"), spline=coeff.astype(numpy.float32),
                           points=pts, values=vals)
    print(name, n)


def main():
    if not ref_driver.available():
        raise SystemExit("reference libraries missing: run 'make -C oracle ref' first")
    gaussian_case("g_2d", 0, "2d", 50, 128, 100)
    gaussian_case("g_2dfixed", 0, "2dfixed", 50, 128, 101, kw_override={"sigma_range": None})
    gaussian_case("g_2d_rqe_finder", 0, "2d", 40, 128, 102, ptype="finder", rqe_var=True)
    gaussian_case("g_2d_testing", 0, "2d", 40, 128, 103, ptype="testing")
    gaussian_case("g_3d_dense", 1, "3d", 220, 128, 104)
    gaussian_case("g_Z_scmos", 2, "Z", 60, 96, 105)
    spline_case("g_spline3d", 30, 80, 106)
    spline_case("g_spline3d_finder", 25, 80, 107, ptype="finder")
    spline_points("g_spline_points")


if __name__ == "__main__":
    main()
