"""The FFT PSF fitter (psf_fft/fft_fit.c) on the GPU against the oracle.

The reference's fft_fit.c and psf_fft.c need FFTW (not installed), so the
fits are compared with the oracle's FP64 restatement (oracle/sa_oracle.c,
its FFT PSF evaluation pinned to the reference's own psf_fft_py.py by
tests/test_psf_fft_cpu.py).  The same images, backgrounds and starting
peaks go to both; the engine runs the FFT model in its FP64 path.  Bar:
every status equal, iterations equal, positions within 1e-7 px, z within
1e-7 z pixels, height and background within 1e-7 relative; "testing"
peaks, which start at height 1, are held to >= 90 % equal statuses and
>= 70 % of the peaks converged in both within the spec bar.  The library's
z property is in z pixel units, as the reference's (the caller converts
with the PSF object's rescaleZ)."""
import numpy
import pytest

pytestmark = pytest.mark.gpu


def make_case(seed, n_peaks, shape=(96, 104), psf_shape=(17, 20), ptype="hdf5", background=10.0):
    """An image of n_peaks FFT-PSF emitters (the oracle's model, Poisson
    noise) and starting peaks: for "hdf5" perturbed truth, for "finder" /
    "testing" rounded positions at z = 0."""
    from oracle import oracle, psf_fft as opf
    psf = opf.test_psf(psf_shape[0], psf_shape[1], seed=3)
    rng = numpy.random.default_rng(seed)
    ny, nx = shape
    ref = oracle.OracleFitter("fft", shape, psf=psf)
    xoff, yoff = opf.fit_psf_offsets(psf.shape)
    img = numpy.full(shape, background)
    truth = []
    size = psf.shape[1]
    for _ in range(n_peaks):
        x, y, z = rng.uniform(size, nx - size), rng.uniform(size, ny - size), rng.uniform(-3.0, 3.0)
        h = rng.uniform(3000.0, 20000.0)
        px, py = x - xoff, y - yoff
        xi, yi = int(numpy.floor(px)), int(numpy.floor(py))
        g = oracle.fft_eval(ref, px - xi, py - yi, z)[0]
        img[yi:yi + size, xi:xi + size] += h * g
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
    return psf, img, bg, peaks


def fit_both(psf, img, bg, peaks, ptype, max_iterations=200, rqe=None, scmos=None, precision=64):
    from oracle import oracle
    from sa_gb300 import fft_fit_c, psf_fft_c
    ref = oracle.OracleFitter("fft", img.shape, psf=psf, rqe=rqe, scmos_cal=scmos)
    ref.newImage(img)
    ref.newBackground(bg)
    ref.newPeaks(peaks, ptype)
    ref.doFit(max_iterations)
    fn = psf_fft_c.PSFFnBase(psf_data={"psf": psf, "pixel_size": 100.0, "zmin": -800.0, "zmax": 800.0})
    gpu = fft_fit_c.CFFTFit(psf_fn=fn, rqe=rqe, scmos_cal=scmos, precision=precision)
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
    # a PSF of even x / y size 16 and 21 planes, sCMOS calibration and RQE
    dict(seed=5, n_peaks=20, ptype="hdf5", psf_shape=(21, 16), calibration=True),
    # a handle asked for the FP32 engine runs the FFT model in FP64 all the same
    dict(seed=6, n_peaks=12, ptype="hdf5", precision=32),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: "seed%d-%s" % (c["seed"], c["ptype"]))
def test_fft_fit_matches_oracle(case):
    case = dict(case)
    ptype = case["ptype"]
    calibration = case.pop("calibration", False)
    precision = case.pop("precision", 64)
    psf, img, bg, peaks = make_case(case["seed"], case["n_peaks"], ptype=ptype,
                                    psf_shape=case.get("psf_shape", (17, 20)))
    rqe = scmos = None
    if calibration:
        rng = numpy.random.default_rng(case["seed"] + 100)
        rqe = rng.uniform(0.8, 1.2, img.shape)
        scmos = rng.uniform(0.5, 3.0, img.shape)
    out = fit_both(psf, img, bg, peaks, ptype, rqe=rqe, scmos=scmos, precision=precision)
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
    for name in ("x", "y"):
        a, b = out[name]
        assert numpy.abs(a[ok] - b[ok]).max() < 1.0e-7, name
    a, b = out["z"]   # z pixel units in both (rescaleZ is the caller's)
    assert numpy.abs(a[ok] - b[ok]).max() < 1.0e-7
    for name in ("height", "background"):
        a, b = out[name]
        assert (numpy.abs(a[ok] - b[ok]) / numpy.abs(a[ok])).max() < 1.0e-7, name
