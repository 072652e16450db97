"""Golden vectors of the reference's multi-plane fitter with 2D Gaussians
(multi_plane/mp_fit.c + mp_fit_dao.c, compiled from its sources by
``make -C oracle ref`` into oracle/_ref/libmp_fit_dao.so), driven as the
reference's MPFitDao2D drives it (oracle/ref_driver.py RefMPDaoFitter).

    python tests/golden/make_golden_mp.py

Writes tests/golden/g_mp_dao.npz: two cases (two and three planes, one
with sCMOS calibration), their images, backgrounds, calibration, affine
maps, starting peaks and, per channel, the fitted x, y, height, background,
x / y sigma, error, status, iterations and the fitter's counters."""
import os
import sys

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import ref_driver  # noqa: E402

SHAPE = (72, 80)


def affine(nc, seed):
    """Channel 0 the identity; the others a small rotation / scale and a
    shift, with their exact inverses."""
    rng = numpy.random.default_rng(seed)
    x0N, y0N, xN0, yN0 = [], [], [], []
    for c in range(nc):
        if c == 0:
            a = numpy.array([[1.0, 0.0], [0.0, 1.0]])
            t = numpy.zeros(2)
        else:
            th = rng.uniform(-0.01, 0.01)
            s = 1.0 + rng.uniform(-0.004, 0.004)
            a = s * numpy.array([[numpy.cos(th), -numpy.sin(th)], [numpy.sin(th), numpy.cos(th)]])
            t = rng.uniform(-2.0, 2.0, 2)
        ai = numpy.linalg.inv(a)
        ti = -ai @ t
        x0N += [t[0], a[0, 0], a[0, 1]]
        y0N += [t[1], a[1, 0], a[1, 1]]
        xN0 += [ti[0], ai[0, 0], ai[0, 1]]
        yN0 += [ti[1], ai[1, 0], ai[1, 1]]
    return [numpy.array(v) for v in (x0N, y0N, xN0, yN0)]


def make_case(nc, n_peaks, seed, calibration):
    rng = numpy.random.default_rng(seed)
    maps = affine(nc, seed + 1)
    ny, nx = SHAPE
    x = rng.uniform(12.0, nx - 12.0, n_peaks)
    y = rng.uniform(12.0, ny - 12.0, n_peaks)
    h = rng.uniform(400.0, 1500.0, n_peaks)
    images, bgs, rqes, vars_ = [], [], [], []
    yy, xx = numpy.mgrid[0:ny, 0:nx]
    for c in range(nc):
        cx = maps[0][3 * c] + maps[0][3 * c + 1] * x + maps[0][3 * c + 2] * y
        cy = maps[1][3 * c] + maps[1][3 * c + 1] * x + maps[1][3 * c + 2] * y
        sig = 1.3 + 0.35 * c
        img = numpy.full(SHAPE, 20.0)
        for i in range(n_peaks):
            img += (h[i] / (1.0 + 0.5 * c)) * numpy.exp(-((xx - cx[i]) ** 2 + (yy - cy[i]) ** 2) / (2 * sig * sig))
        images.append(rng.poisson(img).astype(numpy.float64))
        bgs.append(numpy.full(SHAPE, 20.0))
        if calibration:
            rqes.append(rng.uniform(0.85, 1.15, SHAPE))
            vars_.append(rng.uniform(0.5, 2.0, SHAPE))
        else:
            rqes.append(numpy.ones(SHAPE))
            vars_.append(numpy.zeros(SHAPE))
    peaks = numpy.stack([numpy.round(x) + rng.uniform(-0.4, 0.4, n_peaks),
                         numpy.round(y) + rng.uniform(-0.4, 0.4, n_peaks),
                         numpy.zeros(n_peaks), numpy.full(n_peaks, 1.5)], axis=1)
    return dict(images=numpy.stack(images), backgrounds=numpy.stack(bgs), rqe=numpy.stack(rqes),
                variance=numpy.stack(vars_), maps=numpy.stack(maps), peaks=peaks)


PROPS = ("x", "y", "height", "background", "xsigma", "ysigma", "error")


def run_ref(case):
    nc = case["images"].shape[0]
    f = ref_driver.RefMPDaoFitter(SHAPE, nc, case["rqe"], case["variance"], (1.0, 3.0), 10, list(case["maps"]))
    f.newImage(list(case["images"]))
    f.newBackground(list(case["backgrounds"]))
    f.newPeaks(case["peaks"], "finder")
    f.doFit(200)
    out = {}
    for c in range(nc):
        for p in PROPS + ("status", "iterations"):
            out["c%d_%s" % (c, p)] = f.getPeakProperty(p, c)
        out["c%d_counters" % c] = f.counters(c)
    f.cleanup()
    return out


def main():
    out = {}
    for name, (nc, n_peaks, seed, cal) in (("a", (2, 14, 3, False)), ("b", (3, 12, 7, True))):
        case = make_case(nc, n_peaks, seed, cal)
        for k, v in case.items():
            out[name + "_" + k] = v
        for k, v in run_ref(case).items():
            out[name + "_" + k] = v
    numpy.savez_compressed(os.path.join(HERE, "g_mp_dao.npz"), **out)


if __name__ == "__main__":
    main()
