"""
Generate tests/golden/g_finder.npz from the REFERENCE's own peak-finder C
code, compiled from its sources by ``make -C oracle ref``:

  * libdraw_gaussians.so (simulator/draw_gaussians.c): the unit-sum
    Gaussian PSFs of the matched filters, as sa_library/fitting.py:38-46
    draws them, for even, odd and clamped image sizes;
  * libia_utilities.so (sa_library/ia_utilities.c): calcMaxPeaks and
    findLocalMaxima on seeded images with many exact ties, several z planes,
    fractional radii and repeated calls that advance the taken counts; and
    the post-fit culling (markDimmerPeaks, markLowSignificancePeaks,
    runningIfHasNeighbors, createKDTree / nearestKDTree) on clustered
    peaks with mixed statuses.

Run here, where the reference tree exists:

    make -C oracle ref
    python tests/golden/make_golden_finder.py
"""
import ctypes
import os

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(os.path.dirname(os.path.dirname(HERE)), "oracle", "_ref")


class FlmData(ctypes.Structure):
    """The field order of flmData in sa_library/ia_utilities.c:20-36."""
    _fields_ = [("margin", ctypes.c_int), ("n_peaks", ctypes.c_int), ("z_range", ctypes.c_int),
                ("xsize", ctypes.c_int), ("ysize", ctypes.c_int), ("zsize", ctypes.c_int),
                ("radius", ctypes.c_double), ("threshold", ctypes.c_double),
                ("z_values", ctypes.c_void_p), ("taken", ctypes.c_void_p), ("images", ctypes.c_void_p)]


def ref_psf(dg, shape, sigma):
    img = numpy.zeros(shape, dtype=numpy.float64)
    obj = numpy.array([[0.5 * shape[0], 0.5 * shape[1], 1.0, sigma, sigma]], dtype=numpy.float64)
    dg.drawGaussians(img.ctypes.data_as(ctypes.c_void_p), obj.ctypes.data_as(ctypes.c_void_p),
                     ctypes.c_int(shape[1]), ctypes.c_int(shape[0]), ctypes.c_int(1), ctypes.c_int(1))
    return img / numpy.sum(img)


def ref_maxima(ia, images, taken, margin, radius, threshold, z_range, z_values):
    """One findMaxima call as ia_utilities_c.py:173-231 makes it (margin is
    already the finder's margin + 1).  taken is updated in place."""
    zsize = len(images)
    P = ctypes.c_void_p * zsize
    c_img = P(*[im.ctypes.data for im in images])
    c_tk = P(*[t.ctypes.data for t in taken])
    zv = numpy.ascontiguousarray(z_values, dtype=numpy.float64)
    flm = FlmData(margin=margin, n_peaks=0, z_range=z_range, xsize=images[0].shape[1],
                  ysize=images[0].shape[0], zsize=zsize, radius=radius, threshold=threshold,
                  z_values=zv.ctypes.data, taken=ctypes.addressof(c_tk), images=ctypes.addressof(c_img))
    n = ia.calcMaxPeaks(ctypes.byref(flm)) + 1
    out = [numpy.zeros(n) for _ in range(4)]
    flm.n_peaks = n
    z, y, x, h = out
    ia.findLocalMaxima(ctypes.byref(flm), *[a.ctypes.data_as(ctypes.c_void_p) for a in (z, y, x, h)])
    k = flm.n_peaks
    return n - 1, x[:k].copy(), y[:k].copy(), z[:k].copy(), h[:k].copy()


def main():
    dg = ctypes.CDLL(os.path.join(REF, "libdraw_gaussians.so"))
    ia = ctypes.CDLL(os.path.join(REF, "libia_utilities.so"))
    ia.calcMaxPeaks.restype = ctypes.c_int
    out = {}
    psf_cases = [((80, 90), 1.0), ((41, 53), 2.0), ((41, 53), 8.0), ((96, 96), 8.0), ((75, 64), 1.5)]
    for i, (shape, sigma) in enumerate(psf_cases):
        out["psf%d" % i] = ref_psf(dg, shape, sigma)
        out["psf%d_shape" % i] = numpy.array(shape)
        out["psf%d_sigma" % i] = numpy.array(sigma)

    rng = numpy.random.default_rng(5)
    # (rows, cols, planes, margin, radius, threshold, z_range, calls, n_duplicates)
    cases = [(48, 40, 1, 2, 1.5, 4.0, 1, 2, 1),
             (40, 48, 1, 3, 5.0, 5.0, 1, 1, 1),
             (37, 45, 3, 2, 2.7, 3.0, 1, 2, 1),
             (36, 36, 3, 1, 1.0, 2.0, 3, 3, 2),
             (33, 41, 2, 4, 0.5, 6.0, 0, 1, 1)]
    for i, (rows, cols, planes, margin, radius, thr, zr, calls, ndup) in enumerate(cases):
        images = [numpy.ascontiguousarray(rng.integers(0, 10, size=(rows, cols)).astype(numpy.float64))
                  for _ in range(planes)]
        if i == 1:   # a smooth image: isolated maxima, no ties
            yy, xx = numpy.mgrid[0:rows, 0:cols]
            img = numpy.zeros((rows, cols))
            for _ in range(12):
                cy, cx, h = rng.uniform(0, rows), rng.uniform(0, cols), rng.uniform(4, 20)
                img += h * numpy.exp(-((yy - cy) ** 2 + (xx - cx) ** 2) / 4.0)
            images = [numpy.ascontiguousarray(img)]
        zvals = list(rng.uniform(-0.5, 0.5, planes))
        taken = [numpy.ascontiguousarray(numpy.ones((rows, cols), dtype=numpy.int32) - ndup)
                 for _ in range(planes)]
        out["lm%d_images" % i] = numpy.stack(images)
        out["lm%d_params" % i] = numpy.array([margin, radius, thr, zr, calls, ndup], dtype=numpy.float64)
        out["lm%d_zvalues" % i] = numpy.array(zvals)
        for c in range(calls):
            n, x, y, z, h = ref_maxima(ia, images, taken, margin, radius, thr, zr, zvals)
            out["lm%d_c%d_max" % (i, c)] = numpy.array(n)
            out["lm%d_c%d_xyzh" % (i, c)] = numpy.stack([x, y, z, h]) if x.size else numpy.zeros((4, 0))
            out["lm%d_c%d_taken" % (i, c)] = numpy.stack(taken).copy()
    # post-fit culling (ia_utilities.c:221-430): clustered peaks, mixed statuses
    f64 = ctypes.c_double
    dp = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    ia.markDimmerPeaks.restype = ctypes.c_int
    ia.markLowSignificancePeaks.restype = ctypes.c_int
    ia.createKDTree.restype = ctypes.c_void_p
    for i, (n, r1, r2) in enumerate([(300, 1.5, 7.5), (60, 2.0, 5.0), (1000, 1.0, 5.0)]):
        centres = rng.uniform(10, 90, (n // 3, 2))
        pts = numpy.concatenate([centres + rng.normal(0, 0.8, centres.shape) for _ in range(3)])[:n]
        x = numpy.ascontiguousarray(pts[:, 0])
        y = numpy.ascontiguousarray(pts[:, 1])
        h = numpy.ascontiguousarray(rng.uniform(100, 1000, x.size))
        sig = numpy.ascontiguousarray(rng.uniform(0, 12, x.size))
        st = numpy.ascontiguousarray(rng.choice([0, 1, 1, 1, 2], x.size).astype(numpy.int32))
        out["cull%d_xyhs" % i] = numpy.stack([x, y, h, sig])
        out["cull%d_status" % i] = st.copy()
        out["cull%d_r" % i] = numpy.array([r1, r2])
        s1 = st.copy()
        n1 = ia.markDimmerPeaks(dp(x), dp(y), dp(h), dp(s1), f64(r1), f64(r2), x.size)
        out["cull%d_dimmer" % i] = s1
        out["cull%d_dimmer_n" % i] = numpy.array(n1)
        s2 = st.copy()
        n2 = ia.markLowSignificancePeaks(dp(x), dp(y), dp(sig), dp(s2), f64(6.0), f64(r2), x.size)
        out["cull%d_lowsig" % i] = s2
        out["cull%d_lowsig_n" % i] = numpy.array(n2)
        nx = numpy.ascontiguousarray(rng.uniform(10, 90, n // 10 + 1))
        ny = numpy.ascontiguousarray(rng.uniform(10, 90, n // 10 + 1))
        s3 = st.copy()
        ia.runningIfHasNeighbors(dp(x), dp(y), dp(nx), dp(ny), dp(s3), f64(r2), x.size, nx.size)
        out["cull%d_new" % i] = numpy.stack([nx, ny])
        out["cull%d_running" % i] = s3
        kd = ia.createKDTree(dp(nx), dp(ny), nx.size)
        dist = numpy.zeros(x.size)
        idx = numpy.zeros(x.size, dtype=numpy.int32)
        ia.nearestKDTree(ctypes.c_void_p(kd), dp(x), dp(y), dp(dist), dp(idx), f64(r2), x.size)
        ia.freeKDTree(ctypes.c_void_p(kd))
        out["cull%d_nearest_d" % i] = dist
        out["cull%d_nearest_i" % i] = idx
    numpy.savez_compressed(os.path.join(HERE, "g_finder.npz"), **out)
    print("wrote g_finder.npz:", len(out), "arrays")


if __name__ == "__main__":
    main()
