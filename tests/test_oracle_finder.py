"""The CPU oracle of the peak finder (oracle/finder.py) against the golden
fixture made from the reference's own C (tests/golden/make_golden_finder.py:
draw_gaussians.c PSFs; ia_utilities.c calcMaxPeaks / findLocalMaxima with
ties, several planes, fractional radii and repeated calls), and against the
reference's own matched-filter test criteria (test/test_matched_filter.py)."""
import os

import numpy
import pytest

from oracle import finder as F

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "g_finder.npz")


@pytest.fixture(scope="module")
def g():
    return numpy.load(GOLDEN)


def test_psf_matches_reference_drawing(g):
    for i in range(5):
        shape = tuple(int(v) for v in g["psf%d_shape" % i])
        psf = F.gaussian_psf(shape, float(g["psf%d_sigma" % i]))
        assert numpy.abs(psf - g["psf%d" % i]).max() <= 1e-15 * g["psf%d" % i].max()


def lm_cases(g):
    i = 0
    while "lm%d_images" % i in g:
        yield i
        i += 1


def test_local_maxima_match_reference_exactly(g):
    n_cases = 0
    for i in lm_cases(g):
        imgs = list(g["lm%d_images" % i])
        m, r, thr, zr, calls, nd = g["lm%d_params" % i]
        zv = list(g["lm%d_zvalues" % i])
        taken = [numpy.ones(imgs[0].shape, numpy.int32) - int(nd) for _ in imgs]
        for c in range(int(calls)):
            n = F.calc_max_peaks(imgs, taken, int(m), thr)
            x, y, z, h = F.find_local_maxima(imgs, taken, int(m), r, thr, int(zr), zv)
            got = numpy.stack([x, y, z, h]) if x.size else numpy.zeros((4, 0))
            assert n == int(g["lm%d_c%d_max" % (i, c)])
            assert numpy.array_equal(got, g["lm%d_c%d_xyzh" % (i, c)])
            assert numpy.array_equal(numpy.stack(taken), g["lm%d_c%d_taken" % (i, c)])
            n_cases += 1
    assert n_cases >= 9


def _psf(shape, s):
    return F.gaussian_psf(shape, s)


def test_matched_filter_normalisation_and_numpy_fft():
    """Unit-sum PSF keeps the image sum; the result is numpy's FFT
    convolution with the recentred PSF."""
    psf = _psf((80, 90), 1.0)
    flt = F.MatchedFilter(psf)
    for i in range(1, 5):
        img = numpy.zeros((80, 90))
        img[40, 45] = float(i)
        conv = flt.convolve(img)
        assert abs(img.sum() - conv.sum()) < 1e-6
    img = numpy.zeros((80, 90))
    img[40, 45] = 100.0
    t = numpy.real(numpy.fft.ifft2(numpy.fft.fft2(F.recenter_psf(psf)) * numpy.fft.fft2(img)))
    assert numpy.allclose(flt.convolve(img), t)


def test_matched_filter_memo():
    psf = _psf((40, 50), 2.0)
    flt = F.MatchedFilter(psf, memoize=True, max_diff=0.1)
    img = numpy.zeros((40, 50))
    img[20, 25] = 1.0
    r1 = flt.convolve(img)
    img2 = img.copy()
    img2[20, 25] = 1.05
    assert numpy.abs(flt.convolve(img2) - r1).max() < 1e-12
    img3 = img.copy()
    img3[20, 25] = 1.1
    assert numpy.abs(flt.convolve(img3) - r1).max() > 1e-12
    # before any convolution a memo filter returns the recentred PSF
    f2 = F.MatchedFilter(psf, memoize=True, max_diff=0.1)
    assert numpy.array_equal(f2.convolve(numpy.zeros((40, 50))), F.recenter_psf(psf))


def test_pad_array_mirrors_edges():
    a = numpy.arange(20.0).reshape(4, 5)
    p = F.pad_array(a, 2)
    assert p.shape == (8, 9)
    assert numpy.array_equal(p[2:6, 2:7], a)
    assert numpy.array_equal(p[0:2, 2:7], numpy.flipud(a[0:2]))
    assert numpy.array_equal(p[2:6, 0:2], numpy.fliplr(a[:, 0:2]))


def test_culling_matches_reference_exactly(g):
    """markDimmerPeaks, markLowSignificancePeaks, runningIfHasNeighbors and
    the kd-tree nearest query of the oracle equal the reference's C."""
    i = 0
    while "cull%d_xyhs" % i in g:
        x, y, h, sig = g["cull%d_xyhs" % i]
        st = g["cull%d_status" % i]
        r1, r2 = g["cull%d_r" % i]
        s1 = st.copy()
        assert F.mark_dimmer_peaks(x, y, h, s1, r1, r2) == int(g["cull%d_dimmer_n" % i])
        assert numpy.array_equal(s1, g["cull%d_dimmer" % i])
        s2 = st.copy()
        assert F.mark_low_significance_peaks(x, y, sig, s2, 6.0, r2) == int(g["cull%d_lowsig_n" % i])
        assert numpy.array_equal(s2, g["cull%d_lowsig" % i])
        nx, ny = g["cull%d_new" % i]
        assert numpy.array_equal(F.running_if_has_neighbors(x, y, nx, ny, st.copy(), r2), g["cull%d_running" % i])
        d, ix = F.nearest(nx, ny, x, y, r2)
        assert numpy.array_equal(d, g["cull%d_nearest_d" % i]) and numpy.array_equal(ix, g["cull%d_nearest_i" % i])
        i += 1
    assert i == 3


def test_spline_psf_matches_spline3d_evaluation():
    """SplinePSF.getPSF (the PSF object Spliner's finder draws its filters
    from) samples the spline as Spline3D.f does (spliner/spline3D.py:150-163,
    spliner/spline1D.py:12-28), restated point by point here."""
    import math
    from sa_gb300 import cubic_fit_c, synth
    sp = synth.make_spline(3)
    S = cubic_fit_c.SplinePSF(coeff=sp["coeff"], zmin=synth.SPLINE_ZMIN_NM, zmax=synth.SPLINE_ZMAX_NM)
    n = S.getSize()

    def rc(v):
        if v < 0 or v > n:
            return -1, -1.0
        fl = math.floor(v)
        i, d = int(fl), v - fl
        if v == n:
            i, d = i - 1, 1.0
        return i, d

    def f(z, y, x):
        (ix, dx), (iy, dy), (iz, dz) = rc(x), rc(y), rc(z)
        if -1 in (ix, iy, iz):
            return 0.0
        return sum(S.coeff[ix, iy, iz, i * 16 + j * 4 + k] * dx ** i * dy ** j * dz ** k
                   for i in range(4) for j in range(4) for k in range(4))

    for zval in (-300.0, 0.0, 250.0):
        psf = S.getPSF(zval, normalize=False)
        sz = S.getScaledZ(zval)
        off = 0.5 if (n - 1) % 2 == 0 else 1.0
        ref = numpy.array([[f(sz, y + off, x + off) for x in range(n - 1)] for y in range(n - 1)])
        assert numpy.abs(psf - ref).max() <= 1e-12 * numpy.abs(ref).max()
    big = S.getPSF(0.0, shape=(64, 64), normalize=True)
    assert big.shape == (64, 64) and abs(big.sum() - 1.0) < 1e-12
    assert S.isValidZ(0.0) and not S.isValidZ(S.getZMax())


def _two_phase(x, y, status, marked, r_neighbors):
    """The GPU kernels' formulation (k_mark_* then k_mark_apply): marked
    peaks become ERROR; a CONVERGED peak within r_neighbors of a marked one
    becomes RUNNING; every peak decided from the statuses on entry."""
    out = status.copy()
    out[marked] = F.ERROR
    for i in numpy.nonzero(~marked & (status == F.CONVERGED))[0]:
        nb = F._within(x, y, x[i], y[i], r_neighbors)
        if marked[nb].any():
            out[i] = F.RUNNING
    return out


def test_culling_does_not_depend_on_visiting_order():
    """The parallel culling rests on this: in the reference's sequential
    loops (ia_utilities.c:221-340) a peak's mark depends only on its own
    height / significance and its status on entry, so marking all peaks
    first and applying after gives the sequential result."""
    rng = numpy.random.default_rng(21)
    for trial in range(40):
        n = int(rng.integers(5, 400))
        centres = rng.uniform(5, 60, (max(n // 3, 1), 2))
        pts = numpy.concatenate([centres + rng.normal(0, 0.9, centres.shape) for _ in range(3)])[:n]
        x, y = numpy.ascontiguousarray(pts[:, 0]), numpy.ascontiguousarray(pts[:, 1])
        n = x.size
        h = rng.uniform(100, 1000, n)
        h[rng.integers(0, n, n // 10)] = 500.0          # exact height ties
        sig = rng.uniform(0, 12, n)
        st = rng.choice([0, 1, 1, 1, 2], n).astype(numpy.int32)
        r1, r2 = rng.uniform(0.5, 2.0), rng.uniform(2.0, 8.0)
        s_seq = st.copy()
        n_seq = F.mark_dimmer_peaks(x, y, h, s_seq, r1, r2)
        marked = numpy.array([st[i] != F.ERROR and (h[F._within(x, y, x[i], y[i], r1)] > h[i]).any()
                              for i in range(n)])
        assert marked.sum() == n_seq
        assert numpy.array_equal(_two_phase(x, y, st, marked, r2), s_seq)
        s_seq = st.copy()
        n_seq = F.mark_low_significance_peaks(x, y, sig, s_seq, 6.0, r2)
        marked = (st != F.ERROR) & ~(sig > 6.0)
        assert marked.sum() == n_seq
        assert numpy.array_equal(_two_phase(x, y, st, marked, r2), s_seq)
