"""Host logic of the GPU matched filter, on the CPU (no device needed):
saFilterAnalyze is the analysis saFilterCreate runs on a recentred PSF --
its circular support and rank-1 split.  The separable convolution those
taps define (computed here in numpy, as the two GPU passes compute it)
must equal the oracle's FFT convolution; a PSF that is not rank 1 must be
sent to the 2D path with its full support."""
import ctypes

import numpy
import pytest

from oracle import finder as F


@pytest.fixture(scope="module")
def lib():
    from sa_gb300 import build, loadclib
    build.build()
    return loadclib.load(require_device=False)


def analyze(lib, rc):
    rc = numpy.ascontiguousarray(rc, dtype=numpy.float64)
    out = numpy.zeros(5, dtype=numpy.int32)
    u = numpy.zeros(rc.shape[0])
    v = numpy.zeros(rc.shape[1])
    assert lib.saFilterAnalyze(rc, rc.shape[0], rc.shape[1], out, u.ctypes.data_as(ctypes.c_void_p),
                               v.ctypes.data_as(ctypes.c_void_p)) == 0
    sep, na, nb, a0, b0 = (int(x) for x in out)
    return sep, na, nb, a0, b0, u[:na], v[:nb]


def separable_conv(img, u, v, a0, b0):
    """out[r][c] = sum_i sum_j u[i] v[j] img[(r - a0 - i) mod R][(c - b0 - j) mod C]."""
    tmp = numpy.zeros_like(img)
    for j, w in enumerate(v):
        tmp += w * numpy.roll(img, b0 + j, axis=1)
    out = numpy.zeros_like(img)
    for i, w in enumerate(u):
        out += w * numpy.roll(tmp, a0 + i, axis=0)
    return out


@pytest.mark.parametrize("shape,sigma", [((80, 90), 1.0), ((41, 53), 2.0), ((41, 53), 8.0), ((96, 96), 8.0),
                                         ((75, 64), 1.5), ((23, 17), 1.0)])
def test_gaussian_psfs_split_exactly(lib, shape, sigma):
    psf = F.gaussian_psf(shape, sigma)
    rc = F.recenter_psf(psf)
    sep, na, nb, a0, b0, u, v = analyze(lib, rc)
    assert sep == 1
    aw = max(int(5.0 * sigma), 1)
    assert na == min(2 * aw + 1, shape[0]) and nb == min(2 * aw + 1, shape[1])
    img = numpy.random.default_rng(3).uniform(0.0, 100.0, shape)
    ref = F.MatchedFilter(psf).convolve(img)
    assert numpy.abs(separable_conv(img, u, v, a0, b0) - ref).max() <= 1e-12 * numpy.abs(ref).max()


def test_non_separable_psf_takes_2d_path(lib):
    rng = numpy.random.default_rng(8)
    blob = numpy.zeros((37, 45))
    blob[14:23, 17:28] = rng.uniform(0.0, 1.0, (9, 11))
    sep, na, nb, a0, b0, _, _ = analyze(lib, F.recenter_psf(blob))
    assert sep == 0 and (na, nb) == (9, 11)
    # support straddling the wrap: offsets are signed, first tap at a0
    rc = F.recenter_psf(blob)
    rows = numpy.nonzero(rc.any(axis=1))[0]
    assert sorted(((a0 + i) % 37) for i in range(na)) == sorted(rows.tolist())


def test_degenerate_psfs(lib):
    sep, na, nb, a0, b0, u, v = analyze(lib, numpy.zeros((16, 16)))
    assert (sep, na, nb) == (1, 1, 1)
    delta = numpy.zeros((16, 20))
    delta[0, 0] = 1.0
    sep, na, nb, a0, b0, u, v = analyze(lib, delta)
    assert (sep, na, nb, a0, b0) == (1, 1, 1, 0, 0) and u[0] * v[0] == 1.0
