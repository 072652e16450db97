"""The oracle's multi-plane fitter (oracle/sa_oracle.c oraMP*, a
restatement of multi_plane/mp_fit.c with mp_fit_dao.c / mp_fit_arb.c)
against the reference's own multi-plane C.

tests/golden/g_mp_dao.npz holds the reference's 2D Gaussian multi-plane
fitter (mp_fit.c + mp_fit_dao.c compiled from its sources, driven as its
MPFitDao2D drives it) on a two-plane and a three-plane case, one with
sCMOS calibration: per channel the fitted parameters, statuses, iterations
and counters.  The oracle must give the same statuses, iterations and
counters, and parameters within 1e-9."""
import numpy
import pytest

GOLDEN = "tests/golden/g_mp_dao.npz"
PROPS = ("x", "y", "height", "background", "xsigma", "ysigma", "error")


def oracle_fit(g, n):
    from oracle import oracle
    imgs = g[n + "_images"]
    nc = imgs.shape[0]
    chans = [oracle.OracleFitter("2d", imgs.shape[1:], rqe=g[n + "_rqe"][c], scmos_cal=g[n + "_variance"][c],
                                 roi_size=10, sigma_range=(1.0, 3.0), tol=1.0e-6 * nc) for c in range(nc)]
    f = oracle.OracleMPFitter(chans, list(g[n + "_maps"]), kind="dao", independent_heights=1)
    f.newImage(list(imgs))
    f.newBackground(list(g[n + "_backgrounds"]))
    p = g[n + "_peaks"]
    f.newPeaks({"x": p[:, 0], "y": p[:, 1], "z": p[:, 2], "sigma": p[:, 3]}, "finder")
    f.doFit(200)
    return f, nc


@pytest.mark.parametrize("n", ["a", "b"])
def test_oracle_mp_dao_matches_reference_goldens(n):
    import os
    g = numpy.load(os.path.join(os.path.dirname(__file__), "golden", "g_mp_dao.npz"))
    f, nc = oracle_fit(g, n)
    try:
        for c in range(nc):
            key = "%s_c%d_" % (n, c)
            assert numpy.array_equal(f.getPeakProperty("status", c), g[key + "status"])
            assert numpy.array_equal(f.getPeakProperty("iterations", c), g[key + "iterations"])
            ctr = f.channels[c].counters()
            assert [ctr[k] for k in ("n_dposv", "n_iterations", "n_lost", "n_margin", "n_neg_fi", "n_neg_height",
                                     "n_non_converged", "n_non_decr")] == list(g[key + "counters"])
            for p in PROPS:
                a, b = f.getPeakProperty(p, c), g[key + p]
                assert numpy.abs(a - b).max() <= 1.0e-9 * max(1.0, numpy.abs(b).max()), p
            # the reference's 2D Gaussian multi-plane update moves the x width
            # only (mp_fit_dao.c:186-200): the y width keeps its start value
            assert numpy.all(f.getPeakProperty("ysigma", c) == 1.5)
    finally:
        f.cleanup()
