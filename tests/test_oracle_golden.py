"""The CPU oracle against the reference's own outputs (golden fixtures).

The fixtures were produced by the reference's C fitter compiled from its
sources (tests/golden/make_golden.py); this pins the oracle restatement on
machines where the reference is absent.
"""
import numpy
import pytest

from golden_io import CASES, load_case, run_fitter
from oracle.oracle import OracleFitter, load

STATUS_RUNNING, STATUS_CONVERGED, STATUS_ERROR = 0, 1, 2


def make_oracle(case):
    return OracleFitter(case["model"], case["image"].shape, rqe=case["rqe"], scmos_cal=case["scmos"],
                        spline=case["spline"], **case["kw"])


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference(name):
    case = load_case(name)
    ora = make_oracle(case)
    init, out = run_fitter(ora, case)
    ref = case["out"]
    # Initial estimates (newPeaks): exact up to rounding.
    for p in ["height", "background", "error"]:
        numpy.testing.assert_allclose(init[p], case["init"][p], rtol=1e-10, atol=1e-10)
    assert numpy.array_equal(init["status"], case["init"]["status"])
    # After doFit: identical control flow, parameters equal to rounding.
    assert numpy.array_equal(out["status"], ref["status"])
    assert numpy.array_equal(out["iterations"], ref["iterations"])
    # xsigma/ysigma have no meaning for splines (the reference reads an
    # unset width slot there), so they are compared for Gaussians only.
    pos = ["x", "y", "z"] if case["spline"] is not None else ["x", "y", "z", "xsigma", "ysigma"]
    for p in pos:
        numpy.testing.assert_allclose(out[p], ref[p], rtol=0, atol=1e-8)
    for p in ["height", "background", "error", "significance", "sum"]:
        numpy.testing.assert_allclose(out[p], ref[p], rtol=1e-8, atol=1e-8)
    ctr = ora.counters()
    assert [ctr[k] for k in ["n_dposv", "n_iterations", "n_lost", "n_margin", "n_neg_fi",
                             "n_neg_height", "n_non_converged", "n_non_decr"]] == case["counters"].tolist()
    fimg = ora.getFitImage()
    assert abs(fimg.sum() - case["fit_sum"]) <= 1e-9 * abs(case["fit_sum"])
    ora.cleanup()


def test_oracle_spline_points():
    d = numpy.load(__import__("golden_io").GOLDEN + "/g_spline_points.npz")
    lib = load()
    coeff = numpy.ascontiguousarray(d["spline"].astype(numpy.float64))
    s = coeff.shape[0]
    for (z, y, x), vals in zip(d["points"], d["values"]):
        got = [lib.oraSplineEval3D(coeff.ravel(), s, s, s, z, y, x, w) for w in range(4)]
        numpy.testing.assert_allclose(got, vals, rtol=1e-12, atol=1e-12)


def test_oracle_solver_known_answers():
    """FP64 Cholesky against numpy on random SPD systems and a non-PD failure."""
    lib = load()
    rng = numpy.random.default_rng(0)
    for k in range(4, 8):
        for _ in range(20):
            m = rng.normal(size=(k, k))
            a = m @ m.T + k * numpy.eye(k)
            b = rng.normal(size=k)
            up = numpy.ascontiguousarray(numpy.triu(a))
            x = numpy.ascontiguousarray(b.copy())
            assert lib.oraSolve(up.ravel().copy(), x, k) == 0
            numpy.testing.assert_allclose(x, numpy.linalg.solve(a, b), rtol=1e-9, atol=1e-12)
        a = -numpy.eye(k)
        x = numpy.ones(k)
        assert lib.oraSolve(numpy.ascontiguousarray(a.ravel()), x, k) != 0
