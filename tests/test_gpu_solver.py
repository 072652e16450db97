"""The engine's damped solves against LAPACK dposv, and the reference's
counters of the GPU fits.

mFitSolve (sa_library/multi_fit.c:1839-1883) solves (H + lam diag H) x = b
with dposv("Lower") and reports failure when H is not positive definite or
x has a NaN.  saSolveDamped runs the engine's device solvers on batches of
such systems: the FP64 Cholesky (engine 0), the FP32 Gaussian step's
LDL^T with float-float refinements (1) and the FP32 spline step's LU with
FP64 refinements (2).  scipy's LAPACK dposv is the reference here.

The counters (multi_fit.h:87-94: n_dposv, n_iterations, n_lost, n_margin,
n_neg_fi, n_neg_height, n_non_converged, n_non_decr) of the FP64 engine on
the golden cases equal the reference's."""
import numpy
import pytest

from golden_io import CASES, load_case, run_fitter
from gpu_helpers import make_gpu_fitter

pytestmark = pytest.mark.gpu

LAMBDAS = (0.0, 1.0e-3, 1.0, 1.0e6)


def lm_systems(k, n, seed):
    """Normal equations shaped like an LM step's: H = J^T W J of a random
    Jacobian over 80 pixels with columns of very different scales (height,
    positions, widths, background), b = J^T r."""
    rng = numpy.random.default_rng(seed)
    scale = 10.0 ** rng.uniform(-2.0, 2.0, size=(n, 1, k))
    J = rng.normal(size=(n, 80, k)) * scale
    W = rng.uniform(0.05, 2.0, size=(n, 80))
    H = numpy.einsum("npk,np,npl->nkl", J, W, J)
    b = numpy.einsum("npk,np->nk", J, rng.normal(size=(n, 80)))
    return numpy.ascontiguousarray(H), numpy.ascontiguousarray(b)


def indefinite_systems(k, n, seed):
    """Symmetric matrices with one clearly negative eigenvalue."""
    rng = numpy.random.default_rng(seed)
    H = numpy.zeros((n, k, k))
    for i in range(n):
        q, _ = numpy.linalg.qr(rng.normal(size=(k, k)))
        ev = rng.uniform(0.5, 5.0, size=k)
        ev[rng.integers(k)] = -rng.uniform(0.5, 5.0)
        H[i] = (q * ev) @ q.T
    return H, rng.normal(size=(n, k))


def dposv(H, b, lam):
    from scipy.linalg import lapack
    xs, infos = [], []
    for Hi, bi in zip(H, b):
        A = Hi.copy()
        A[numpy.diag_indices_from(A)] *= (1.0 + lam)
        _, x, info = lapack.dposv(A, bi, lower=1)
        if info == 0 and numpy.isnan(x).any():
            info = -999   # mFitSolve's NaN check
        xs.append(x)
        infos.append(info)
    return numpy.array(xs), numpy.array(infos)


def solve(H, b, lam, engine):
    from sa_gb300 import loadclib
    lib = loadclib.load()
    n, k = b.shape
    x = numpy.zeros((n, k))
    info = numpy.zeros(n, dtype=numpy.int32)
    r = lib.saSolveDamped(numpy.ascontiguousarray(H).ravel(), numpy.ascontiguousarray(b).ravel(), n, k, lam,
                          engine, x.ravel(), info)
    assert r == 0, loadclib.last_error()
    return x, info


def rel_err(x, ref):
    return numpy.linalg.norm(x - ref, axis=1) / numpy.linalg.norm(ref, axis=1)


@pytest.mark.parametrize("k", [4, 5, 6, 7])
def test_fp64_cholesky_matches_dposv(k):
    for lam in LAMBDAS:
        H, b = lm_systems(k, 200, seed=k)
        ref, info_ref = dposv(H, b, lam)
        x, info = solve(H, b, lam, 0)
        assert (info_ref == 0).all() and (info == 0).all()
        assert rel_err(x, ref).max() < 1e-11, (k, lam, rel_err(x, ref).max())


@pytest.mark.parametrize("engine,ks", [(1, [4, 5, 6]), (2, [4, 5])])
def test_fp32_solvers_match_dposv(engine, ks):
    """The FP32 solvers given the matrix they see in their step (engine 1:
    the Hessian rounded to FP32) return dposv's solution of that matrix to
    ~1e-10 (the float-float / FP64 refinements), not to FP32 accuracy."""
    for k in ks:
        for lam in LAMBDAS:
            H, b = lm_systems(k, 200, seed=10 + k)
            Hs = H.astype(numpy.float32).astype(numpy.float64) if engine == 1 else H
            ref, info_ref = dposv(Hs, b, lam)
            x, info = solve(H, b, lam, engine)
            assert (info_ref == 0).all() and (info == 0).all()
            assert rel_err(x, ref).max() < 1e-10, (engine, k, lam, rel_err(x, ref).max())


@pytest.mark.parametrize("engine", [0, 1, 2])
def test_solvers_report_what_dposv_reports(engine):
    """Not positive definite (dposv info > 0) and a NaN in the solution are
    failures for every solver, as mFitSolve reports them."""
    for k in ([4, 5, 6] if engine == 1 else [4, 5, 7] if engine == 0 else [4, 5]):
        H, b = indefinite_systems(k, 100, seed=20 + k)
        _, info_ref = dposv(H, b, 0.0)
        _, info = solve(H, b, 0.0, engine)
        assert (info_ref > 0).all()
        assert (info != 0).all(), (engine, k)
        H, b = lm_systems(k, 8, seed=30 + k)
        b[:, 0] = numpy.nan
        _, info = solve(H, b, 1.0, engine)
        assert (info != 0).all(), (engine, k)


COUNTERS = ["n_dposv", "n_iterations", "n_lost", "n_margin", "n_neg_fi", "n_neg_height", "n_non_converged",
            "n_non_decr"]


@pytest.mark.parametrize("name", [c for c in CASES if c != "g_2d_testing"])
def test_fp64_engine_counters_match_reference(name):
    """The reference's eight fit counters (what printFittingInfo reports) of
    the FP64 engine's fit equal the reference C's on every golden case
    (g_2d_testing, whose fits the reference itself cannot reproduce under a
    1e-15 perturbation, is left out)."""
    case = load_case(name)
    f = make_gpu_fitter(case["model"], case["image"], rqe=case["rqe"], scmos=case["scmos"],
                        spline=case["spline"], precision=64, **case["kw"])
    run_fitter(f, case)
    ctr = f.counters()
    assert [ctr[c] for c in COUNTERS] == case["counters"].tolist(), (name, ctr)
    f.cleanup(verbose=False)
