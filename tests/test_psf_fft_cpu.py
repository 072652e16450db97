"""The FFT PSF model's translated PSF (psf_fft/psf_fft.c) on the CPU.

tests/golden/g_psf_fft.npz holds the reference's own pure-Python version
of psf_fft.c (psf_fft/psf_fft_py.py) on two PSF stacks and five
translations: the PSF and its x, y and z derivatives.  The reference's test
holds its C and Python versions to 1e-6 of each other (test/test_psf_fft.py,
tests 6-10); the oracle restatement (numpy transforms), the oracle's
separable evaluation (the one its fitter uses) and libsa_cuda.so's
pFTInitialize / pFTTranslate / pFTGetPSF* host functions are held to the
same bar against the goldens, and to 1e-14 of each other."""
import os
import sys

import numpy
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GOLDEN = os.path.join(HERE, "golden", "g_psf_fft.npz")


def cases():
    g = numpy.load(GOLDEN)
    for name in ("a", "b"):
        psf = g[name + "_psf"]
        for t, ref in zip(g["translations"], g[name + "_out"]):
            yield psf, tuple(t), ref


def test_oracle_matches_the_reference_python():
    from oracle import psf_fft as opf
    for psf, t, ref in cases():
        o = opf.PSFFFT(psf)
        o.translate(*t)
        mine = numpy.stack([o.get_psf(), o.get_psf_dx(), o.get_psf_dy(), o.get_psf_dz()])
        assert numpy.abs(mine - ref).max() < 1.0e-6, t


def test_oracle_fitter_evaluation_matches_the_restatement():
    from oracle import oracle, psf_fft as opf
    for psf, t, _ in cases():
        f = oracle.OracleFitter("fft", (48, 48), psf=psf)
        mine = numpy.stack(oracle.fft_eval(f, *t))
        f.cleanup()
        o = opf.PSFFFT(psf)
        o.translate(*t)
        npy = numpy.stack([o.get_psf(), o.get_psf_dx(), o.get_psf_dy(), o.get_psf_dz()])
        assert numpy.abs(mine - npy).max() < 1.0e-14, t


def test_library_psf_fft_functions():
    sys.path.insert(0, os.path.join(ROOT, "storm-analysis_gb300"))
    from sa_gb300 import loadclib
    if not os.path.exists(loadclib.LIB_PATH):
        pytest.skip("libsa_cuda.so is not built")
    from oracle import psf_fft as opf
    from sa_gb300 import psf_fft_c
    for psf, t, ref in cases():
        p = psf_fft_c.PSFFFT(psf)
        assert (p.lib.pFTGetZSize(p.pfft), p.lib.pFTGetYSize(p.pfft), p.lib.pFTGetXSize(p.pfft)) == psf.shape
        p.translate(*t)
        mine = numpy.stack([p.getPSF(), p.getPSFdx(), p.getPSFdy(), p.getPSFdz()])
        p.cleanup()
        o = opf.PSFFFT(psf)
        o.translate(*t)
        npy = numpy.stack([o.get_psf(), o.get_psf_dx(), o.get_psf_dy(), o.get_psf_dz()])
        assert numpy.abs(mine - npy).max() < 1.0e-14, t
        assert numpy.abs(mine - ref).max() < 1.0e-6, t


def test_derivatives_are_the_translation_derivatives():
    """As the reference's tests 3-5: the analytic derivative against a
    finite difference of the translated PSF (here a central one)."""
    from oracle import psf_fft as opf
    psf = numpy.load(GOLDEN)["a_psf"]
    o = opf.PSFFFT(psf)
    base = (0.2, -0.1, 0.3)
    eps = 1.0e-5
    for axis, get in ((0, "get_psf_dx"), (1, "get_psf_dy"), (2, "get_psf_dz")):
        o.translate(*base)
        exact = getattr(o, get)()
        tp = list(base)
        tm = list(base)
        tp[axis] += eps
        tm[axis] -= eps
        o.translate(*tp)
        fp = o.get_psf()
        o.translate(*tm)
        fm = o.get_psf()
        # the derivatives are those of the translated PSF with respect to
        # the translation (the reference's tests 3-5 check the same with a
        # forward difference)
        fd = (fp - fm) / (2 * eps)
        assert numpy.abs(exact - fd).max() < 1.0e-9, axis
