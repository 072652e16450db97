"""The pupil-function PSF model (pupilfn/pupil_function.c) on the CPU.

tests/golden/g_pupilfn.npz holds the reference's own Python pupil math
(simulator/pupil_math.py, which pupil_function.c is written to match) on
two geometries (20 px as the reference's tests, 30 px as its
pupil-function diagnostics) and five translations: the complex PSF and its
x, y and z derivatives as pupil_function.c defines them.  The reference's
test holds its C library to that Python with numpy.allclose
(test/test_pupilfn.py, tests 1, 2, 9); the oracle's numpy restatement, the
oracle's C evaluation (the one its fitter uses) and libsa_cuda.so's pfn*
host functions are held to 1e-12 of the goldens' scale and to 1e-12 of
each other."""
import os
import sys

import numpy
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GOLDEN = os.path.join(HERE, "golden", "g_pupilfn.npz")
sys.path.insert(0, os.path.join(ROOT, "storm-analysis_gb300"))


def cases():
    g = numpy.load(GOLDEN)
    for name, size in (("a", 20), ("b", 30)):
        geo = (g[name + "_kx"], g[name + "_ky"], g[name + "_kz"], g[name + "_pf"])
        for t, ref in zip(g["translations"], g["%s_out" % name]):
            yield size, geo, tuple(t), ref


def rel(a, b):
    return (numpy.abs(a - b).max(axis=(-2, -1)) / numpy.abs(b).max(axis=(-2, -1))).max()


def test_oracle_matches_the_reference_python():
    from oracle import pupil_fn as opf
    for size, (kx, ky, kz, pf), t, ref in cases():
        o = opf.PupilFunction(kx, ky, kz, size)
        o.set_pf(pf)
        o.translate(*t)
        mine = numpy.stack([o.get_psf(), o.get_psf_dx(), o.get_psf_dy(), o.get_psf_dz()])
        assert rel(mine, ref) < 1.0e-12, t


def test_oracle_fitter_evaluation_matches_the_restatement():
    from oracle import oracle, pupil_fn as opf
    for size, (kx, ky, kz, pf), t, _ in cases():
        f = oracle.OracleFitter("pupil", (64, 64), pupil=(kx, ky, kz, pf))
        mine = numpy.stack(oracle.pupil_eval(f, *t))
        f.cleanup()
        o = opf.PupilFunction(kx, ky, kz, size)
        o.set_pf(pf)
        o.translate(*t)
        npy = numpy.stack([o.get_psf(), o.get_psf_dx(), o.get_psf_dy(), o.get_psf_dz()])
        assert rel(mine, npy) < 1.0e-12, t


def test_library_pupil_function_calls():
    from sa_gb300 import loadclib
    if not os.path.exists(loadclib.LIB_PATH):
        pytest.skip("libsa_cuda.so is not built")
    from oracle import pupil_fn as opf
    from sa_gb300 import pupil_function_c

    class Geo(object):
        pass

    for size, (kx, ky, kz, pf), t, ref in cases():
        geo = Geo()
        geo.size, geo.kx, geo.ky, geo.kz = size, kx, ky, kz
        c = pupil_function_c.PupilFunction(geometry=geo)
        assert c.lib.pfnGetSize(c.getCPointer()) == size
        c.setPF(pf)
        c.translate(*t)
        mine = numpy.stack([c.getPSF(), c.getPSFdx(), c.getPSFdy(), c.getPSFdz()])
        inten = c.getPSFIntensity()
        o = opf.PupilFunction(kx, ky, kz, size)
        o.set_pf(pf)
        o.translate(*t)
        npy = numpy.stack([o.get_psf(), o.get_psf_dx(), o.get_psf_dy(), o.get_psf_dz()])
        assert rel(mine, npy) < 1.0e-12, t
        assert rel(mine, ref) < 1.0e-12, t
        assert numpy.abs(inten - o.get_psf_intensity()).max() < 1.0e-12 * o.get_psf_intensity().max()
        # pfnTranslateZ (pupil_function.c:515-556)
        c.translateZ(t[2])
        o.translate_z(t[2])
        assert rel(c.getPSF(), o.get_psf()) < 1.0e-12
        c.cleanup()


def test_geometry_matches_the_reference_python():
    """sa_gb300.pupil_math's kx, ky, kz equal the reference Geometry's
    (the goldens' arrays) bit for bit."""
    from sa_gb300 import pupil_math
    g = numpy.load(GOLDEN)
    for name, cls, size in (("a", pupil_math.Geometry, 20), ("b", pupil_math.GeometrySim, 30)):
        geo = cls(size, 0.1, 0.6, 1.5, 1.4)
        assert numpy.array_equal(geo.kx, g[name + "_kx"])
        assert numpy.array_equal(geo.ky, g[name + "_ky"])
        assert numpy.array_equal(numpy.real(geo.kz), g[name + "_kz"])


def test_derivatives_are_the_translation_derivatives():
    """As the reference's tests 3, 5 and 6: the intensity derivative from
    the complex derivatives against a difference of translated intensities
    (here a central one)."""
    from oracle import pupil_fn as opf
    g = numpy.load(GOLDEN)
    o = opf.PupilFunction(g["a_kx"], g["a_ky"], g["a_kz"], 20)
    o.set_pf(g["a_pf"])
    base = (0.2, -0.1, 0.15)
    eps = 1.0e-6
    for axis, get in ((0, "get_psf_dx"), (1, "get_psf_dy"), (2, "get_psf_dz")):
        o.translate(*base)
        p = o.get_psf()
        d = getattr(o, get)()
        exact = 2.0 * (p.real * d.real + p.imag * d.imag)
        tp, tm = list(base), list(base)
        tp[axis] += eps
        tm[axis] -= eps
        o.translate(*tp)
        fp = o.get_psf_intensity()
        o.translate(*tm)
        fm = o.get_psf_intensity()
        assert numpy.abs(exact - (fp - fm) / (2 * eps)).max() < 1.0e-7, axis


def test_translation_is_a_shift():
    """As the reference's test 7: a one-pixel x translation rolls the PSF
    one pixel along the pupil's first index, whatever the size."""
    from sa_gb300 import pupil_math
    from oracle import pupil_fn as opf
    for size in (10, 20, 40):
        geo = pupil_math.Geometry(size, 0.1, 0.6, 1.5, 1.4)
        pf = geo.createFromPhase(1.0, 1.3 * geo.r * geo.r * numpy.cos(2.0 * numpy.arctan2(geo.ky, geo.kx)))
        o = opf.PupilFunction(geo.kx, geo.ky, numpy.real(geo.kz), size)
        o.set_pf(pf)
        untranslated = numpy.roll(o.get_psf_intensity(), 1, axis=0)
        o.translate(1.0, 0.0, 0.0)
        assert numpy.allclose(untranslated, o.get_psf_intensity())


def test_pfit_initialize_rejects_non_separable_kx():
    """The engine takes kx per pupil row (as pfnTranslate takes the x
    shift); pfitInitialize refuses a kx that varies along a row."""
    from sa_gb300 import loadclib, pupil_math
    if not os.path.exists(loadclib.LIB_PATH):
        pytest.skip("libsa_cuda.so is not built")
    lib = loadclib.load(require_device=False)
    geo = pupil_math.Geometry(20, 0.1, 0.6, 1.5, 1.4)
    kx = numpy.ascontiguousarray(geo.kx + 1.0e-3 * geo.ky)
    h = lib.pfnInitialize(kx, numpy.ascontiguousarray(geo.ky), numpy.ascontiguousarray(numpy.real(geo.kz)), 20)
    rqe = numpy.ones((64, 64))
    sc = numpy.zeros((64, 64))
    assert not lib.pfitInitialize(h, rqe, sc, 1.0e-6, 64, 64)
    assert "constant along" in loadclib.last_error()
    lib.saClearLastError()
    lib.pfnCleanup(h)
