"""CPU checks of the engine library: it builds, loads, exports every entry
point its header declares, and refuses to run without a GPU."""
import os
import re
import subprocess

import numpy
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "sa_cuda.h")


def header_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", src)
    skip = {"if", "for", "while", "return", "sizeof"}
    return sorted(set(n for n in names if n not in skip))


@pytest.fixture(scope="module")
def lib():
    from sa_gb300 import build, loadclib
    build.build()
    return loadclib.load(require_device=False)


def test_library_exports_header(lib):
    from sa_gb300 import loadclib
    nm = subprocess.run(["nm", "-D", "--defined-only", loadclib.LIB_PATH], capture_output=True,
                        text=True, check=True).stdout
    exported = set(line.split()[-1] for line in nm.splitlines() if " T " in line)
    declared = header_functions()
    assert len(declared) > 50
    missing = [n for n in declared if n not in exported]
    assert missing == []
    assert sorted(loadclib.EXPORTS) == sorted(declared)


def test_no_device_here_fails_loudly(lib):
    from sa_gb300 import dao_fit_c, loadclib
    if lib.saDeviceCount() > 0:
        pytest.skip("a GPU is visible")
    with pytest.raises(loadclib.EngineUnavailable):
        dao_fit_c.MultiFitter2D(sigma_range=[1.0, 2.0])


def test_handle_layout_matches_reference_fitdata(lib):
    """Fields Python reads through the reference's ctypes mirror of fitData
    (sa_library/dao_fit_c.py:22-77) sit at the same offsets."""
    import ctypes
    from sa_gb300 import loadclib
    s = loadclib.saFitData
    ints = ["n_dposv", "n_iterations", "n_lost", "n_margin", "n_neg_fi", "n_neg_height",
            "n_non_converged", "n_non_decr", "fit_size_x", "fit_size_y", "image_size_x",
            "image_size_y", "jac_size", "max_nfit", "nfit", "roi_n_index"]
    for i, n in enumerate(ints):
        assert getattr(s, n).offset == 4 * i
    assert s.minimum_height.offset == 64
    assert s.roi_x_index.offset == 64 + 5 * 8 + ctypes.sizeof(ctypes.c_void_p)


def test_handle_creation_without_device(lib):
    """Handle set-up is host-only; ROI geometry follows multi_fit.c:1031-1060."""
    from sa_gb300 import loadclib
    from oracle.oracle import OracleFitter
    img = numpy.ones((40, 40))
    for r in [7, 8, 9, 12, 15, 20]:
        h = lib.daoInitialize(img, numpy.zeros((40, 40)), 1e-6, 40, 40, r)
        lib.daoInitialize2DFixed(h)
        c = h.contents
        n = c.roi_n_index
        rx = numpy.array([c.roi_x_index[i] for i in range(n)])
        ry = numpy.array([c.roi_y_index[i] for i in range(n)])
        o = OracleFitter("2dfixed", (40, 40), roi_size=r)
        ox, oy = o.roiIndex()
        assert numpy.array_equal(rx, ox) and numpy.array_equal(ry, oy)
        assert c.jac_size == 4 and c.fit_size_x == r
        assert abs(c.xoff - (0.5 * r - 1.0)) < 1e-15
        lib.daoCleanup(h)
        o.cleanup()


def test_bad_inputs_report_errors(lib):
    from sa_gb300 import loadclib
    img = numpy.ones((40, 40))
    assert not lib.daoInitialize(img, img, 1e-6, 40, 40, 1)
    assert "ROI" in loadclib.last_error()
    sp = lib.initSpline2D(numpy.zeros(6 * 5 * 16), 6, 5)
    assert not lib.cfInitialize(sp, img, img, 1e-6, 40, 40)
    assert "square" in loadclib.last_error()
    lib.splineCleanup(sp)
    h = lib.daoInitialize(img, img * 0, 1e-6, 40, 40, 10)
    lib.daoInitialize2DFixedALS(h)
    assert "MLE" in loadclib.last_error()
    lib.daoCleanup(h)


def test_synthetic_workloads_shapes():
    from sa_gb300 import synth
    wl = synth.make_workload(1, frames=2, nx=128, ny=128)
    assert len(wl["images"]) == 2 and wl["images"][0].shape == (128, 128)
    assert (wl["images"][0] >= 1.0).all()
    g = wl["guesses"][0]
    assert set(g) >= {"x", "y", "z", "background", "height", "xsigma", "ysigma"}
    wl3 = synth.make_workload(3, frames=1, nx=64, ny=64, n_emitters=5)
    assert wl3["spline"]["coeff"].shape == (20, 20, 20, 64)


def test_spline_handle_from_reference_library(lib):
    """cfInitialize accepts a spline made by the reference's own
    initSpline3D (spliner/cubic_spline.c:749, splineData layout
    cubic_spline.h:16-26), as the reference's cubic_spline_c.py would pass
    it after a library swap, and cfCleanup frees it."""
    import ctypes
    import os
    ref = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref",
                       "libcubic_fit.so")
    if not os.path.exists(ref):
        pytest.skip("the reference's compiled C is not present")
    rlib = ctypes.CDLL(ref)
    f64 = numpy.ctypeslib.ndpointer(dtype=numpy.float64, flags="C_CONTIGUOUS")
    rlib.initSpline3D.argtypes = [f64, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    rlib.initSpline3D.restype = ctypes.c_void_p
    coeff = numpy.random.default_rng(3).uniform(0, 1, 9 * 9 * 9 * 64)
    img = numpy.ones((40, 40))
    geo = []
    for make in (rlib.initSpline3D, lib.initSpline3D):
        sp = make(coeff, 9, 9, 9)
        h = lib.cfInitialize(sp, img, img * 0, 1e-6, 40, 40)
        assert h, "cfInitialize refused the spline"
        lib.cfInitialize3D(h)
        c = h.contents
        geo.append((c.roi_n_index, c.fit_size_x, c.jac_size, c.xoff))
        lib.cfCleanup(h)
    assert geo[0] == geo[1] and geo[0][1] == 8 and geo[0][2] == 5


def _declared(header):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", src)
    return sorted(set(names) - {"if", "for", "while", "return", "sizeof"})


def _exported(path):
    nm = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True,
                        check=True).stdout
    return set(line.split()[-1] for line in nm.splitlines() if " T " in line)


def test_finder_exports_header(lib):
    """The peak finder's entry points (include/sa_finder.h) are exported by
    libsa_cuda.so, and libsa_matched_filter.so exports the reference's
    matched-filter names (include/sa_matched_filter.h)."""
    from sa_gb300 import loadclib
    declared = _declared("sa_finder.h")
    assert len(declared) >= 30
    assert [n for n in declared if n not in _exported(loadclib.LIB_PATH)] == []
    assert sorted(loadclib.FINDER_EXPORTS) == declared
    mf = _declared("sa_matched_filter.h")
    assert mf == ["cleanup", "convolve", "convolveMemo", "initialize"]
    assert sorted(loadclib.MATCHED_FILTER_EXPORTS) == mf
    assert set(mf) <= _exported(loadclib.MF_LIB_PATH)
    ia = _declared("sa_ia_utilities.h")
    assert sorted(loadclib.IA_UTILITIES_EXPORTS) == ia and len(ia) == 8
    assert set(ia) <= _exported(loadclib.IA_LIB_PATH)


def test_finder_without_device_fails_loudly(lib):
    """No CUDA device: the finder classes raise and the C entry points
    return NULL with a recorded message -- there is no CPU fallback."""
    from sa_gb300 import fitting, loadclib, matched_filter_c
    if lib.saDeviceCount() > 0:
        pytest.skip("a GPU is visible")
    with pytest.raises(loadclib.EngineUnavailable):
        matched_filter_c.MatchedFilter(numpy.ones((8, 8)))
    with pytest.raises(loadclib.EngineUnavailable):
        fitting.PeakFinderGaussian({"find_max_radius": 5, "iterations": 1, "sigma": 1.5, "threshold": 6.0,
                                    "background_sigma": 8.0, "roi_size": 18})
    psf = numpy.zeros((16, 16))
    psf[0, 0] = 1.0
    lib.saClearLastError()
    assert not lib.saFilterCreate(psf, 0.0, 16, 16, 0)
    assert "saFilterCreate" in loadclib.last_error() or "failed" in loadclib.last_error()


def test_find_fit_loop_without_device_fails_loudly(lib):
    """The find / fit loop and the frame readers need the GPU: without one
    they raise instead of running anything on the host."""
    from sa_gb300 import find_peaks, loadclib
    if lib.saDeviceCount() > 0:
        pytest.skip("a GPU is visible")
    params = {"find_max_radius": 5, "iterations": 1, "sigma": 1.5, "threshold": 6.0, "background_sigma": 8.0,
              "roi_size": 18, "model": "3d"}
    with pytest.raises(loadclib.EngineUnavailable):
        find_peaks.initFindAndFit(params)
