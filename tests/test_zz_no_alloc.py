"""saGetFitImageNoAlloc: the fit image / residual through the library's
static device scratch, for callers that cannot allocate device memory,
compared with mFitGetFitImage / mFitGetResidual through the C ABI, two
calls in a row.  Collected last (file name) so that it also runs after
every other test has used the device."""
import numpy
import pytest

from golden_io import load_case, run_fitter
from gpu_helpers import make_gpu_fitter

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [32, 64])
def test_no_alloc_fit_image_matches(precision):
    """On a handle that has never used the allocating output path: one
    warm-up call, then two calls of each kind leave the device's free memory
    unchanged, and their outputs equal what mFitGetFitImage /
    mFitGetResidual return afterwards (bit for bit)."""
    import torch
    from sa_gb300 import loadclib
    case = load_case("g_3d_dense")
    f = make_gpu_fitter(case["model"], case["image"], rqe=case["rqe"], scmos=case["scmos"],
                        spline=case["spline"], precision=precision, **case["kw"])
    run_fitter(f, case)
    lib = loadclib.load()
    shape = case["image"].shape
    warm = numpy.zeros(shape)
    assert lib.saGetFitImageNoAlloc(f.mfit, 0, warm, 0) == 0, loadclib.last_error()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    got = {}
    for residual in (0, 1):
        got[residual] = []
        for _ in range(2):
            out = numpy.full(shape, numpy.nan)
            assert lib.saGetFitImageNoAlloc(f.mfit, 0, out, residual) == 0, loadclib.last_error()
            got[residual].append(out)
    assert torch.cuda.mem_get_info()[0] == free0
    for residual, ref_fn in ((0, lib.mFitGetFitImage), (1, lib.mFitGetResidual)):
        ref = numpy.zeros(shape)
        ref_fn(f.mfit, ref)
        for out in got[residual]:
            assert numpy.array_equal(out, ref)
    f.cleanup(verbose=False)


def test_no_alloc_rejects_large_frames_and_bad_frames():
    from sa_gb300 import loadclib
    lib = loadclib.load()
    big = numpy.ones((1100, 1000))
    h = lib.daoInitialize(big, big * 0, 1e-6, 1000, 1100, 10)
    lib.daoInitialize2DFixed(h)
    out = numpy.zeros((1100, 1000))
    assert lib.saGetFitImageNoAlloc(h, 0, out, 0) == -1
    assert "capacity" in loadclib.last_error()
    lib.daoCleanup(h)
    small = numpy.ones((64, 64))
    h = lib.daoInitialize(small, small * 0, 1e-6, 64, 64, 10)
    lib.daoInitialize2DFixed(h)
    lib.mFitNewImage(h, small)
    out = numpy.zeros((64, 64))
    assert lib.saGetFitImageNoAlloc(h, 1, out, 0) == -1
    assert lib.saGetFitImageNoAlloc(h, 0, out, 0) == 0
    lib.daoCleanup(h)
