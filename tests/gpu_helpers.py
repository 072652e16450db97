"""Helpers shared by the GPU tests."""
import numpy

from golden_io import run_fitter  # noqa: F401


def make_gpu_fitter(model, image, rqe=None, scmos=None, spline=None, precision=64, device_loop=True,
                    **kw):
    from sa_gb300 import cubic_fit_c, dao_fit_c
    if model.startswith("spline"):
        sp = cubic_fit_c.SplinePSF(coeff=spline)
        cls = cubic_fit_c.CSpline3DFit if model == "spline3D" else cubic_fit_c.CSpline2DFit
        f = cls(spline_fn=sp, rqe=rqe, scmos_cal=scmos, precision=precision, device_loop=device_loop)
    else:
        cls = {"2dfixed": dao_fit_c.MultiFitter2DFixed, "2d": dao_fit_c.MultiFitter2D,
               "3d": dao_fit_c.MultiFitter3D, "Z": dao_fit_c.MultiFitterZ}[model]
        f = cls(rqe=rqe, scmos_cal=scmos, precision=precision, device_loop=device_loop, **kw)
    f.initializeC(image)
    return f


def fit_workload_gpu(wl, frames, precision, max_iterations=200):
    kw = dict(wl["fitter"])
    model = kw.pop("model")
    spline = kw.pop("spline", None)
    out = []
    f = make_gpu_fitter(model, wl["images"][frames[0]], rqe=wl["rqe"], scmos=wl["scmos_cal"],
                        spline=(spline["coeff"] if spline is not None else None),
                        precision=precision, **kw)
    for i in frames:
        f.newImage(wl["images"][i])
        f.newBackground(wl["backgrounds"][i])
        f.newPeaks(wl["guesses"][i], "hdf5")
        f.doFit(max_iterations)
        out.append({p: f.getPeakProperty(p) for p in ["x", "y", "z", "height", "background",
                                                        "status", "iterations", "error"]})
    f.cleanup(verbose=False)
    return out


def concat(results):
    keys = results[0].keys()
    return {k: numpy.concatenate([r[k] for r in results]) for k in keys}
