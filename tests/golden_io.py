"""Loader for the golden fixtures made by tests/golden/make_golden.py."""
import os

import numpy

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

CASES = ["g_2d", "g_2dfixed", "g_2d_rqe_finder", "g_2d_testing", "g_3d_dense", "g_Z_scmos",
         "g_spline3d", "g_spline3d_finder"]


def load_case(name):
    d = dict(numpy.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False))
    out = {"model": str(d["model"]), "ptype": str(d["ptype"]),
           "image": d["image"].astype(numpy.float64), "bg": d["bg"].astype(numpy.float64),
           "max_it": int(d["max_it"]), "nsweeps": int(d["nsweeps"]),
           "fit_sum": float(d["fit_sum"]), "fit_sq": float(d["fit_sq"]),
           "counters": d["counters"]}
    out["rqe"] = d["rqe"].astype(numpy.float64) if "rqe" in d else None
    out["scmos"] = d["scmos"].astype(numpy.float64) if "scmos" in d else None
    if out["model"].startswith("spline"):
        sp = numpy.load(os.path.join(GOLDEN, "g_spline_points.npz"))
        out["spline"] = sp["spline"].astype(numpy.float64)
    else:
        out["spline"] = None
    out["kw"] = {k[3:]: (d[k].tolist() if d[k].ndim else d[k].item()) for k in d if k.startswith("kw_")}
    if "wx_params" in out["kw"]:
        out["kw"]["wx_params"] = numpy.asarray(out["kw"]["wx_params"])
        out["kw"]["wy_params"] = numpy.asarray(out["kw"]["wy_params"])
    out["peaks"] = {k[3:]: d[k] for k in d if k.startswith("in_")}
    out["init"] = {k[5:]: d[k] for k in d if k.startswith("init_")}
    out["out"] = {k[4:]: d[k] for k in d if k.startswith("out_")}
    return out


def run_fitter(fitter, case, sweeps=None):
    """Drive any MultiFitter-like object through the fixture's call sequence."""
    fitter.newImage(case["image"])
    fitter.newBackground(case["bg"])
    fitter.newPeaks(case["peaks"], case["ptype"])
    init = {p: fitter.getPeakProperty(p) for p in ["height", "background", "error", "status"]}
    if sweeps is None:
        fitter.doFit(case["max_it"])
    else:
        for _ in range(sweeps):
            fitter.iterate()
    props = ["x", "y", "z", "height", "background", "xsigma", "ysigma", "status", "iterations",
             "error", "significance", "sum"]
    out = {p: fitter.getPeakProperty(p) for p in props}
    return init, out
