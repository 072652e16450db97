"""Sweep bursts launched as captured CUDA graphs give the results of the
same bursts launched kernel by kernel (SA_CUDA_GRAPHS=0): every peak's
parameters, status and iteration count, the counters and the sweep count.
The sweep epoch lives on the device, so the graphs are captured once and
relaunched unchanged."""
import os

import numpy
import pytest

pytestmark = pytest.mark.gpu

CASES = [(1, 32, {}), (2, 32, {}), (1, 64, {}), (3, 32, dict(n_emitters=60))]


def fit_once(wl, precision, graphs, refits=2):
    from sa_gb300 import cubic_fit_c, engine
    old = os.environ.get("SA_CUDA_GRAPHS")
    os.environ["SA_CUDA_GRAPHS"] = "1" if graphs else "0"
    try:
        kw = dict(wl["fitter"])
        model = kw.pop("model")
        spl = kw.pop("spline", None)
        if spl is not None:
            kw["spline"] = cubic_fit_c.SplinePSF(coeff=spl["coeff"])
        fit = engine.BatchFitter(model, (wl["ny"], wl["nx"]), len(wl["images"]), rqe=wl["rqe"],
                                 scmos_cal=wl["scmos_cal"], precision=precision, **kw)
    finally:
        if old is None:
            del os.environ["SA_CUDA_GRAPHS"]
        else:
            os.environ["SA_CUDA_GRAPHS"] = old
    outs = []
    # several fits on the same handle: the graphs are reused across fits
    for _ in range(refits):
        fit.load(numpy.stack(wl["images"]), numpy.stack(wl["backgrounds"]), wl["guesses"], "hdf5")
        sweeps = fit.fit(200)
        out = fit.results()
        out["counters"] = fit.counters()
        out["sweeps"] = sweeps
        outs.append(out)
    fit.close()
    return outs


@pytest.mark.parametrize("cfg,precision,kw", CASES)
def test_graph_bursts_give_the_kernel_by_kernel_results(cfg, precision, kw):
    from sa_gb300 import synth
    wl = synth.make_workload(cfg, frames=3, nx=128, ny=128, seed=43, **kw)
    direct = fit_once(wl, precision, False)
    graph = fit_once(wl, precision, True)
    for a, b in zip(direct, graph):
        for k in ("x", "y", "z", "height", "background", "status", "iterations"):
            assert numpy.array_equal(a[k], b[k]), k
        assert a["sweeps"] == b["sweeps"]
    # the counters accumulate over the handle's fits
    assert numpy.array_equal(direct[-1]["counters"], graph[-1]["counters"])
