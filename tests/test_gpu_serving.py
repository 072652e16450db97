"""Serving loop: continuous batching of frames of different size, model and
density.  Each request's result is the same fitted alone (its own server,
one slot) and in the mix (slots shared, lanes on separate streams, arrivals
overlapping); with FP64 lanes the results agree with the FP64 oracle within
the benchmark spec's tolerance (the FP32 engine's own parity is tested per
configuration in test_gpu_parity.py)."""
import numpy
import pytest

pytestmark = pytest.mark.gpu

MIX = [("3d", 256, 0.5), ("2d", 128, 0.3), ("Z", 128, 1.0), ("3d", 128, 2.0), ("2d", 256, 0.1),
       ("3d", 256, 1.5), ("Z", 256, 0.4), ("2d", 128, 1.2), ("spline3D", 128, 0.3)]


def make_requests():
    from sa_gb300 import synth
    reqs = []
    for i, (model, size, dens) in enumerate(MIX):
        wl = synth.serving_frame(model, size, dens, seed=100 + i)
        reqs.append({"model": model, "image": wl["images"][0], "background": wl["backgrounds"][0],
                     "peaks": wl["guesses"][0], "ptype": "hdf5", "fitter": wl["fitter"],
                     "rqe": wl["rqe"], "scmos_cal": wl["scmos_cal"], "camera": (model, size),
                     "max_iterations": 200})
    return reqs


def test_serving_alone_equals_mixed():
    from sa_gb300.serving import FitServer
    reqs = make_requests()
    alone = []
    for r in reqs:
        s = FitServer(slots=1)
        ids = s.run([r])
        alone.append(s.done[ids[0]])
        s.close()
    s = FitServer(slots=2, ticks_per_launch=2)
    arrivals = numpy.arange(len(reqs)) * 0.002
    ids = s.run(reqs, arrivals)
    lat = s.latencies(ids)
    assert numpy.all(lat > 0)
    for i, rid in enumerate(ids):
        a, b = alone[i], s.done[rid]
        for k in ("x", "y", "z", "height", "background", "status", "iterations"):
            assert numpy.array_equal(a[k], b[k]), (MIX[i], k)
    s.close()


def test_serving_results_match_oracle():
    from oracle.oracle import fit_frames
    from sa_gb300 import parity, synth
    from sa_gb300.serving import FitServer
    reqs = make_requests()[:4]
    s = FitServer(slots=2, precision=64)
    ids = s.run(reqs)
    for i, rid in enumerate(ids):
        model, size, dens = MIX[i]
        wl = synth.serving_frame(model, size, dens, seed=100 + i)
        ref = fit_frames(wl, [0])[0]
        st = parity.compare(s.done[rid], ref)
        assert st["status_agree"] >= 0.999, (MIX[i], st)
        assert parity.within_tolerance(st, min_fraction=0.999), (MIX[i], st)
    s.close()
