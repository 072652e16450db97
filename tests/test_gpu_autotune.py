"""The sweep-schedule autotuner (sa_gb300.autotune): every schedule it tries
gives bit-identical results (the scheduler keeps the reference's update
order of every pixel), and the schedule it picks is one it timed."""
import pytest

pytestmark = pytest.mark.gpu


def test_autotune_schedules_are_result_invariant():
    from sa_gb300 import autotune, synth
    wl = synth.make_workload(1, frames=3, nx=256, ny=256, seed=5)
    kw = dict(wl["fitter"])
    model = kw.pop("model")
    frames = autotune.sample(wl["images"], wl["backgrounds"], wl["guesses"], n=3)
    space = {"dilation": [1, 3], "dil_switch": [5, 10], "dil_late": [0, 1], "ctas_per_sm": [2, 0]}
    best, trials = autotune.tune(model, (wl["ny"], wl["nx"]), frames, kw, repeats=1, space=space)
    assert len(trials) >= 5
    assert any(t[0] == best for t in trials)
    assert min(ms for _, ms in trials) == [ms for s, ms in trials if s == best][0]
