"""
Autotuner of the batched engine's sweep schedule.

The persistent sweep kernel's throughput depends on parameters that do not
change any result -- the scheduler reproduces the reference's update order
of every pixel whatever they are (each peak waits for the lower-index peaks
whose dilated footprints overlap its own; a trial that leaves its footprint
is rolled back and re-run):

    dilation     footprint dilation (pixels) of a fit's early sweeps: small
                 dilations let more peaks run at once but make anchor moves
                 escape (and re-run) more often
    dil_late     dilation once most peaks have converged
    dil_switch   the sweep at which the dilation changes
    ctas_per_sm  resident CTAs (4 peaks each) per SM of the persistent
                 sweep grid: more overlap of the peaks' latency chains,
                 more contention

tune() times complete fits of a sample of the workload's frames for each
candidate, one parameter at a time (coordinate descent from the default),
and returns the fastest schedule.  Every candidate's fit is checked to give
the same peaks as the first, bit for bit.
"""
import numpy

from . import loadclib
from .engine import BatchFitter

DEFAULT = {"dilation": 3, "dil_late": 0, "dil_switch": 10, "ctas_per_sm": 0}
SPACE = {"dilation": [1, 2, 3, 4], "dil_switch": [5, 10, 20], "dil_late": [0, 1], "ctas_per_sm": [3, 4, 5, 0]}


def apply(fitter, schedule):
    """Set a schedule on a BatchFitter whose frame set is not loaded yet
    (the dilation must be set before the first image).  ctas_per_sm needs
    the SM count; 0 keeps the full persistent grid."""
    lib = fitter.clib
    if lib.saSetDilation(fitter.h, int(schedule["dilation"])) != 0:
        raise RuntimeError(loadclib.last_error())
    late = min(int(schedule["dil_late"]), int(schedule["dilation"]))
    if lib.saSetSchedule(fitter.h, late, int(schedule["dil_switch"])) != 0:
        raise RuntimeError(loadclib.last_error())
    if schedule.get("ctas_per_sm"):
        import torch
        nsm = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
        lib.saSetSweepCTAs(fitter.h, int(schedule["ctas_per_sm"]) * nsm)


def _fit_time(model, shape, frames, schedule, fitter_kw, max_iterations, repeats):
    import torch
    f = BatchFitter(model, shape, len(frames["images"]), **fitter_kw)
    apply(f, schedule)
    f.load(frames["images"], frames["backgrounds"], frames["peaks"], frames.get("ptype", "hdf5"))
    best = None
    for _ in range(repeats):
        f.load_images(frames["images"])
        f.load_backgrounds(frames["backgrounds"])
        f.load_peaks(frames["peaks"], frames.get("ptype", "hdf5"))
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        f.fit(max_iterations)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        best = ms if best is None else min(best, ms)
    vals, ints = f.results_fast()
    f.close()
    return best, vals, ints


def tune(model, shape, frames, fitter_kw, max_iterations=200, repeats=2, space=None):
    """frames: dict of images (F, ny, nx), backgrounds and peaks (a list of
    per-frame peak dicts, as BatchFitter.load takes).  Returns (schedule,
    trials) with trials a list of (schedule, ms)."""
    space = dict(SPACE if space is None else space)
    for name in SPACE:
        space.setdefault(name, [])
    best = dict(DEFAULT)
    ref = None
    trials = []
    cache = {}

    def run(s):
        nonlocal ref
        key = tuple(sorted(s.items()))
        if key not in cache:
            ms, vals, ints = _fit_time(model, shape, frames, s, fitter_kw, max_iterations, repeats)
            if ref is None:
                ref = (vals, ints)
            elif not (numpy.array_equal(vals, ref[0]) and numpy.array_equal(ints, ref[1])):
                raise RuntimeError("schedule %s changed the results" % (s,))
            cache[key] = ms
            trials.append((dict(s), ms))
        return cache[key]

    best_ms = run(best)
    for name in ("dilation", "dil_switch", "dil_late", "ctas_per_sm"):
        for v in space[name]:
            cand = dict(best, **{name: v})
            ms = run(cand)
            if ms < best_ms:
                best, best_ms = cand, ms
    return best, trials


def sample(images, backgrounds, peaks, n=8):
    """The first n frames of a workload as tune() takes them."""
    n = min(n, len(images))
    return {"images": numpy.ascontiguousarray(numpy.stack(images[:n])),
            "backgrounds": numpy.ascontiguousarray(numpy.stack(backgrounds[:n])),
            "peaks": list(peaks[:n])}
