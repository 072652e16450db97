"""
Serving loop with continuous batching for the LM fitting engine.

Requests -- one camera frame each, with its background and initial peak
guesses -- arrive over time and differ in frame size, model and emitter
density.  A request runs in a *lane*: one engine handle (frame set) for one
(model, frame size, fitter parameters, camera calibration), whose frames are
independent slots (saSlotLoad / saSlotLaunch / saSlotPoll / saSlotResults).

* Admission: a request is loaded into a free slot of its lane as soon as one
  frees up.  Lanes are created on demand while the estimated device memory of
  all lanes stays under the budget (default 40 GB); requests whose lane
  cannot be created wait until a lane drains and is retired.
* Continuous batching: a slot starts fitting while the lane's other slots
  are mid-fit (the device state machine runs every loaded slot's sweeps, a
  slot finishes independently of the others), and each lane runs on its own
  CUDA stream, so the sweeps of different lanes overlap on the device.  The
  host never waits on one lane: a lane gets its next burst of sweep ticks
  as soon as its previous burst has completed, whatever the others do.
* State stays resident: a frame's fit image and peak records live in its
  slot from admission to completion.

A frame's result does not depend on what else is in flight: its peaks only
interact with peaks of the same frame, the device reproduces the
reference's sequential peak order within a frame, and the fit image is
accumulated in fixed point (order-free).
"""
import ctypes
import time

import numpy

from . import loadclib
from .dao_fit_c import MultiFitterException, formatPeaksArbitraryPSF, formatPeaksGaussianPSF
from .engine import BatchFitter

BYTES_PER_PIXEL = {32: 40, 64: 52}   # frame state per pixel and frame
BYTES_PER_PEAK = 2 * 128 + 5 * 4 + 9 * 4


def lane_key(req):
    """Requests sharing a key can share a handle."""
    kw = req["fitter"]
    parts = [req["model"], req["image"].shape, req.get("camera", None)]
    for k in sorted(kw):
        v = kw[k]
        if isinstance(v, numpy.ndarray):
            v = tuple(numpy.asarray(v).ravel().tolist())
        elif isinstance(v, list):
            v = tuple(v)
        elif isinstance(v, dict):
            v = id(v)
        parts.append((k, v))
    return tuple(parts)


def estimate_lane_bytes(shape, slots, capacity, precision):
    npix = int(shape[0]) * int(shape[1])
    return (slots * npix * BYTES_PER_PIXEL[precision] + slots * capacity * BYTES_PER_PEAK +
            4 * npix * 8 + (1 << 20))


class Lane(object):
    def __init__(self, key, req, slots, capacity, precision, stream=None, ctas_per_slot=12):
        self.key = key
        self.model = req["model"]
        self.shape = req["image"].shape
        self.slots = slots
        self.capacity = capacity
        kw = dict(req["fitter"])
        kw.pop("model", None)
        spline = kw.pop("spline", None)
        if isinstance(spline, dict):
            from .cubic_fit_c import SplinePSF
            spline = SplinePSF(coeff=spline["coeff"])
        self._spline = spline
        self.fitter = BatchFitter(self.model, self.shape, slots, rqe=req.get("rqe"),
                                  scmos_cal=req.get("scmos_cal"), spline=spline,
                                  precision=precision, peaks_capacity=capacity, stream=stream, **kw)
        self.lib = self.fitter.clib
        # a grid sized for the lane's slots, so that lanes run side by side
        self.lib.saSetSweepCTAs(self.fitter.h, ctas_per_slot * slots)
        self.busy = [None] * slots          # request id per slot
        self.phases = numpy.zeros(slots, dtype=numpy.int32)
        self.sweeps = numpy.zeros(slots, dtype=numpy.int32)
        self.launched = False
        self.bytes = estimate_lane_bytes(self.shape, slots, capacity, precision)

    def free_slot(self):
        for i, b in enumerate(self.busy):
            if b is None:
                return i
        return -1

    def load(self, slot, rid, req):
        img = numpy.ascontiguousarray(req["image"], dtype=numpy.float64)
        bg = numpy.ascontiguousarray(req["background"], dtype=numpy.float64)
        rows = self.fitter.format(req["peaks"], req["ptype"])
        rows = numpy.ascontiguousarray(rows, dtype=numpy.float64)
        if rows.shape[0] > self.capacity:
            raise MultiFitterException("request has %d peaks, lane capacity %d" % (rows.shape[0], self.capacity))
        r = self.lib.saSlotLoad(self.fitter.h, slot, img.ctypes.data_as(ctypes.c_void_p),
                                bg.ctypes.data_as(ctypes.c_void_p), 64, rows, rows.shape[0],
                                ctypes.c_char_p(req["ptype"].encode()), int(req.get("max_iterations", 200)))
        if r != 0:
            raise MultiFitterException("saSlotLoad: " + loadclib.last_error())
        self.busy[slot] = rid

    def active(self):
        return any(b is not None for b in self.busy)

    def launch(self, ticks):
        if self.lib.saSlotLaunch(self.fitter.h, ticks) != 0:
            raise MultiFitterException("saSlotLaunch: " + loadclib.last_error())
        self.launched = True

    def ready(self):
        """True when the last launch's read-back has completed."""
        if not self.launched:
            return True
        r = self.lib.saSlotReady(self.fitter.h)
        if r < 0:
            raise MultiFitterException("saSlotReady: " + loadclib.last_error())
        return r == 1

    def poll(self):
        """Wait for the last launch; return the slots that finished."""
        if not self.launched:
            return []
        n = self.lib.saSlotPoll(self.fitter.h, self.phases, self.sweeps)
        self.launched = False
        if n < 0:
            raise MultiFitterException("saSlotPoll: " + loadclib.last_error())
        return [i for i, b in enumerate(self.busy) if b is not None and self.phases[i] == 4]

    def results(self, slot):
        n = self.capacity
        vals = numpy.zeros((n, 8), dtype=numpy.float64)
        ints = numpy.zeros((n, 2), dtype=numpy.int32)
        m = self.lib.saSlotResults(self.fitter.h, slot, vals, ints)
        if m < 0:
            raise MultiFitterException("saSlotResults: " + loadclib.last_error())
        out = {name: vals[:m, i].copy() for i, name in
               enumerate(["x", "y", "z", "height", "background", "xsigma", "ysigma", "error"])}
        out["status"] = ints[:m, 0].copy()
        out["iterations"] = ints[:m, 1].copy()
        out["sweeps"] = int(self.sweeps[slot])
        return out

    def close(self):
        self.fitter.close()


class FitServer(object):
    """Continuous-batching request loop.

    submit(req) queues a request: a dict with model, image, background, peaks
    (the newPeaks columns), ptype, fitter (constructor keywords of the model,
    as synth.fitter_kwargs gives), optional rqe / scmos_cal / camera (a label
    telling requests of different calibrations apart) and max_iterations.
    step() admits, launches and collects once; run() drives a timed stream.
    """

    def __init__(self, mem_cap_bytes=40e9, slots=8, ticks_per_launch=4, precision=32,
                 capacity_per_pixel=0.06, streams=True, ctas_per_slot=12):
        self.mem_cap = float(mem_cap_bytes)
        self.slots = int(slots)
        self.ticks = int(ticks_per_launch)
        self.precision = int(precision)
        self.cpp = float(capacity_per_pixel)
        self.use_streams = streams
        self.ctas_per_slot = int(ctas_per_slot)
        self.lanes = {}
        self.queue = []
        self.reqs = {}
        self.done = {}
        self.t_submit = {}
        self.t_done = {}
        self.next_id = 0
        self._streams = []

    def _stream(self):
        if not self.use_streams:
            return None
        try:
            import torch
            s = torch.cuda.Stream()
            self._streams.append(s)
            return s.cuda_stream
        except Exception:
            return None

    def memory_in_use(self):
        return sum(l.bytes for l in self.lanes.values())

    def submit(self, req, t=None):
        rid = self.next_id
        self.next_id += 1
        self.reqs[rid] = req
        self.queue.append(rid)
        self.t_submit[rid] = time.perf_counter() if t is None else t
        return rid

    def _lane_for(self, req):
        key = lane_key(req)
        lane = self.lanes.get(key)
        if lane is not None:
            return lane
        shape = req["image"].shape
        cap = max(100, int(self.cpp * shape[0] * shape[1]))
        need = estimate_lane_bytes(shape, self.slots, cap, self.precision)
        if self.memory_in_use() + need > self.mem_cap:
            self._retire_idle()
            if self.memory_in_use() + need > self.mem_cap:
                return None
        lane = Lane(key, req, self.slots, cap, self.precision, stream=self._stream(),
                    ctas_per_slot=self.ctas_per_slot)
        self.lanes[key] = lane
        return lane

    def _retire_idle(self):
        for key in [k for k, l in self.lanes.items() if not l.active() and not l.launched]:
            self.lanes.pop(key).close()

    def step(self):
        """One pass over the lanes without waiting on any of them: collect
        the lanes whose burst of sweep ticks has completed, admit queued
        requests into the free slots of lanes that are not running, and
        give every idle lane with work its next burst.  A lane whose frames
        take long sweeps does not hold the others back.  Returns the
        finished ids."""
        finished = []
        for lane in self.lanes.values():
            if lane.launched and lane.ready():
                for slot in lane.poll():
                    rid = lane.busy[slot]
                    self.done[rid] = lane.results(slot)
                    self.t_done[rid] = time.perf_counter()
                    lane.busy[slot] = None
                    finished.append(rid)
        waiting = []
        for rid in self.queue:
            req = self.reqs[rid]
            lane = self._lane_for(req)
            slot = lane.free_slot() if (lane is not None and not lane.launched) else -1
            if slot < 0:
                waiting.append(rid)
                continue
            lane.load(slot, rid, req)
        self.queue = waiting
        for lane in self.lanes.values():
            if not lane.launched and lane.active():
                lane.launch(self.ticks)
        return finished

    def pending(self):
        return len(self.queue) + sum(sum(b is not None for b in l.busy) for l in self.lanes.values())

    def run(self, requests, arrival_s=None):
        """Feed requests at their arrival times (seconds from the start; None:
        all at once) and run until every one has finished.  Returns the ids in
        input order; latencies in self.latencies()."""
        t0 = time.perf_counter()
        order = list(range(len(requests)))
        ids = [None] * len(requests)
        k = 0
        while k < len(order) or self.pending():
            now = time.perf_counter() - t0
            while k < len(order) and (arrival_s is None or arrival_s[order[k]] <= now):
                i = order[k]
                ids[i] = self.submit(requests[i], t=t0 + (0.0 if arrival_s is None else arrival_s[i]))
                k += 1
            if self.pending():
                if not self.step():
                    time.sleep(2e-5)   # every lane mid-burst
            elif k < len(order):
                time.sleep(max(0.0, min(0.001, arrival_s[order[k]] - now)))
        return ids

    def latencies(self, ids):
        return numpy.array([self.t_done[i] - self.t_submit[i] for i in ids])

    def close(self):
        for lane in self.lanes.values():
            lane.close()
        self.lanes = {}
