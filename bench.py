#!/usr/bin/env python
"""
bench.py -- localizations/s of the multi-emitter Levenberg-Marquardt fitting
step (storm-analysis 3D-DAOSTORM '3d' model) on GB300.

Workload (one "step"): benchmark configuration 1 -- 64 frames of 512 x 512,
Poisson(0.5 / um^2) emitters per frame (~3355, overlapping ROIs), '3d'
Gaussian model, MLE, roi_size 18, tolerance 1e-6, at most 200 sweeps, seeded
synthetic data, initial guesses = truth + jitter ("hdf5" peak format).  One
step fits all 64 frames to termination through the batched engine.

  value   localizations/s with the frames, backgrounds and peak rows already
          resident in HBM (device pointers into the engine's C ABI)
  e2e     the same through the public API with pinned host buffers: host ->
          device copies of images, backgrounds and peak rows and the
          device -> host read of all results inside the timed region
  plain   the one-frame-per-launch GPU fitter (MultiFitter with the
          reference's host-driven sweep loop), for comparison
  cpu_baseline  the FP64 CPU oracle (our C restatement of the reference's
          fitter) on the host cores, one process per core, a bounded sample
  finder  the GPU peak finder (matched filters + local maxima) on the same
          frames, mirror-padded, with its own CPU baseline (the oracle); its
          e2e starts from raw uint16 camera frames (GPU ingest: ADU to e-,
          clip, mirror pad), and "ingest" times that kernel alone
  culling the post-fit culling (markDimmerPeaks, markLowSignificancePeaks)
          on the step's fitted peaks, per frame, reference call shape
  analysis  the whole per-frame find / fit loop (sa_gb300.find_peaks) on two
          of the frames, with the oracle's loop on one frame beside it;
          analysis_batch the same loop for all frames at once (BatchFindFit)

`python bench.py --impl reference` times the CPU oracle on all host cores on
the same workload and prints the same JSON line with "impl": "reference".

Multi-GPU: frames are independent and a frame does not shard, so N GPUs run
N independent replicas (weak scaling); no collective is on the data path.
"""
import argparse
import ctypes
import json
import math
import multiprocessing
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "storm-analysis_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

MAX_IT = 200


# ----------------------------------------------------------------------------
# CPU side (oracle); workers are spawned, never forked from a CUDA process
# ----------------------------------------------------------------------------

PARITY_PROPS = ("x", "y", "z", "height", "background", "xsigma", "ysigma", "status", "iterations")


def _cpu_worker(args):
    """Fit frames with the oracle (one process); returns (peaks, seconds,
    [(frame index, properties)]).  lib selects the oracle build."""
    import oracle.oracle as O
    frames, fitter_kw, shape, rqe, scmos, lib = args
    O.LIB = os.path.join(ROOT, "oracle", lib)
    kw = dict(fitter_kw)
    model = kw.pop("model")
    spline = kw.pop("spline", None)
    if model == "pupil":
        # the oracle takes the pupil function as pfnInitialize / pfnSetPF do
        from sa_gb300 import pupil_math
        pf_data = kw.pop("pf_data")
        cls = pupil_math.GeometrySim if pf_data["geo_sim_pf"] else pupil_math.Geometry
        geo = cls(pf_data["pf"].shape[0], pf_data["pixel_size"], pf_data["wavelength"],
                  pf_data["immersion_index"], pf_data["numerical_aperture"])
        kw = {"pupil": (geo.kx, geo.ky, numpy.real(geo.kz), pf_data["pf"]),
              "min_z": kw.pop("zmin"), "max_z": kw.pop("zmax")}
    f = O.OracleFitter(model, shape, rqe=rqe, scmos_cal=scmos,
                       spline=(spline["coeff"] if spline is not None else None), **kw)
    n = 0
    out = []
    t0 = time.perf_counter()
    for idx, img, bg, g in frames:
        f.newImage(img)
        f.newBackground(bg)
        f.newPeaks(g, "hdf5")
        f.doFit(MAX_IT)
        n += f.getNFit()
        out.append((idx, {p: f.getPeakProperty(p) for p in PARITY_PROPS}))
    dt = time.perf_counter() - t0
    f.cleanup()
    return n, dt, out


def cpu_sample(wl, n_frames, cores, pool, lib="liboracle.so"):
    """Fit n_frames of the workload on `cores` processes, each frame as the
    GPU sees it (images and backgrounds rounded to float32); returns
    (peaks, wall s, {frame: properties})."""
    shape = (wl["ny"], wl["nx"])
    jobs = [[] for _ in range(cores)]
    f32 = lambda a: numpy.asarray(a, dtype=numpy.float32).astype(numpy.float64)
    for i in range(n_frames):
        f = i % len(wl["images"])
        jobs[i % cores].append((f, f32(wl["images"][f]), f32(wl["backgrounds"][f]), wl["guesses"][f]))
    args = [(j, wl["fitter"], shape, wl["rqe"], wl["scmos_cal"], lib) for j in jobs if j]
    t0 = time.perf_counter()
    res = pool.map(_cpu_worker, args, chunksize=1)
    wall = time.perf_counter() - t0
    return sum(r[0] for r in res), wall, {idx: props for r in res for idx, props in r[2]}


def build_oracle():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "liboracle.so", "liboracle_timing.so"],
                   check=True)


def parity_block(vals, ints, counts, oracle_frames):
    """Per-peak agreement of the GPU step's results with the oracle's fits of
    the same frames (spec tolerance: status agreement >= 99.9 %, and
    for peaks converged in both |dx|, |dy| <= 1e-4 px, |dz| <= 1e-3,
    relative height / background <= 1e-4 for >= 99.9 % of them)."""
    from sa_gb300 import parity
    edges = numpy.concatenate([[0], numpy.cumsum(counts)])
    cols = {"x": 0, "y": 1, "z": 2, "height": 3, "background": 4, "xsigma": 5, "ysigma": 6}
    got = {k: [] for k in PARITY_PROPS}
    ref = {k: [] for k in PARITY_PROPS}
    for f in sorted(oracle_frames):
        a, b = edges[f], edges[f + 1]
        for k in PARITY_PROPS:
            if k in cols:
                got[k].append(vals[a:b, cols[k]])
            else:
                got[k].append(ints[a:b, 0 if k == "status" else 1])
            ref[k].append(oracle_frames[f][k])
    got = {k: numpy.concatenate(v) for k, v in got.items()}
    ref = {k: numpy.concatenate(v) for k, v in ref.items()}
    st = parity.compare(got, ref)
    fr = [st[k] for k in ("frac_ok_dx", "frac_ok_dy", "frac_ok_dz", "frac_ok_rel_h", "frac_ok_rel_bg") if k in st]
    return {"frames": len(oracle_frames), "peaks": st["n"], "status_agree": st["status_agree"],
            "frac_within": min(fr) if fr else 1.0,
            "max_dx": st.get("max_dx"), "max_dy": st.get("max_dy"), "max_dz": st.get("max_dz"),
            "max_rel_height": st.get("max_rel_h"), "max_rel_background": st.get("max_rel_bg"),
            "iterations_equal": float(numpy.mean(got["iterations"] == ref["iterations"])),
            "bar": {"status_agree": parity.TOL["status"], "frac_within": 0.999, "xy_px": parity.TOL["xy"],
                    "z": parity.TOL["z"], "rel_height_background": parity.TOL["rel"]},
            "oracle": "FP64 restatement of the reference's C (oracle/sa_oracle.c), on the same float32 frames"}


# ----------------------------------------------------------------------------
# clocks
# ----------------------------------------------------------------------------

class ClockSampler(object):
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self.thread is not None:
            self.thread.join(timeout=2)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------------------
# GPU side
# ----------------------------------------------------------------------------

def flops_per_iteration(model, nroi):
    """Algorithmic FP32 work of one LM inner iteration of one peak (counted per
    ROI pixel): Jacobian row + normal-equation accumulation 2(k(k+1)/2 + k) + 3k + 5,
    the model (1) and the error / add / subtract terms (20)."""
    k = {"2dfixed": 4, "2d": 5, "3d": 6, "Z": 5, "spline2D": 4, "spline3D": 5}[model]
    per_px = 2 * (k * (k + 1) // 2 + k) + 3 * k + 5 + 1 + 20
    if model.startswith("spline"):
        per_px += 512
    return per_px * nroi


def roi_pixels(roi):
    c = 0.5 * roi
    n = 0
    for i in range(roi):
        for j in range(roi):
            if ((j - c + 0.5) ** 2 + (i - c + 0.5) ** 2) <= c * c:
                n += 1
    return n


def load_profile_traffic():
    """DRAM bytes of sweep-kernel launches from one ncu capture (see
    profiles/k_sweep_cfg1.md), per frame of the workload."""
    p = os.path.join(ROOT, "profiles", "k_sweep_cfg1_traffic.json")
    if os.path.exists(p):
        with open(p) as fp:
            return json.load(fp)
    return None


def load_measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fp:
            return json.load(fp)
    return {}


def bytes_per_iteration(nroi):
    """Algorithmic bytes of one LM inner iteration of one peak: per ROI pixel
    the start state (fit image and background words 8 + 8, count 4, the
    fixed-point data 8, rqe 4) read once and the fit-image / background
    update (8 + 8) written once: 48 B."""
    return 48 * nroi


def peaks_rows(wl):
    from sa_gb300.dao_fit_c import formatPeaksArbitraryPSF, formatPeaksGaussianPSF
    fmt = formatPeaksArbitraryPSF if wl["model"].startswith("spline") else formatPeaksGaussianPSF
    rows = [fmt(g, "hdf5") for g in wl["guesses"]]
    counts = numpy.array([r.shape[0] for r in rows], dtype=numpy.int32)
    return numpy.ascontiguousarray(numpy.concatenate(rows)), counts


def run_ours(args, rank, world, local_rank):
    import torch
    from sa_gb300 import engine, loadclib, replicas, synth

    lib = loadclib.load()
    lib.saSetDevice(local_rank)
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    cfg = args.config
    wl = synth.make_workload(cfg, frames=args.frames, seed=replicas.replica_seed(cfg, rank))
    kw = dict(wl["fitter"])
    model = kw.pop("model")
    spl = kw.pop("spline", None)
    spline_psf = None
    if spl is not None:
        from sa_gb300 import cubic_fit_c
        spline_psf = cubic_fit_c.SplinePSF(coeff=spl["coeff"])
        kw["spline"] = spline_psf
    F = len(wl["images"])
    shape = (wl["ny"], wl["nx"])
    images = numpy.ascontiguousarray(numpy.stack(wl["images"]).astype(numpy.float32))
    bgs = numpy.ascontiguousarray(numpy.stack(wl["backgrounds"]).astype(numpy.float32))
    rows, counts = peaks_rows(wl)
    units = int(counts.sum())

    fit = engine.BatchFitter(model, shape, F, rqe=wl["rqe"], scmos_cal=wl["scmos_cal"],
                             precision=args.precision, peaks_capacity=int(counts.max()), **kw)
    # resident inputs
    d_img = torch.from_numpy(images).cuda()
    d_bg = torch.from_numpy(bgs).cuda()
    d_rows = torch.from_numpy(rows).cuda()
    torch.cuda.synchronize()

    def step_resident():
        fit.load_images(d_img.data_ptr(), on_device=True, dtype_bits=32)
        fit.load_backgrounds(d_bg.data_ptr(), on_device=True, dtype_bits=32)
        fit.load_peaks_device(d_rows.data_ptr(), counts, "hdf5")
        fit.fit(MAX_IT)

    p_img = torch.from_numpy(images).pin_memory()
    p_bg = torch.from_numpy(bgs).pin_memory()
    p_rows = torch.from_numpy(rows).pin_memory()
    p_img_np, p_bg_np, p_rows_np = p_img.numpy(), p_bg.numpy(), p_rows.numpy()
    out_vals = {}

    def step_e2e():
        fit.load_images(p_img_np)
        fit.load_backgrounds(p_bg_np)
        fit.clib.saNewPeaksBatch(fit.h, p_rows_np, counts, F, b"hdf5")
        fit.fit(MAX_IT)
        out_vals["v"] = fit.results_fast()

    def timed(fn, k):
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(k):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return replicas.max_over_ranks(e0.elapsed_time(e1) / k, dist, device="cuda")

    for _ in range(args.warmup):
        step_resident()
    launches0 = fit.kernel_launches()
    clocks = ClockSampler(local_rank)
    clocks.start()
    ms_value = timed(step_resident, args.steps)
    clk = clocks.stop()
    launches = (fit.kernel_launches() - launches0) // max(args.steps, 1)

    # roofline pass: one resident step with the sweep kernels timed by events
    c0 = fit.counters()
    fit.set_timing(True)
    step_resident()
    per_sweep = fit.sweep_times()
    sweep_ms, sweep_launches, ticks = fit.timing()
    fit.set_timing(False)
    c1 = fit.counters()
    iters = int(c1[1] - c0[1])
    roi = kw.get("roi_size", 10) if spl is None else spl["coeff"].shape[0] - 1
    nroi = roi_pixels(roi)
    flops = flops_per_iteration(model, nroi) * iters
    res_vals, res_ints = fit.results_fast()
    status = res_ints[:, 0]

    for _ in range(max(1, args.warmup // 2)):
        step_e2e()
    ms_e2e = timed(step_e2e, args.steps)
    h2d = images.nbytes + bgs.nbytes + rows.nbytes + counts.nbytes
    d2h = int(units * 128)

    # plain one-frame-per-launch fitter (host-driven sweep loop), bounded sample
    plain = None
    if not args.no_plain and rank == 0:
        from sa_gb300 import cubic_fit_c, dao_fit_c
        if spline_psf is not None:
            pf = cubic_fit_c.CSpline3DFit(spline_fn=spline_psf, rqe=wl["rqe"], scmos_cal=wl["scmos_cal"],
                                          precision=args.precision, device_loop=False)
        else:
            cls = {"2d": dao_fit_c.MultiFitter2D, "3d": dao_fit_c.MultiFitter3D,
                   "Z": dao_fit_c.MultiFitterZ, "2dfixed": dao_fit_c.MultiFitter2DFixed}[model]
            pf = cls(rqe=wl["rqe"], scmos_cal=wl["scmos_cal"], precision=args.precision, device_loop=False,
                     **kw)
        pf.initializeC(wl["images"][0])
        nplain = min(args.plain_frames, F)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        n = 0
        for i in range(nplain):
            pf.newImage(wl["images"][i])
            pf.newBackground(wl["backgrounds"][i])
            pf.newPeaks(wl["guesses"][i], "hdf5")
            pf.doFit(MAX_IT)
            n += pf.getNFit()
            pf.getPeakProperty("x")
        plain = {"value": n / (time.perf_counter() - t0), "frames": nplain}
        pf.cleanup(verbose=False)

    value = replicas.job_throughput(units, world, ms_value)
    e2e = replicas.job_throughput(units, world, ms_e2e)
    props = torch.cuda.get_device_properties(local_rank)
    nsm = props.multi_processor_count
    mx = clk["sm_max_mhz"] or 2070.0
    if args.precision == 32:
        peak_tf = nsm * 128 * 2 * mx * 1e6 / 1e12
        bound = "fp32"
    else:
        peak_tf = 1.25
        bound = "fp64"
    achieved = flops / (sweep_ms / 1e3) / 1e12 if sweep_ms > 0 else None
    traffic = load_profile_traffic()
    peaks = load_measured_peaks()
    hbm_peak = peaks.get("hbm_gbs")
    alg_bytes = bytes_per_iteration(nroi) * iters if nroi else None
    hbm_achieved = alg_bytes / (sweep_ms / 1e3) / 1e9 if (alg_bytes and sweep_ms > 0) else None
    # DRAM bytes per launch: the ncu capture's bytes per LM step of a first
    # sweep times this step's average LM iterations per sweep launch
    traffic_launch = None
    if traffic and traffic.get("dram_bytes_per_step_first_sweep") and sweep_launches:
        traffic_launch = traffic["dram_bytes_per_step_first_sweep"] * iters / float(sweep_launches)
    alg_launch = alg_bytes / float(sweep_launches) if (alg_bytes and sweep_launches) else None
    line = {
        "metric": "localizations/s (LM to convergence)",
        "value": value,
        "unit": "localizations/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_value,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": ("f32 (float-float gradient, error change and solve refinement)"
                  if args.precision == 32 else "f64"),
        "data": "synthetic (seeded, benchmark configuration %d shapes)" % cfg,
        "config": {"workload": "cfg%d: %s model, %d frames %dx%d, %d emitters, roi %s, max %d sweeps"
                               % (cfg, model, F, shape[1], shape[0], units, roi, MAX_IT),
                   "frames_per_step": F, "localizations_per_step": units,
                   "l2": "working set %.2f GB per step > 129 MB L2" % (F * shape[0] * shape[1] * 32 / 1e9),
                   "parallelism": "replicas x%d" % world},
        "e2e": {"value": e2e, "unit": "localizations/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": d2h, "ms_per_step": ms_e2e},
        "gpu_launches": int(launches * args.steps),
        "clocks": clk,
        "roofline": {"bound": "hbm", "kernel": "k_sweep", "achieved": hbm_achieved,
                     "peak": hbm_peak, "unit": "GB/s",
                     "frac": (hbm_achieved / hbm_peak) if (hbm_achieved and hbm_peak) else None,
                     "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if hbm_peak else None,
                     "traffic": traffic_launch,
                     "algorithmic_bytes_per_launch": alg_launch,
                     "traffic_note": "ncu DRAM read+write bytes per LM step of a first-sweep launch "
                                     "(16-frame capture) times this step's LM iterations per sweep launch"
                     if traffic_launch else None,
                     "bytes_per_iteration": bytes_per_iteration(nroi) if nroi else None,
                     "sweep_launches": int(sweep_launches), "sweep_ms_per_step": sweep_ms,
                     "lm_iterations_per_step": iters,
                     "sweep_ms_first5": [round(float(v), 3) for v in per_sweep[:5]],
                     "sweep_ms_median_after20": float(numpy.median(per_sweep[20:])) if per_sweep.size > 20 else None,
                     "sweep_ms_sum_after20": float(per_sweep[20:].sum()) if per_sweep.size > 20 else None},
        "roofline_fp32": {"bound": bound, "kernel": "k_sweep", "achieved": achieved, "peak": peak_tf,
                          "unit": "TFLOP/s", "frac": (achieved / peak_tf) if achieved else None,
                          "peak_source": "nominal %d SMs x 128 FP32 lanes x 2 x %.0f MHz" % (nsm, mx)
                          if bound == "fp32" else "nominal FP64",
                          "flops_per_iteration": flops_per_iteration(model, nroi)},
        "fit": {"converged": int((status == 1).sum()), "error": int((status == 2).sum()),
                "running": int((status == 0).sum()), "sweeps": fit.sweeps,
                "scheduler": fit.sched_stats()},
    }
    if plain is not None:
        line["plain_gpu"] = {"value": plain["value"], "unit": "localizations/s",
                             "frames": plain["frames"], "speedup_batched_vs_plain": value / world / plain["value"]}
    if rank == 0 and not args.no_cpu:
        build_oracle()
        cores = args.cpu_cores or os.cpu_count()
        ctx = multiprocessing.get_context("spawn")
        nf = min(cores, F)
        with ctx.Pool(cores) as pool:
            # timed: the oracle built as the reference's C is built; then the
            # parity oracle (no floating-point contraction) on the same frames
            n_cpu, wall, _ = cpu_sample(wl, nf, cores, pool, lib="liboracle_timing.so")
            _, wall_p, ora = cpu_sample(wl, nf, cores, pool)
            if not args.no_configs:
                line["configs"] = run_config_reports(args, pool, cores)
        line["cpu_baseline"] = {"value": n_cpu / wall, "unit": "localizations/s", "cores": cores,
                                "kind": "port", "sample": "%d frames of the step's workload, one "
                                "process per core, %.1f s wall" % (nf, wall),
                                "build": "oracle/sa_oracle.c with the reference's compiler flags (-O3)",
                                "port_vs_reference_c": "the port's speed is within 5-10 %% of the reference's own C "
                                "compiled from its sources (x86 build machine, same frames); %.1f s wall for the "
                                "no-contraction parity build" % wall_p}
        line["parity"] = parity_block(res_vals, res_ints, counts, ora)
    if rank == 0 and not args.no_serving:
        line["serving"] = run_serving_block(args, local_rank)
    if rank == 0 and not args.no_finder:
        line["finder"] = run_finder(args, wl, torch)
        line["culling"] = run_culling(args, fit)
        line["analysis"] = run_analysis(args, wl)
        line["analysis_batch"] = run_analysis_batch(args, wl)
    if dist is not None:
        dist.destroy_process_group()
    fit.close()
    if rank == 0:
        print(json.dumps(line), flush=True)


FINDER_PARAMS = dict(background_sigma=8.0, foreground_sigma=1.0, find_max_radius=5, iterations=20,
                     sigma=1.5, threshold=6.0, roi_size=18)


def run_finder(args, wl, torch):
    """The GPU peak finder (PeakFinderGaussian.peakFinder with background
    estimation) over the step's frames, mirror-padded by the finder margin
    (11 px for roi 18): one finder step = newImages + estimateBackground +
    findPeaks for all frames.  Two frame sets alternate between steps (the
    second is each frame flipped top to bottom) so that the memoised
    matched filters convolve every step, as they do on a movie."""
    from sa_gb300 import fitting
    margin = int(FINDER_PARAMS["roi_size"] / 2 + 2)
    frames = numpy.ascontiguousarray(numpy.stack([fitting.padArray(im, margin) for im in wl["images"]]))
    alt = numpy.ascontiguousarray(frames[:, ::-1, :])
    F = frames.shape[0]
    shape = frames.shape[1:]
    d_sets = [torch.from_numpy(frames).cuda(), torch.from_numpy(alt).cuda()]
    # the e2e path starts from raw camera frames: ADU = e- x gain + offset as
    # uint16 (what a .dax movie holds), converted and padded on the GPU
    gain, offset = 2.0, 100.0
    raw = numpy.clip(numpy.rint(numpy.stack(wl["images"]) * gain + offset), 0, 65535).astype(numpy.uint16)
    p_raw = [torch.from_numpy(raw).pin_memory().numpy(),
             torch.from_numpy(numpy.ascontiguousarray(raw[:, ::-1, :])).pin_memory().numpy()]
    lib = fitting.loadclib.load()
    ih = lib.saIngestCreate(raw.shape[1], raw.shape[2], margin, None, None, offset, 1.0 / gain, 1)
    torch.cuda.synchronize()
    bf = fitting.BatchPeakFinder(FINDER_PARAMS, shape, F)
    found = []
    count = [0]

    def step(host=False):
        # strictly alternating frame sets, across warm-up and timed steps:
        # a repeated set would let the memoised filters skip their work
        i = count[0]
        count[0] += 1
        if host:
            lib.saIngestFrames(ih, p_raw[i % 2].ctypes.data_as(ctypes.c_void_p), F, 16, 0, 0, None)
            bf.newImages(lib.saIngestResultDevice(ih))
        else:
            bf.newImages(d_sets[i % 2])
        bf.estimateBackground()
        bf.findPeaks()
        found.append(bf.total)
        if host:
            bf.peaks()

    def timed(k, host=False):
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(k):
            step(host)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / k

    for _ in range(max(args.warmup, 3)):
        step()
    l0 = bf.kernel_launches()
    del found[:]
    ms = timed(args.steps)
    launches = (bf.kernel_launches() - l0) // max(args.steps, 1)
    mean_found = float(numpy.mean(found))
    ms_e2e = timed(args.steps, host=True)
    # ingest alone (device raw frames -> padded photo-electrons), HBM roofline
    d_raw = torch.from_numpy(raw).cuda()
    torch.cuda.synchronize()
    for _ in range(3):
        lib.saIngestFrames(ih, ctypes.c_void_p(d_raw.data_ptr()), F, 16, 0, 1, None)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(max(args.steps, 5)):
        lib.saIngestFrames(ih, ctypes.c_void_p(d_raw.data_ptr()), F, 16, 0, 1, None)
    e1.record()
    torch.cuda.synchronize()
    ms_ingest = e0.elapsed_time(e1) / max(args.steps, 5)
    lib.saIngestCleanup(ih)
    ingest_bytes = raw.nbytes + frames.nbytes
    hbm_peak = load_measured_peaks().get("hbm_gbs")
    ingest_gbs = ingest_bytes / (ms_ingest / 1e3) / 1e9
    taps = 0
    for f in (bf.bg_filter, bf.fg_mfilter, bf.fg_vfilter):
        if f is not None:
            info = f.info()
            taps += (info[1] + info[2]) if info[0] else info[1] * info[2]
    flops = 2.0 * taps * F * shape[0] * shape[1]
    achieved = flops / (ms / 1e3) / 1e12
    out = {"metric": "frames/s (peak finding: background + matched filters + local maxima)",
           "value": F / (ms / 1e3), "unit": "frames/s", "ms_per_step": ms,
           "frames_per_step": F, "frame": "%dx%d padded (margin %d)" % (shape[1], shape[0], margin),
           "peaks_found_per_step": mean_found,
           "params": FINDER_PARAMS,
           "gpu_launches_per_step": int(launches),
           "e2e": {"value": F / (ms_e2e / 1e3), "unit": "frames/s", "ms_per_step": ms_e2e,
                   "from": "raw uint16 camera frames in pinned host memory: ingest (ADU to e-, clip, "
                           "mirror pad) + finder + peak rows to the host",
                   "h2d_bytes_per_step": int(raw.nbytes), "d2h_bytes_per_step": int(mean_found * 32)},
           "ingest": {"kernel": "k_ingest", "ms_per_launch": ms_ingest, "frames_per_launch": F,
                      "value": F / (ms_ingest / 1e3), "unit": "frames/s",
                      "roofline": {"bound": "hbm", "achieved": ingest_gbs, "peak": hbm_peak, "unit": "GB/s",
                                   "frac": (ingest_gbs / hbm_peak) if hbm_peak else None,
                                   "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)",
                                   "algorithmic_bytes_per_launch": int(ingest_bytes),
                                   "note": "uint16 read once + padded float64 written once; the exact "
                                           "FP64 subtract and multiply per pixel (2 FP64 instructions "
                                           "at GB300's FP64 issue rate) bound it before HBM does"}},
           "roofline": {"bound": "fp32 pipe (double-float taps)",
                        "kernel": "k_conv_fast_ff + k_conv_slow_ff (separable convolution)",
                        "achieved": achieved, "unit": "TFLOP/s (2 per FP64-exact tap)",
                        "fp64_roof": 1.25, "frac_of_fp64_roof": achieved / 1.25,
                        "fp64_roof_source": "nominal FP64 (no measured FP64 peak on this pool): the rate "
                                            "the same taps reach as FP64 FMAs",
                        "flops_per_pixel": 2 * taps,
                        "note": "whole finder step time (all kernels) in the denominator; each tap is ~15 "
                                "FP32-pipe instructions (exact product + two-sum), ncu issue ~80 %"}}
    if not args.no_cpu:
        cores = args.cpu_cores or os.cpu_count() or 1
        per = max(1, min(F, 2 * cores) // cores)
        ctx = multiprocessing.get_context("spawn")
        with ctx.Pool(cores) as pool:
            pool.map(_finder_warm, range(cores), chunksize=1)
            work = [frames[i::cores][:per] for i in range(cores)]
            t0 = time.perf_counter()
            done = sum(pool.map(_finder_worker, work, chunksize=1))
            wall = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": done / wall, "unit": "frames/s", "cores": cores, "kind": "port",
                               "sample": "%d frames, one process per core: numpy FFT matched filters (the "
                               "reference uses FFTW) + the local-maxima loop, %.1f s" % (done, wall)}
    bf.cleanUp()
    return out


def _finder_warm(_):
    from oracle import finder  # noqa: F401
    return 0


def _finder_worker(frames):
    """The oracle's finder (background, foreground, maxima) on some frames."""
    from oracle import finder as ofinder
    of = ofinder.PeakFinderGaussian(FINDER_PARAMS)
    for im in frames:
        of.newImage(im)
        z = numpy.zeros(im.shape)
        of.estimateBackground(z)
        of.findPeaks(z)
    return len(frames)


def _cull_warm(_):
    from oracle import finder  # noqa: F401
    import scipy.spatial  # noqa: F401
    return 0


def _cull_worker(args):
    """The reference's two culling loops on some frames (CPU baseline)."""
    from oracle import finder as ofinder
    frames, sigma, nbhd, thr = args
    n = 0
    for fx, fy, fh, fs, fst in frames:
        s = fst.copy()
        ofinder.mark_dimmer_peaks_kd(fx, fy, fh, s, sigma, nbhd)
        ofinder.mark_low_significance_peaks_kd(fx, fy, fs, s, thr, nbhd)
        n += fx.size
    return n


def run_culling(args, fit):
    """The post-fit culling of the find / fit loop (markDimmerPeaks and
    markLowSignificancePeaks with the reference's radii: sigma 1.5,
    neighbourhood 5 sigma, significance threshold 6) on every frame's fitted
    peaks, called per frame through the reference-shaped API (host arrays),
    as PeakFitter.fitPeaks calls it."""
    from sa_gb300 import ia_utilities_c as U
    counts = fit.counts()
    x, y, h, st = fit.prop("x"), fit.prop("y"), fit.prop("height"), fit.prop("status")
    sig = fit.prop("fg_sum") / numpy.sqrt(fit.prop("bg_sum"))
    edges = numpy.concatenate([[0], numpy.cumsum(counts)])
    frames = [tuple(numpy.ascontiguousarray(a[edges[f]:edges[f + 1]]) for a in (x, y, h, sig, st))
              for f in range(len(counts))]
    sigma, nbhd, thr = 1.5, 7.5, 6.0

    def one(fr, mod):
        fx, fy, fh, fs, fst = fr
        s = fst.copy()
        a = mod.markDimmerPeaks(fx, fy, fh, s, sigma, nbhd)
        b = mod.markLowSignificancePeaks(fx, fy, fs, s, thr, nbhd)
        return a + b

    for fr in frames[:2]:
        one(fr, U)
    t0 = time.perf_counter()
    removed = sum(one(fr, U) for fr in frames)
    wall = time.perf_counter() - t0
    n = int(counts.sum())
    out = {"metric": "peaks/s (markDimmerPeaks + markLowSignificancePeaks per frame)", "value": n / wall,
           "unit": "peaks/s", "ms_per_step": wall * 1e3, "frames": len(frames), "peaks": n,
           "removed": int(removed), "api": "host arrays per frame (reference call shape)"}
    if not args.no_cpu:
        cores = min(args.cpu_cores or os.cpu_count() or 1, len(frames))
        ctx = multiprocessing.get_context("spawn")
        with ctx.Pool(cores) as pool:
            pool.map(_cull_warm, range(cores), chunksize=1)
            chunks = [frames[i::cores] for i in range(cores)]
            t0 = time.perf_counter()
            nk = sum(pool.map(_cull_worker, [(c, sigma, nbhd, thr) for c in chunks], chunksize=1))
            w = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": nk / w, "unit": "peaks/s", "cores": cores, "kind": "port",
                               "sample": "all %d frames, one process per core, kd-tree neighbour queries (scipy "
                                         "cKDTree, as the reference's C builds one per call), %.3f s" % (len(frames), w)}
    return out


def run_analysis(args, wl):
    """The whole 3D-DAOSTORM frame analysis (PeakFinderFitter.analyzeImage:
    finder passes with the threshold count-down, fits, culling, removal of
    unconverged peaks) through sa_gb300.find_peaks on two of the step's
    512 x 512 frames, one frame at a time as the reference analyses a
    movie; the CPU baseline runs the oracle's loop on the first frame."""
    from sa_gb300 import find_peaks
    params = dict(FINDER_PARAMS, model="3d")
    n = 2
    ff = find_peaks.initFindAndFit(params, precision=args.precision)
    ff.analyzeFrame(wl["images"][0])    # warm-up: filters, handles, first launches
    t0 = time.perf_counter()
    found = [ff.analyzeFrame(wl["images"][i])["x"].size for i in range(n)]
    wall = time.perf_counter() - t0
    ff.cleanUp()
    out = {"metric": "frames/s (find / fit loop per frame, host-driven as the reference)",
           "value": n / wall, "unit": "frames/s", "frames": n, "localizations": int(sum(found)),
           "localizations_per_s": sum(found) / wall}
    if not args.no_cpu:
        from oracle import analysis
        t0 = time.perf_counter()
        ref = analysis.analyze_frame(params, wl["images"][0], [0.75, 7.5])
        w = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": 1.0 / w, "unit": "frames/s", "cores": 1, "kind": "port",
                               "sample": "1 frame through the oracle's loop (FP64 C fitter, numpy finder "
                                         "and culling), %.1f s" % w}
        out["oracle_localizations_frame0"] = int(ref["x"].size)
        out["gpu_localizations_frame0"] = int(found[0])
    return out


def _loop_worker(frame):
    """One frame through the oracle's find / fit loop (CPU baseline)."""
    from oracle import analysis
    t0 = time.perf_counter()
    r = analysis.analyze_frame(dict(FINDER_PARAMS, model="3d"), frame, [0.75, 7.5])
    return int(r["x"].size), time.perf_counter() - t0


def _loop_warm(_):
    """Import the oracle's loop in a pool worker (outside the timed region)."""
    from oracle import analysis  # noqa: F401
    return 0


def loop_cpu_sample(frames, cores):
    """The oracle's loop on min(cores, frames) frames, one process per core
    (spawned: this process already holds a CUDA context).  The pool is
    started and every worker has imported the oracle before the timed
    region, which is the map of the frames alone."""
    n = min(cores, len(frames))
    ctx = multiprocessing.get_context("spawn")
    with ctx.Pool(n) as pool:
        pool.map(_loop_warm, range(n), chunksize=1)
        work = [numpy.ascontiguousarray(frames[i]) for i in range(n)]
        t0 = time.perf_counter()
        res = pool.map(_loop_worker, work, chunksize=1)
        wall = time.perf_counter() - t0
    return n, sum(r[0] for r in res), wall


def run_analysis_batch(args, wl):
    """The same find / fit loop for all of the step's frames at once
    (sa_gb300.find_peaks.BatchFindFit): finder and fits stay on the GPU
    across passes, all frames' fits run in one batched sweep loop."""
    from sa_gb300 import find_peaks
    params = dict(FINDER_PARAMS, model="3d")
    frames = numpy.stack(wl["images"])
    bf = find_peaks.BatchFindFit(params, frames.shape[1:], frames.shape[0], precision=args.precision)
    # no warm-up pass: the kernels and filters are already loaded by the
    # blocks before, and one pass of this loop takes seconds
    t0 = time.perf_counter()
    res = bf.analyze(frames)
    wall = time.perf_counter() - t0
    passes = bf.passes
    bf.cleanUp()
    n = sum(r["x"].size for r in res)
    out = {"metric": "frames/s (find / fit loop, all frames batched)", "value": frames.shape[0] / wall,
            "unit": "frames/s", "frames": int(frames.shape[0]), "localizations": int(n),
            "localizations_per_s": n / wall, "passes": passes, "wall_s": wall,
            "note": "each doFit runs up to 2000 sweeps as the reference's does; a few oscillating "
                    "peaks keep every fit to that limit, and a sweep of a handful of peaks costs "
                    "~0.24 ms (the latency of one LM step), so the fits' tails set this number"}
    if not args.no_cpu:
        cores = args.cpu_cores or os.cpu_count()
        nf, nloc, w = loop_cpu_sample(frames, cores)
        out["cpu_baseline"] = {"value": nf / w, "unit": "frames/s", "cores": nf, "kind": "port",
                               "sample": "%d frames through the oracle's loop, one process per core, %.1f s "
                                         "wall (%d localizations)" % (nf, w, nloc)}
    return out


def run_reference(args, rank, world):
    """The reference's CPU fitter (the oracle port of it) on all host cores."""
    if rank != 0:
        return
    from sa_gb300 import synth
    build_oracle()
    cfg = args.config
    wl = synth.make_workload(cfg, frames=args.frames, seed=cfg)
    cores = args.cpu_cores or os.cpu_count()
    ctx = multiprocessing.get_context("spawn")
    sample = min(cores, len(wl["images"]))
    with ctx.Pool(cores) as pool:
        for _ in range(args.warmup if args.warmup < 2 else 1):
            cpu_sample(wl, sample, cores, pool, lib="liboracle_timing.so")
        vals = []
        t_all = 0.0
        n_all = 0
        for _ in range(args.steps):
            n, wall, _ = cpu_sample(wl, sample, cores, pool, lib="liboracle_timing.so")
            vals.append(n / wall)
            t_all += wall
            n_all += n
    value = n_all / t_all
    kw = wl["fitter"]
    line = {"impl": "reference", "metric": "localizations/s (LM to convergence)", "value": value,
            "unit": "localizations/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * t_all / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp64", "data": "synthetic (seeded, benchmark configuration %d shapes)" % cfg,
            "config": {"workload": "cfg%d: %s model, frames %dx%d, roi %s, max %d sweeps; each step a %d-frame "
                                   "sample" % (cfg, kw["model"], wl["nx"], wl["ny"],
                                               kw.get("roi_size", wl["roi"]), MAX_IT, sample)},
            "cpu_baseline": {"value": value, "unit": "localizations/s", "cores": cores, "kind": "port",
                             "sample": "%d frames per step, one process per core" % sample},
            "e2e": {"value": value, "unit": "localizations/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


CONFIG_SAMPLES = {0: 1, 2: 16, 3: 8}   # frames per configuration in the per-configuration report


def run_config_reports(args, pool, cores):
    """Benchmark configurations 0, 2 and 3 (2d; Z with sCMOS; 3D spline) on
    a sample of frames each: the batched engine's localizations/s on the
    sample, and the errors of x, y, z, height, widths and background against
    the FP64 oracle's fits of the same (float32-rounded) frames."""
    import torch
    from sa_gb300 import cubic_fit_c, engine, parity, synth
    out = {}
    for cfg, nf in CONFIG_SAMPLES.items():
        wl = synth.make_workload(cfg, frames=nf)
        kw = dict(wl["fitter"])
        model = kw.pop("model")
        spl = kw.pop("spline", None)
        if spl is not None:
            kw["spline"] = cubic_fit_c.SplinePSF(coeff=spl["coeff"])
        F = len(wl["images"])
        shape = (wl["ny"], wl["nx"])
        images = numpy.ascontiguousarray(numpy.stack(wl["images"]).astype(numpy.float32))
        bgs = numpy.ascontiguousarray(numpy.stack(wl["backgrounds"]).astype(numpy.float32))
        fit = engine.BatchFitter(model, shape, F, rqe=wl["rqe"], scmos_cal=wl["scmos_cal"],
                                 precision=args.precision, **kw)
        fit.load(images, bgs, wl["guesses"], "hdf5")
        fit.fit(MAX_IT)   # warm-up
        ms = []
        for _ in range(2):
            fit.load(images, bgs, wl["guesses"], "hdf5")
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fit.fit(MAX_IT)
            e1.record()
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        got = fit.results(props=("x", "y", "z", "height", "background", "xsigma", "ysigma"))
        units = int(fit.counts().sum())
        fit.close()
        _, _, ora = cpu_sample(wl, F, cores, pool)
        ref = {k: numpy.concatenate([ora[f][k] for f in range(F)]) for k in ora[0]}
        st = parity.compare(got, ref)
        conv = (got["status"] == ref["status"]) & (ref["status"] == 1)
        rec = {"workload": "cfg%d: %s model, %d frames %dx%d, %d emitters" % (cfg, model, F, shape[1], shape[0], units),
               "localizations_per_s": units / (min(ms) / 1e3), "ms_per_fit": min(ms),
               "peaks": st["n"], "status_agree": st["status_agree"],
               "frac_within": min([st[k] for k in st if k.startswith("frac_ok")] or [1.0]),
               "max_dx": st.get("max_dx"), "max_dy": st.get("max_dy"), "max_dz": st.get("max_dz"),
               "max_rel_height": st.get("max_rel_h"), "max_rel_background": st.get("max_rel_bg")}
        if not model.startswith("spline") and conv.any():
            for w in ("xsigma", "ysigma"):
                rec["max_rel_" + w] = float(numpy.max(numpy.abs(got[w][conv] - ref[w][conv]) / numpy.abs(ref[w][conv])))
        out["cfg%d" % cfg] = rec
    out["fft"] = run_fft_report(args, pool, cores)
    out["pupil"] = run_fft_report(args, pool, cores, model="pupil")
    out["multi_plane"] = run_mp_report(args, pool)
    return out


FFT_FRAMES = 4        # frames of the oracle's CPU sample (and of the parity check)
FFT_GPU_FRAMES = 16   # frames of the GPU fit


def run_fft_report(args, pool, cores, model="fft"):
    """An arbitrary-PSF model in the FP64 engine -- the FFT PSF (psf_fft /
    fft_fit) or the pupil function (pupilfn / pupil_fit) -- on synthetic
    frames drawn with the model itself: localizations/s of the batched
    engine and the errors against the oracle's fits of the same frames."""
    import torch
    from sa_gb300 import engine, parity, psf_fft_c, pupil_fn, synth
    wl = (synth.fft_workload(frames=FFT_GPU_FRAMES) if model == "fft"
          else synth.pupil_workload(frames=FFT_GPU_FRAMES))
    F = len(wl["images"])
    shape = (wl["ny"], wl["nx"])
    images = numpy.ascontiguousarray(numpy.stack(wl["images"]).astype(numpy.float32))
    bgs = numpy.ascontiguousarray(numpy.stack(wl["backgrounds"]).astype(numpy.float32))
    if model == "fft":
        obj = psf_fft_c.PSFFFT(wl["fitter"]["psf"])
        fit = engine.BatchFitter("fft", shape, F, psf_fft=obj, precision=64)
    else:
        obj = pupil_fn.PupilFunction(pf_data=wl["fitter"]["pf_data"], zmin=wl["fitter"]["zmin"],
                                     zmax=wl["fitter"]["zmax"])
        fit = engine.BatchFitter("pupil", shape, F, pupil_fn=obj, precision=64)
    fit.load(images, bgs, wl["guesses"], "hdf5")
    fit.fit(MAX_IT)   # warm-up
    ms = []
    for _ in range(2):
        fit.load(images, bgs, wl["guesses"], "hdf5")
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fit.fit(MAX_IT)
        e1.record()
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    got = fit.results(props=("x", "y", "z", "height", "background"))
    counts = fit.counts()
    units = int(counts.sum())
    fit.close()
    obj.cleanup()
    # the oracle fits the first FFT_FRAMES frames (a bounded CPU sample);
    # parity on those
    n_cpu, wall_cpu, ora = cpu_sample(wl, FFT_FRAMES, cores, pool)
    ref = {k: numpy.concatenate([ora[f][k] for f in range(FFT_FRAMES)]) for k in ora[0]}
    n_s = int(counts[:FFT_FRAMES].sum())
    st = parity.compare({k: v[:n_s] for k, v in got.items()}, ref)
    if model == "fft":
        psf = wl["fitter"]["psf"]
        what = "FFT PSF model (%dx%dx%d stack)" % psf.shape
    else:
        what = "pupil-function model (%d px pupil)" % wl["fitter"]["pf_data"]["pf"].shape[0]
    return {"workload": "%s, %d frames %dx%d, %d emitters, FP64 engine" % (what, F, shape[1], shape[0], units),
            "localizations_per_s": units / (min(ms) / 1e3), "ms_per_fit": min(ms),
            "cpu_localizations_per_s": n_cpu / wall_cpu if wall_cpu > 0 else None, "cpu_cores": cores,
            "cpu_kind": "port (the oracle: direct separable DFTs; the reference's C transforms with FFTW, "
                        "which is not installed, so it cannot be built or timed here)",
            "peaks": st["n"], "status_agree": st["status_agree"],
            "frac_within": min([st[k] for k in st if k.startswith("frac_ok")] or [1.0]),
            "max_dx": st.get("max_dx"), "max_dy": st.get("max_dy"), "max_dz": st.get("max_dz"),
            "max_rel_height": st.get("max_rel_h"), "max_rel_background": st.get("max_rel_bg")}


def _mp_cpu_job(args):
    """The oracle's multi-plane fit of one frame (spawned worker): returns
    (seconds, per-plane properties)."""
    import oracle.oracle as O
    wl, lib = args
    O.LIB = os.path.join(ROOT, "oracle", lib)
    shape = (wl["ny"], wl["nx"])
    nc = wl["n_channels"]
    chans = [O.OracleFitter("2d", shape, roi_size=10, sigma_range=(1.0, 3.0), tol=1.0e-6 * nc) for _ in range(nc)]
    f = O.OracleMPFitter(chans, list(wl["maps"]), kind="dao", independent_heights=1)
    t0 = time.perf_counter()
    f.newImage(wl["images"])
    f.newBackground(wl["backgrounds"])
    f.newPeaks(wl["peaks"], "finder")
    f.doFit(MAX_IT)
    props = [{k: f.getPeakProperty(k, c) for k in ("x", "y", "height", "background", "status")} for c in range(nc)]
    dt = time.perf_counter() - t0
    f.cleanup()
    return dt, props


MP_FRAMES = 512       # frames of the batched multi-plane fit
MP_CPU_FRAMES = 32    # frames of its CPU sample


def run_mp_report(args, pool):
    """Multi-plane fitting (multi_plane/mp_fit.c + mp_fit_dao.c, 2D
    Gaussians) of one two-plane 256 x 256 frame with 200 emitters through
    the reference's Python surface (MPFitDao2D: one coupled sweep per
    iterate()): wall time and localizations/s against the oracle's fit of
    the same frame on one host core, and the per-plane agreement."""
    from sa_gb300 import mp_fit_dao_c, synth
    wl = synth.multiplane_workload()
    nc = wl["n_channels"]
    shape = (wl["ny"], wl["nx"])
    # the fitter is made once (as the reference's analysis makes it once per
    # movie); a frame is newImage .. doFit .. getPeakProperty
    walls = []
    f = mp_fit_dao_c.MPFitDao2D(n_channels=nc, roi_size=10, sigma_range=(1.0, 3.0))
    for c in range(nc):
        f.initializeChannel(numpy.ones(shape), numpy.zeros(shape), c)
    f.setMapping(*wl["maps"])
    f.setWeights(verbose=False)
    for rep in range(3):
        t0 = time.perf_counter()
        f.newImage(wl["images"])
        f.newBackground(wl["backgrounds"])
        f.newPeaks(wl["peaks"], "finder")
        f.doFit(MAX_IT)
        got = [{k: f.getPeakProperty(k, c) for k in ("x", "y", "height", "background", "status")} for c in range(nc)]
        walls.append(time.perf_counter() - t0)
    f.cleanup(verbose=False)
    cpu_s, ref = pool.map(_mp_cpu_job, [(wl, "liboracle_timing.so")])[0]
    # batched: MP_FRAMES frames at once (one warp each) against the oracle's
    # frames on the host cores (one frame per process)
    # 64 distinct frames, repeated to MP_FRAMES (the content of a frame does
    # not depend on its neighbours in the batch)
    distinct = [synth.multiplane_workload(seed=100 + i) for i in range(64)]
    wls = [distinct[i % 64] for i in range(MP_FRAMES)]
    f = mp_fit_dao_c.MPFitDao2D(n_channels=nc, roi_size=10, sigma_range=(1.0, 3.0))
    for c in range(nc):
        f.initializeChannel(numpy.ones(shape), numpy.zeros(shape), c)
    f.setMapping(*wl["maps"])
    f.setWeights(verbose=False)
    images = [numpy.stack([w["images"][c] for w in wls]) for c in range(nc)]
    bgs = [numpy.stack([w["backgrounds"][c] for w in wls]) for c in range(nc)]
    f.fitBatch(images, bgs, [w["peaks"] for w in wls], "finder", max_iterations=MAX_IT)   # warm-up
    batch_s = None
    for _ in range(2):
        t0 = time.perf_counter()
        bout, _ = f.fitBatch(images, bgs, [w["peaks"] for w in wls], "finder", max_iterations=MAX_IT)
        w_s = time.perf_counter() - t0
        batch_s = w_s if batch_s is None else min(batch_s, w_s)
    f.cleanup(verbose=False)
    n_batch = int(bout[0]["status"].size)
    ncpu = min(MP_CPU_FRAMES, len(wls))
    t0 = time.perf_counter()
    cpu_res = pool.map(_mp_cpu_job, [(w, "liboracle_timing.so") for w in wls[:ncpu]], chunksize=1)
    cpu_batch_s = time.perf_counter() - t0
    n_cpu_batch = sum(int(r[1][0]["status"].size) for r in cpu_res)
    n = int(got[0]["status"].size)
    agree = min(float((got[c]["status"] == ref[c]["status"]).mean()) for c in range(nc))
    ok = [(got[c]["status"] == 1) & (ref[c]["status"] == 1) for c in range(nc)]
    max_dxy = max(float(numpy.abs(got[c][k][ok[c]] - ref[c][k][ok[c]]).max(initial=0.0)) for c in range(nc)
                  for k in ("x", "y"))
    return {"workload": "multi-plane 2D Gaussians (MPFitDao2D), %d planes of %dx%d, %d emitters, FP64 engine, "
                        "one frame through the reference's Python surface" % (nc, shape[1], shape[0], n),
            "localizations_per_s": n / min(walls), "wall_s": min(walls),
            "cpu_localizations_per_s": n / cpu_s, "cpu_wall_s": cpu_s, "cpu_cores": 1,
            "cpu_kind": "port (the oracle's multi-plane restatement, reference compiler flags)",
            "status_agree": agree, "max_dxy_converged": max_dxy,
            "batch_frames": MP_FRAMES, "batch_localizations_per_s": n_batch / batch_s, "batch_wall_s": batch_s,
            "batch_cpu_localizations_per_s": n_cpu_batch / cpu_batch_s, "batch_cpu_frames": ncpu,
            "batch_cpu_cores": getattr(pool, "_processes", None),
            "batch_timing": "best of 2 fits after a warm-up fit, host images to results",
            "note": "a frame is one CTA: batches of consecutive groups whose grown ROIs do not overlap "
                    "step at once (up to 8 for a lone frame, 2-3 when many frames share the GPU), committed "
                    "in index order (the reference's sweep order); frames run in parallel (mpDoFitBatch); "
                    "FP64 throughout"}


DENSITY_BINS = 6   # log-spaced density bins of the serving stream's frame cache


def _serving_frame_job(args):
    """One distinct frame of the serving stream (spawned worker)."""
    from sa_gb300 import synth
    model, size, dens, seed = args
    wl = synth.serving_frame(model, size, dens, seed)
    return {"image": wl["images"][0], "background": wl["backgrounds"][0], "peaks": wl["guesses"][0],
            "fitter": wl["fitter"], "rqe": wl["rqe"], "scmos_cal": wl["scmos_cal"]}


def serving_requests(n_requests, rate, sizes, pool, seed=4):
    """The serving stream (benchmark configuration 4): Poisson arrivals at
    `rate` frames/s, frame size uniform over `sizes`, density log-uniform
    0.05-2 /um^2, model uniform over 2d/3d/Z/spline3D.  Frame content is
    synthesised once per (model, size, density bin) -- DENSITY_BINS bins on
    the log scale, each at its bin's centre -- on the host cores, so that the
    stream's large frames cost seconds, not minutes, to make."""
    from sa_gb300 import synth
    st = synth.serving_requests(n_requests, rate_hz=rate, seed=seed, sizes=sizes)
    lo, hi = math.log(0.05), math.log(2.0)
    bins = numpy.clip(((numpy.log(st["density"]) - lo) / (hi - lo) * DENSITY_BINS).astype(int), 0,
                      DENSITY_BINS - 1)
    keys = sorted({(str(st["model"][i]), int(st["size"][i]), int(bins[i])) for i in range(n_requests)})
    jobs = [(m, sz, math.exp(lo + (b + 0.5) * (hi - lo) / DENSITY_BINS), 5000 + 37 * b + sz) for m, sz, b in keys]
    frames = dict(zip(keys, pool.map(_serving_frame_job, jobs, chunksize=1)))
    reqs = []
    for i in range(n_requests):
        key = (str(st["model"][i]), int(st["size"][i]), int(bins[i]))
        fr = frames[key]
        reqs.append(dict(fr, model=key[0], ptype="hdf5", camera=(key[0], key[1]), max_iterations=MAX_IT))
    return st["t"], reqs


def run_serving_block(args, local_rank):
    """Serving: a bounded configuration-4 stream through FitServer, and the
    single-frame latency of a 512 x 512 frame at 0.5 emitters / um^2."""
    import torch
    from sa_gb300 import synth
    from sa_gb300.serving import FitServer
    sizes = tuple(int(s) for s in args.serving_sizes.split(","))
    ctx = multiprocessing.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(min(os.cpu_count() or 4, 16)) as pool:
        arrivals, reqs = serving_requests(args.requests, args.rate, sizes, pool)
    synth_s = time.perf_counter() - t0
    server = FitServer(mem_cap_bytes=40e9, slots=args.slots, precision=args.precision,
                       ticks_per_launch=args.ticks_per_launch, ctas_per_slot=args.ctas_per_slot)
    # warm-up: one request of every lane, fitted before the stream
    seen, warm = set(), []
    for r in reqs:
        k = (r["model"], r["image"].shape)
        if k not in seen:
            seen.add(k)
            warm.append(r)
    server.run(warm)
    torch.cuda.synchronize()
    clocks = ClockSampler(local_rank)
    clocks.start()
    t0 = time.perf_counter()
    ids = server.run(reqs, arrivals - arrivals[0])
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    lat = server.latencies(ids) * 1e3
    locs = sum(len(server.done[i]["x"]) for i in ids)
    by_size = {}
    for sz in sizes:
        sel = [j for j, r in enumerate(reqs) if r["image"].shape[0] == sz]
        if sel:
            by_size[str(sz)] = {"requests": len(sel), "p50_ms": float(numpy.percentile(lat[sel], 50)),
                                "p99_ms": float(numpy.percentile(lat[sel], 99))}
    lanes = len(server.lanes)
    server.close()
    # a 512 x 512 frame at 0.5 /um^2 (3d model) fitted alone, request after request
    probe = FitServer(mem_cap_bytes=40e9, slots=1, precision=args.precision,
                      ticks_per_launch=args.ticks_per_launch, ctas_per_slot=1000)
    plat = []
    for k in range(args.latency_frames + 1):
        wl = synth.serving_frame("3d", 512, 0.5, seed=900 + k)
        req = {"model": "3d", "image": wl["images"][0], "background": wl["backgrounds"][0],
               "peaks": wl["guesses"][0], "ptype": "hdf5", "fitter": wl["fitter"], "rqe": wl["rqe"],
               "scmos_cal": wl["scmos_cal"], "camera": ("3d", 512), "max_iterations": MAX_IT}
        torch.cuda.synchronize()
        rid = probe.run([req])[0]
        if k > 0:   # the first one loads the lane
            plat.append(float(probe.latencies([rid])[0] * 1e3))
    probe.close()
    plat = numpy.array(plat)
    return {"metric": "localizations/s (serving stream, continuous batching)", "value": locs / wall,
            "unit": "localizations/s", "requests": len(reqs), "localizations": int(locs), "wall_s": wall,
            "stream": "cfg4: Poisson arrivals at %.0f frames/s, sizes %s, density log-U(0.05, 2) /um^2, models "
                      "2d/3d/Z/spline3D, device-memory admission cap 40 GB, %d slots per lane, %d lanes"
                      % (args.rate, "/".join(str(s) for s in sizes), args.slots, lanes),
            "latency_ms": {"p50": float(numpy.percentile(lat, 50)), "p99": float(numpy.percentile(lat, 99)),
                           "max": float(lat.max()), "by_size": by_size},
            "single_frame_512_0.5": {"frames": int(plat.size), "p50_ms": float(numpy.percentile(plat, 50)),
                                     "p99_ms": float(numpy.percentile(plat, 99)), "target_p99_ms": 5.0,
                                     "note": "one 512 x 512 frame at 0.5 emitters / um^2 (3d model, ~3,360 "
                                             "emitters) submitted alone to an idle server, fitted to termination"},
            "frame_synthesis_s": synth_s, "clocks": clk}


def run_serving(args, local_rank):
    """Serving stream (benchmark configuration 4, reduced): requests of frame
    size 128/256/512, density log-uniform 0.05-2 /um^2 and model 2d/3d/Z/
    spline3D arriving Poisson at args.rate frames/s, fitted by the
    continuous-batching FitServer.  Prints one JSON line with the stream's
    localizations/s and the p50 / p99 request latency (arrival to result)."""
    import torch
    from sa_gb300 import loadclib, synth
    from sa_gb300.serving import FitServer
    loadclib.load().saSetDevice(local_rank)
    torch.cuda.set_device(local_rank)
    sizes = tuple(int(s) for s in args.serving_sizes.split(","))
    st = synth.serving_requests(args.requests + args.warmup, rate_hz=args.rate, seed=4, sizes=sizes)
    reqs = []
    for i in range(len(st["t"])):
        model, size, dens = str(st["model"][i]), int(st["size"][i]), float(st["density"][i])
        wl = synth.serving_frame(model, size, dens, seed=1000 + i)
        reqs.append({"model": model, "image": wl["images"][0], "background": wl["backgrounds"][0],
                     "peaks": wl["guesses"][0], "ptype": "hdf5", "fitter": wl["fitter"], "rqe": wl["rqe"],
                     "scmos_cal": wl["scmos_cal"], "camera": (model, size), "max_iterations": MAX_IT})
    server = FitServer(mem_cap_bytes=40e9, slots=args.slots, precision=args.precision,
                       ticks_per_launch=args.ticks_per_launch, ctas_per_slot=args.ctas_per_slot)
    warm = reqs[:args.warmup]
    if warm:
        server.run(warm)
    timed = reqs[args.warmup:]
    arrivals = st["t"][args.warmup:] - st["t"][args.warmup]
    launches0 = sum(l.fitter.kernel_launches() for l in server.lanes.values())
    clocks = ClockSampler(local_rank)
    clocks.start()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ids = server.run(timed, arrivals)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    lat = server.latencies(ids) * 1e3
    locs = sum(len(server.done[i]["x"]) for i in ids)
    big = [j for j, r in enumerate(timed) if r["image"].shape[0] == 512]
    launches = sum(l.fitter.kernel_launches() for l in server.lanes.values()) - launches0
    line = {
        "metric": "localizations/s (serving stream, continuous batching)",
        "value": locs / wall, "unit": "localizations/s", "n_gpus": 1, "steps": 1,
        "warmup": args.warmup, "ms_per_step": wall * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (float-float step decisions)" if args.precision == 32 else "f64",
        "data": "synthetic (seeded, benchmark configuration 4 shapes, sizes %s)" % (sizes,),
        "config": {"workload": "cfg4 serving: %d requests Poisson at %.0f frames/s, models 2d/3d/Z/spline3D, "
                               "density log-U(0.05, 2) /um^2" % (len(timed), args.rate),
                   "slots_per_lane": args.slots, "ticks_per_launch": args.ticks_per_launch,
                   "ctas_per_slot": args.ctas_per_slot, "memory_cap_gb": 40,
                   "lanes": len(server.lanes), "localizations": int(locs)},
        "latency_ms": {"p50": float(numpy.percentile(lat, 50)), "p99": float(numpy.percentile(lat, 99)),
                       "max": float(lat.max()),
                       "p50_512": float(numpy.percentile(lat[big], 50)) if big else None,
                       "p99_512": float(numpy.percentile(lat[big], 99)) if big else None,
                       "p50_by_model": {m: float(numpy.percentile(lat[[j for j, r in enumerate(timed)
                                                                       if r["model"] == m]], 50))
                                        for m in sorted({r["model"] for r in timed})}},
        "e2e": {"value": locs / wall, "unit": "localizations/s", "note": "host frames in, results out"},
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    print(json.dumps(line))
    server.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", type=int, default=32, choices=[32, 64])
    ap.add_argument("--config", type=int, default=1, choices=[0, 1, 2, 3])
    ap.add_argument("--frames", type=int, default=None)
    ap.add_argument("--plain-frames", type=int, default=2)
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-finder", action="store_true", help="skip the peak-finder measurement")
    ap.add_argument("--finder-only", action="store_true", help="measure the peak finder alone")
    ap.add_argument("--loop-only", action="store_true", help="measure the batched find / fit loop alone")
    ap.add_argument("--size", type=int, default=None, help="frame size for --finder-only / --loop-only")
    ap.add_argument("--cpu-cores", type=int, default=None)
    ap.add_argument("--serving", action="store_true", help="run the serving stream instead")
    ap.add_argument("--requests", type=int, default=400)
    ap.add_argument("--no-serving", action="store_true", help="skip the serving block of the default run")
    ap.add_argument("--no-configs", action="store_true", help="skip the per-configuration error report")
    ap.add_argument("--latency-frames", type=int, default=20)
    ap.add_argument("--rate", type=float, default=2000.0)
    ap.add_argument("--slots", type=int, default=32)
    ap.add_argument("--ticks-per-launch", type=int, default=4)
    ap.add_argument("--ctas-per-slot", type=int, default=12)
    ap.add_argument("--serving-sizes", default="128,256,512,2048")
    ap.add_argument("--model-report", default=None, choices=["fft", "pupil", "multi_plane"],
                    help="run one model's report block alone (the FFT PSF, pupil-function or multi-plane fit)")
    ap.add_argument("--report-cores", type=int, default=16, help="host processes of --model-report's CPU sample")
    args = ap.parse_args()
    from sa_gb300.replicas import rank_env
    rank, world, local_rank = rank_env()
    if args.loop_only and args.impl == "ours":
        if rank == 0:
            import torch
            from sa_gb300 import loadclib, synth
            loadclib.load().saSetDevice(local_rank)
            torch.cuda.set_device(local_rank)
            wl = synth.make_workload(args.config, frames=args.frames, seed=args.config, nx=args.size, ny=args.size)
            print(json.dumps(run_analysis_batch(args, wl)), flush=True)
    elif args.finder_only and args.impl == "ours":
        if rank == 0:
            import torch
            from sa_gb300 import loadclib, synth
            loadclib.load().saSetDevice(local_rank)
            torch.cuda.set_device(local_rank)
            wl = synth.make_workload(args.config, frames=args.frames, seed=args.config, nx=args.size, ny=args.size)
            print(json.dumps(run_finder(args, wl, torch)), flush=True)
    elif args.serving and args.impl == "ours":
        if rank == 0:
            run_serving(args, local_rank)
    elif args.model_report and args.impl == "ours":
        if rank == 0:
            import multiprocessing
            import torch
            from sa_gb300 import loadclib
            build_oracle()
            ctx = multiprocessing.get_context("spawn")
            with ctx.Pool(args.report_cores) as pool:
                loadclib.load().saSetDevice(local_rank)
                torch.cuda.set_device(local_rank)
                if args.model_report == "multi_plane":
                    out = run_mp_report(args, pool)
                else:
                    out = run_fft_report(args, pool, args.report_cores, model=args.model_report)
            print(json.dumps({args.model_report: out}), flush=True)
    elif args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
