#!/usr/bin/env python
"""Throughput benchmark: facet-trace pairs/s of the raypath engine.

Workload (``large_scene``): 2000x2000 facets at 5 m (4M, seeded fractal
surface, Hurst 0.8, RMS 5 m), a rough interface 1.5 km deep sampled as
200x200 targets at 50 m, 2000 traces at 50 km altitude with 5 m spacing,
9 MHz / 1 MHz chirp sampled at 4 MHz into 4096 range bins, aperture 3 deg.
All inputs are seeded synthetic data (no public dataset is involved).

A step is one call over a batch of consecutive flyby traces (default 40); the
K timed steps walk along the track.  A call's pair-kernel work items are
traces x target blocks x 4 facet parts, taken by a persistent grid of 304
blocks; at 40 traces (5760 items, 18.95 rounds of the grid) the last round
is nearly full, where 8 traces (1152 items, 3.79 rounds) leave a fifth of
the grid idle in theirs.  ``value`` is pairs/s with the scene and
trace tables already resident on the device (pairs = sum over traces of
N_ill * (1 + 2 N_t), counted exactly by the kernels); ``e2e`` is the same
metric through the public C ABI call ``rp_simulate`` with pinned host trace
tables in and the host radargram out, copies inside the timed region.

``--impl reference`` times the CPU implementation of the path (the FP64
oracle, a restatement of the reference's trace loop) on the host cores, each
step a bounded sample (one trace, a capped number of in-aperture targets).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "facet-trace pairs/s at <=1e-3 rel L2 vs FP64 oracle"
UNIT = "pairs/s"
WORKLOAD = ("large_scene: 2000x2000 facets at 5 m (4M), fractal H=0.8 RMS 5 m; rough interface "
            "1.5 km deep as 200x200 targets at 50 m (eps 3.15); 2000 traces at 50 km, 5 m spacing; "
            "9 MHz/1 MHz, 4 MHz sampling, 4096 bins; aperture 3 deg; seeded synthetic")


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def shard_steps(total_traces, traces_per_step, steps, warmup, rank, world, lo=None, hi=None):
    """Weak scaling: each rank walks its own stretch of the track.

    Batches are taken from the interior [lo, hi) of the track (default: the
    middle half, where the aperture footprint lies wholly inside the scene)
    and wrap around inside it.  Returns the (start, count) batches of this
    rank's warm-up + timed steps."""
    lo = total_traces // 4 if lo is None else lo
    hi = (3 * total_traces) // 4 if hi is None else hi
    span = max(hi - lo - traces_per_step + 1, 1)
    out = []
    per_rank = steps + warmup
    for k in range(per_rank):
        start = lo + ((rank * per_rank + k) * traces_per_step) % span
        out.append((start, traces_per_step))
    return out


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except Exception:
        return {}


def build_scene(device):
    from europaraypaths_gb300 import scenes, simulator, traces
    sc = scenes.large_scene()
    scene = simulator.Scene(sc["params"], sc["facets"], sc["targets"], device=device)
    track = traces.linear_track(scene.params)
    return sc, scene, track


def cpu_baseline(sc, scene, track, max_targets, trace_index):
    """FP64 oracle on one trace of the workload with a capped target count."""
    from oracle import loader
    loader.lib()
    nthreads = os.cpu_count() or 1
    tr = track[trace_index:trace_index + 1]
    t0 = time.perf_counter()
    _, counts = loader.simulate(scene.params, sc["facets"], sc["targets"], tr,
                                nthreads=nthreads, max_targets=max_targets)
    dt = time.perf_counter() - t0
    from europaraypaths_gb300 import opcount
    p = opcount.pairs(counts)
    return {"value": p / dt, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": f"1 trace (index {trace_index}) of the workload, first {max_targets} in-aperture "
                      f"targets: {p} pairs in {dt:.2f} s (FP64 C++ oracle, OpenMP over targets)"}


def accuracy_vs_plain(scene, d_tr, plain_out, plain_counts, stream):
    """The fast form on the traces the plain FP64 form just ran (traces of the
    timed workload, every target), compared at the accuracy bar: relative
    L2, max phase error above -40 dB of each trace's peak, peak-bin match,
    and equal illuminated-facet / in-aperture-target counts."""
    import torch
    from europaraypaths_gb300 import accuracy
    fout = torch.empty((d_tr.shape[0], scene.nr), dtype=torch.complex64, device="cuda")
    fc = np.zeros_like(plain_counts)
    scene.simulate_device(d_tr, fout, form="fast", stream=stream, counts=fc)
    torch.cuda.synchronize()
    res = accuracy.compare(fout.cpu().numpy(), plain_out.cpu().numpy())
    res.update({"reference": "plain FP64 form (complex128) on the same traces, all targets",
                "trace_index": 1000, "counts_match": bool(np.array_equal(fc, plain_counts)),
                "counts": plain_counts.tolist(), "within_bar": accuracy.within_bar(res)})
    return res


def batch_workload(args, device):
    """The uneven-scenes workload: resident scenes and, per step, a few
    interior traces of every scene (the traces of one step are consecutive)."""
    from europaraypaths_gb300 import scenes, simulator, traces
    t0 = time.perf_counter()
    specs = scenes.uneven_batch(n_scenes=args.batch_scenes)
    objs = [simulator.Scene(s["params"], s["facets"], s["targets"], device=device) for s in specs]
    tracks = [traces.linear_track(o.params) for o in objs]
    return specs, objs, tracks, time.perf_counter() - t0


def run_batch(args, objs, tracks, stream):
    """Pairs/s of one rp_simulate_batch call over every scene (the pair stage
    of all scenes in one persistent launch) vs the same traces scene by scene
    (rp_simulate_ws per scene on one stream)."""
    import ctypes
    import torch
    from europaraypaths_gb300 import _abi, opcount, simulator
    K = args.batch_traces
    steps = args.batch_steps + 1                    # first call warms up (and tunes)
    ws = simulator.Workspace(objs[0].device)
    lib = _abi.lib()
    d_tr, d_out = [], []
    for k in range(steps):
        row_t, row_o = [], []
        for o, tr in zip(objs, tracks):
            ns = tr.shape[0]
            lo = ns // 4 + (k * K) % max(ns // 2 - K, 1)
            row_t.append(torch.from_numpy(np.ascontiguousarray(tr[lo:lo + K])).cuda())
            row_o.append(torch.empty((K, o.nr), dtype=torch.complex64, device="cuda"))
        d_tr.append(row_t)
        d_out.append(row_o)
    counts = [[np.zeros((K, 2), np.int64) for _ in objs] for _ in range(steps)]

    def jobs(k):
        arr = (_abi.RpJob * len(objs))()
        for i, o in enumerate(objs):
            arr[i] = _abi.RpJob(o.handle, d_tr[k][i].data_ptr(), K, d_out[k][i].data_ptr(),
                                counts[k][i].ctypes.data)
        return arr

    sp = ctypes.c_void_p(stream.cuda_stream)
    torch.cuda.synchronize()
    _abi.check("rp_simulate_batch", lib.rp_simulate_batch(jobs(0), len(objs), ws.handle, sp))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    launches = 0
    stage = {}
    for k in range(1, steps):
        _abi.check("rp_simulate_batch", lib.rp_simulate_batch(jobs(k), len(objs), ws.handle, sp))
        launches += simulator.last_launch_count()
        for key, v in simulator.last_timing().items():
            stage[key] = stage.get(key, 0.0) + v / (steps - 1)
    torch.cuda.synchronize()
    tb = time.perf_counter() - t0
    pairs = sum(opcount.pairs(np.concatenate(counts[k])) for k in range(1, steps))
    # the same traces, one scene per call
    seq_counts = [[np.zeros((K, 2), np.int64) for _ in objs] for _ in range(steps)]
    t0 = time.perf_counter()
    for k in range(1, steps):
        for i, o in enumerate(objs):
            rc = lib.rp_simulate_ws(ctypes.c_void_p(o.handle), ws.handle, ctypes.c_void_p(d_tr[k][i].data_ptr()),
                                    K, simulator.FORMS["fast"], ctypes.c_void_p(d_out[k][i].data_ptr()),
                                    seq_counts[k][i].ctypes.data, sp)
            _abi.check("rp_simulate_ws", rc)
    torch.cuda.synchronize()
    ts = time.perf_counter() - t0
    ws.close()
    # the first timed step's call recorded as one CUDA graph
    # (rp_graph_create_batch) and replayed on the same device buffers
    g = simulator.capture_batch([(o, d_tr[1][i].cpu().numpy()) for i, o in enumerate(objs)], d_tr[1], d_out[1])
    try:
        ref = [torch.view_as_real(o).clone() for o in d_out[1]]      # the capture's eager batch call
        for o in d_out[1]:
            o.fill_(complex(float("nan"), float("nan")))
        torch.cuda.synchronize()
        g.launch(stream)
        stream.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps - 1):
            g.launch(stream)
        stream.synchronize()
        tg = (time.perf_counter() - t0) / (steps - 1)
        g.check(stream)
        same = all(torch.equal(a.view(torch.int32), torch.view_as_real(b).view(torch.int32))
                   for a, b in zip(ref, d_out[1]))
    finally:
        g.close()
    bands = {}
    for o in objs:
        key = f"{o.params.frequency / 1e6:g} MHz/{o.nr} bins"
        bands[key] = bands.get(key, 0) + 1
    return {"value": pairs / tb, "unit": UNIT, "scenes": len(objs), "traces_per_scene_per_step": K,
            "steps": steps - 1, "ms_per_step": 1e3 * tb / (steps - 1), "pairs_per_step": pairs / (steps - 1),
            "gpu_launches_per_step": launches / (steps - 1), "stage_ms_per_step": stage,
            "one_scene_per_call": {"value": pairs / ts, "ms_per_step": 1e3 * ts / (steps - 1)},
            "batched_over_one_at_a_time": ts / tb,
            "graph": {"replay_ms_per_call": 1e3 * tg, "direct_ms_per_call": 1e3 * tb / (steps - 1),
                      "bitwise_equal": bool(same),
                      "note": "the whole batch call as one CUDA graph (rp_graph_create_batch), host wall clock"},
            "tuned_multi_cfg": simulator.autotune_query(True),
            "mix": bands}


def run_mode(args, sc, track, stream, default_value, specular=False, ttype0=False):
    """Another mode on the same large scene and traces: specular mode with
    linear convolution (the specular pair kernel: both refraction legs with
    their facetReradiation factors, binned as two traces; compression with
    the outbound trace), or every target ttype 0 (genRefrPhasor: one-bin
    phasors, one chirp convolution per trace).  pairs/s over interior traces,
    CUDA events on the launching stream."""
    import torch
    from europaraypaths_gb300 import simulator, opcount
    p = dict(sc["params"])
    p["specular"] = bool(specular)
    tg = np.array(sc["targets"], copy=True)
    if ttype0:
        tg[6, :] = 0.0
    scene = simulator.Scene(p, sc["facets"], tg, device=torch.cuda.current_device())
    try:
        n = args.spec_traces
        steps = args.spec_steps
        d_tr = [torch.from_numpy(np.ascontiguousarray(track[900 + k * n:900 + (k + 1) * n])).cuda()
                for k in range(steps + 1)]
        d_out = torch.empty((n, scene.nr), dtype=torch.complex64, device="cuda")
        c = [np.zeros((n, 2), np.int64) for _ in range(steps + 1)]
        scene.simulate_device(d_tr[0], d_out, form="fast", stream=stream, counts=c[0])   # warm-up, tuning
        torch.cuda.synchronize()
        stage = {"setup_ms": 0.0, "pairs_ms": 0.0, "compress_ms": 0.0, "tail_ms": 0.0}
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for k in range(1, steps + 1):
            scene.simulate_device(d_tr[k], d_out, form="fast", stream=stream, counts=c[k])
            t = simulator.last_timing()
            for key in stage:
                stage[key] += t[key] / steps
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        pairs = float(opcount.pairs(np.concatenate(c[1:]))) / steps
        v = pairs / (ms / 1e3)
        out = {"value": v, "unit": UNIT, "traces_per_step": n, "steps": steps, "ms_per_step": ms,
               "stage_ms_per_step": stage, "over_default_mode": v / default_value if default_value else None,
               "note": ("same scene and traces as the headline with "
                        + ("every target ttype 0" if ttype0 else "specular=true, convolution_linear=true"))}
        if specular:
            out["pair_cfg"] = {f"degree_{d}": simulator.autotune_query(False, d, specular=True)
                               for d in (0, 3, 4, 5, 6) if simulator.autotune_query(False, d, specular=True) >= 0}
        return out
    finally:
        scene.close()


def run_direct(args, sc, track, stream):
    """Specular mode without convolution (reflRadarSignal / refrRadarSignal
    direct sums over sources x bins) on the large scene's facets: the fast
    form over every 64th target (all ttype 0), in source-bin terms/s, and one
    surface-only trace in both forms (the plain form's FP64 direct sum)."""
    import torch
    from europaraypaths_gb300 import simulator
    p = dict(sc["params"])
    p.update(specular=True, convolution=False)
    tg = np.array(sc["targets"], copy=True)[:, ::64]
    tg[6, :] = 0.0
    dev = torch.cuda.current_device()
    out = {"note": "large-scene facets, every 64th target as ttype 0, specular=true, convolution=false"}

    def timed(scene, tr, form):
        d = torch.from_numpy(np.ascontiguousarray(tr)).cuda()
        o = torch.empty((tr.shape[0], scene.nr), dtype=torch.complex64, device="cuda")
        c = np.zeros((tr.shape[0], 2), np.int64)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        scene.simulate_device(d, o, form=form, stream=stream, counts=c)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), c

    scene = simulator.Scene(p, sc["facets"], tg, device=dev)
    try:
        n = 2
        timed(scene, track[900:900 + n], "fast")          # warm-up
        ms, c = timed(scene, track[1000:1000 + n], "fast")
        terms = float(np.sum(c[:, 0].astype(np.float64) * (1 + c[:, 1]))) * scene.nr
        out.update({"value": terms / (ms / 1e3), "unit": "source-bin terms/s", "traces": n, "ms": ms,
                    "mean_counts_per_trace": [float(c[:, 0].mean()), float(c[:, 1].mean())]})
    finally:
        scene.close()
    scene = simulator.Scene(p, sc["facets"], np.zeros((7, 0)), device=dev)
    try:
        tr = track[1000:1001]
        timed(scene, tr, "fast")
        fms, _ = timed(scene, tr, "fast")
        pms, _ = timed(scene, tr, "plain")
        out["surface_only_1_trace"] = {"fast_ms": fms, "plain_ms": pms, "fast_over_plain": pms / fms}
    finally:
        scene.close()
    return out


def run_graph(args, scene, track):
    """One-trace calls, each followed by a sync: a direct
    rp_simulate_device call (host planning from the trace, two host syncs,
    the launches) against the replay of the same call captured as a CUDA
    graph (rp_graph_*).  Wall-clock per call on the host; the replay's
    radargram must equal the direct call's bit for bit.  On the headline
    scene (trace 1000, ~20 ms of device work a call) and on the small plain
    scene (200x200 facets, 1600 targets, 2048 bins: a call short enough
    for the host's share to show)."""
    from europaraypaths_gb300 import scenes, simulator
    out = {"large_scene": _graph_case(args.graph_calls, scene, track[1000:1001])}
    sp = scenes.small_plain()
    with simulator.Scene(sp["params"], sp["facets"], sp["targets"]) as small:
        tr = small.default_traces()
        out["small_scene"] = _graph_case(args.graph_calls * 5, small, tr[50:51])
    return out


def _graph_case(n, scene, trace):
    import torch
    tr = np.ascontiguousarray(trace)
    d_tr = torch.from_numpy(tr).cuda()
    ref = torch.empty((1, scene.nr), dtype=torch.complex64, device="cuda")
    cur = torch.cuda.current_stream()
    for _ in range(3):
        scene.simulate_device(d_tr, ref)
        cur.synchronize()
    t0 = time.perf_counter()
    for _ in range(n):
        scene.simulate_device(d_tr, ref)
        cur.synchronize()
    direct = (time.perf_counter() - t0) / n
    out = torch.empty_like(ref)
    g = scene.capture(tr, d_tr, out)
    try:
        for _ in range(3):
            g.launch()
            cur.synchronize()
        t0 = time.perf_counter()
        for _ in range(n):
            g.launch()
            cur.synchronize()
        replay = (time.perf_counter() - t0) / n
        g.check()
        same = bool(torch.equal(torch.view_as_real(out), torch.view_as_real(ref)))
    finally:
        g.close()
    return {"traces_per_call": 1, "calls": n, "direct_ms_per_call": 1e3 * direct,
            "replay_ms_per_call": 1e3 * replay, "direct_over_replay": direct / replay,
            "bitwise_equal": same, "note": "host wall clock per call, each call followed by a stream sync"}


def run_flyby(args, stream):
    """The flyby-scale scene: 64M facets (8000x8000 at 2.5 m), two rough
    layers (320k targets), 10,000 traces at 25 km, 60 MHz / 10 MHz sampled
    at 24 MHz into 16384 bins.  pairs/s of the fast form over interior
    traces (inputs resident, CUDA events on the launching stream), the stage
    times, and one interior trace against the plain FP64 form (all targets)."""
    import torch
    from europaraypaths_gb300 import accuracy, opcount, scenes, simulator
    dev = torch.cuda.current_device()
    t0 = time.perf_counter()
    sc = scenes.flyby(n_facets_side=args.flyby_facets_side)
    t1 = time.perf_counter()
    scene = simulator.Scene(sc["params"], sc["facets"], sc["targets"], device=dev)
    t2 = time.perf_counter()
    sc["facets"] = None                      # the scene holds its own device stores
    try:
        track = scene.default_traces()
        n, steps = args.flyby_traces, args.flyby_steps
        lo = track.shape[0] // 4
        span = max(track.shape[0] // 2 - n, 1)
        d_tr = [torch.from_numpy(np.ascontiguousarray(track[lo + (97 * k) % span:lo + (97 * k) % span + n])).cuda()
                for k in range(steps + 1)]
        d_out = torch.empty((n, scene.nr), dtype=torch.complex64, device="cuda")
        c = [np.zeros((n, 2), np.int64) for _ in range(steps + 1)]
        scene.simulate_device(d_tr[0], d_out, form="fast", stream=stream, counts=c[0])   # warm-up, tuning
        torch.cuda.synchronize()
        stage = {"setup_ms": 0.0, "pairs_ms": 0.0, "compress_ms": 0.0, "tail_ms": 0.0}
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for k in range(1, steps + 1):
            scene.simulate_device(d_tr[k], d_out, form="fast", stream=stream, counts=c[k])
            t = simulator.last_timing()
            for key in stage:
                stage[key] += t[key] / steps
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        cc = np.concatenate(c[1:])
        pairs = float(opcount.pairs(cc)) / steps
        out = {"value": pairs / (ms / 1e3), "unit": UNIT, "traces_per_step": n, "steps": steps, "ms_per_step": ms,
               "stage_ms_per_step": stage, "mean_counts_per_trace": [float(cc[:, 0].mean()), float(cc[:, 1].mean())],
               "pair_evals_per_s": float(opcount.target_evals(cc)) / steps / (stage["pairs_ms"] / 1e3)
               if stage["pairs_ms"] > 0 else None,
               "scene_generate_s": t1 - t0, "scene_create_s": t2 - t1,
               "workload": (f"flyby: {args.flyby_facets_side}x{args.flyby_facets_side} facets at 2.5 m "
                            f"({args.flyby_facets_side ** 2 / 1e6:g}M), fractal H=0.75 RMS 8 m; rough layers 1 km and "
                            f"3 km deep as targets at 50 m ({sc['targets'].shape[1]}); {track.shape[0]} traces at "
                            "25 km, 2 m spacing; 60 MHz/10 MHz, 24 MHz sampling, 16384 bins; aperture 3 deg; "
                            "seeded synthetic")}
        if args.flyby_plain:
            k = track.shape[0] // 2
            ptr = torch.from_numpy(np.ascontiguousarray(track[k:k + 1])).cuda()
            pout = torch.empty((1, scene.nr), dtype=torch.complex128, device="cuda")
            pc = np.zeros((1, 2), np.int64)
            torch.cuda.synchronize()
            p0 = torch.cuda.Event(enable_timing=True)
            p1 = torch.cuda.Event(enable_timing=True)
            p0.record(stream)
            scene.simulate_device(ptr, pout, form="plain", stream=stream, counts=pc, complex128=True)
            p1.record(stream)
            torch.cuda.synchronize()
            pv = opcount.pairs(pc) / (p0.elapsed_time(p1) / 1e3)
            out["plain_form"] = {"value": pv, "unit": UNIT, "traces": 1, "fast_over_plain": out["value"] / pv}
            acc = accuracy_vs_plain(scene, ptr, pout, pc, stream)
            acc["trace_index"] = k
            out["accuracy"] = acc
        return out
    finally:
        scene.close()


def run_io(n_facets=200_000, n_traces=200, nr=4096):
    """Host file I/O of the binary stores against the reference's text formats
    (seeded synthetic facets; no device work): parse a .fct text file vs map a
    facet store, and write per-trace "%e %e" text files vs one radargram file."""
    import shutil
    import tempfile
    from europaraypaths_gb300 import fileio, simple_surfaces as ss
    rng = np.random.default_rng(7)
    side = int(np.sqrt(n_facets))
    dom = {"fs": 5.0, "nx": side, "ny": side, "ox": 0.0, "oy": 0.0}
    facets = ss.surface_arrays(dom, "flat", heights=rng.normal(0.0, 2.0, (side, side)))
    d = tempfile.mkdtemp()
    try:
        txt, store = os.path.join(d, "f.fct"), os.path.join(d, "f.rpf")
        row = ":".join([",".join(["%.6f"] * 3)] * 4)
        np.savetxt(txt, facets.T, fmt=row)
        fileio.write_store(store, facets, fileio.STORE_FACETS)
        t0 = time.perf_counter()
        a = fileio.read_facets(txt)
        t1 = time.perf_counter()
        with fileio.MappedStore(store, fileio.STORE_FACETS) as m:
            s = float(m.soa[:, ::4096].sum())        # touch the mapping
        t2 = time.perf_counter()
        b = fileio.load_facets(store)
        t3 = time.perf_counter()
        assert a.shape == b.shape and np.isfinite(s)
        rdr = (rng.standard_normal((n_traces, nr)) + 1j * rng.standard_normal((n_traces, nr))).astype(np.complex64)
        tdir = os.path.join(d, "t")
        os.makedirs(tdir)
        t4 = time.perf_counter()
        for k in range(n_traces):
            fileio.write_trace(os.path.join(tdir, f"s{k:06d}.txt"), rdr[k])
        t5 = time.perf_counter()
        fileio.write_radargram(os.path.join(d, "r.rdr"), rdr)
        t6 = time.perf_counter()
    finally:
        shutil.rmtree(d, ignore_errors=True)
    nf = facets.shape[1]
    return {"facets": nf, "text_parse_s": t1 - t0, "store_map_s": t2 - t1, "store_load_copy_s": t3 - t2,
            "parse_over_load": (t1 - t0) / max(t3 - t2, 1e-9), "traces": n_traces, "nr": nr,
            "text_traces_write_s": t5 - t4, "radargram_write_s": t6 - t5,
            "text_over_radargram": (t5 - t4) / max(t6 - t5, 1e-9),
            "note": "host only; facets generated, written as .fct text and as a facet store"}


def run_focus(Nr=4096, Na=2000):
    """Azimuth focusing (focus_rdrgrm) of a radargram the shape of the flyby's
    (4096 bins x 2000 traces at 5 m, 50 km altitude, 3 deg aperture), seeded
    synthetic values, end to end through the C ABI (host radargram in and
    out).  One row also through the NumPy oracle: its rate on the host and the
    parity of that row."""
    import importlib
    from europaraypaths_gb300 import focusing
    rng = np.random.default_rng(9)
    rdr = (rng.standard_normal((Nr, Na)) + 1j * rng.standard_normal((Nr, Na))).astype(np.complex64)
    par = {"rx_window_m": 4096.5 * 299792480 / 4e6 / 4, "rx_window_offset_m": 49000.0, "rx_sample_rate": 4e6,
           "aperture": 3.0, "spacing": 5.0, "altitude": 50000.0, "eps_1": 1.0, "eps_2": 3.15, "frequency": 9e6}
    focusing.focus_rdrgrm(rdr[:64], dict(par))                    # warm-up (context, module load)
    t0 = time.perf_counter()
    out = focusing.focus_rdrgrm(rdr, dict(par))
    t1 = time.perf_counter()
    # algorithmic work: the terms of every pixel's convolution sum
    macs = 0
    for i in range(Nr):
        rr = par["rx_window_m"] * (i / Nr) + par["rx_window_offset_m"]
        h = int(rr * np.sin(np.radians(par["aperture"])) / par["spacing"])
        j = np.arange(Na)
        macs += int((np.minimum(Na, j + h) - np.maximum(0, j - h)).sum())
    line = {"shape": [Nr, Na], "e2e_s": t1 - t0, "pixels_per_s": Nr * Na / (t1 - t0),
            "complex_macs_per_s": macs / (t1 - t0), "complex_macs": macs,
            "note": "host radargram in and out (65 MB each way), geometry and pixels on the device"}
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "oracle"))
    nf = importlib.import_module("np_focus")
    row = Nr // 2
    t2 = time.perf_counter()
    ref = nf.focus_rdrgrm(rdr.astype(np.complex128), dict(par), st=row, en=row + 1)
    t3 = time.perf_counter()
    line["cpu_oracle"] = {"pixels_per_s": 2 * Na / (t3 - t2), "cores": 1, "kind": "port",
                          "sample": f"rows {row}-{row + 1} of the same radargram (NumPy oracle, one FFT per pixel)"}
    a, b = out[row:row + 2].astype(np.complex128), ref[row:row + 2]
    line["row_rel_l2_vs_oracle"] = float(np.linalg.norm(a - b) / np.linalg.norm(b))
    return line


class CompletionClock:
    """Records when each submitted request finishes, so that the latency
    tail can be set against the requests' sizes.  A thread polls the pending
    requests every millisecond (``done()`` is a zero-wait poll); callers read
    the results only after ``finish()``, so no request is polled from two
    threads."""

    def __init__(self):
        self.pending, self.done = [], []
        self.lock = threading.Lock()
        self.stop = False
        self.thread = threading.Thread(target=self._run, daemon=True)
        self.thread.start()

    def add(self, req):
        with self.lock:
            self.pending.append((req, time.perf_counter()))

    def _run(self):
        while not self.stop:
            with self.lock:
                keep = []
                for req, t0 in self.pending:
                    if req.done():
                        self.done.append((req, 1e3 * (time.perf_counter() - t0)))
                    else:
                        keep.append((req, t0))
                self.pending = keep
            time.sleep(0.001)

    def finish(self, timeout):
        t_end = time.perf_counter() + timeout
        while time.perf_counter() < t_end:
            with self.lock:
                if not self.pending:
                    break
            time.sleep(0.01)
        self.stop = True
        self.thread.join()

    def tail(self):
        """Latency against request size over the requests that completed:
        the rank correlation of latency with pairs, and the mean pairs and
        traces of the slowest 1% and 10% of requests against all of them."""
        from europaraypaths_gb300 import opcount
        ok = [(opcount.pairs(r.counts), r.counts.shape[0], lat) for r, lat in self.done if r.status == 0]
        if len(ok) < 10:
            return None
        pairs = np.array([a for a, _, _ in ok], np.float64)
        ntr = np.array([b for _, b, _ in ok], np.float64)
        lat = np.array([c for _, _, c in ok], np.float64)
        rho = float(np.corrcoef(np.argsort(np.argsort(pairs)), np.argsort(np.argsort(lat)))[0, 1])
        order = np.argsort(lat)
        k1, k10 = max(1, len(ok) // 100), max(1, len(ok) // 10)
        return {"requests": len(ok), "spearman_latency_vs_pairs": rho,
                "mean_pairs": float(pairs.mean()), "mean_traces": float(ntr.mean()),
                "slowest_1pct": {"mean_pairs": float(pairs[order[-k1:]].mean()),
                                 "mean_traces": float(ntr[order[-k1:]].mean()),
                                 "mean_ms": float(lat[order[-k1:]].mean())},
                "slowest_10pct": {"mean_pairs": float(pairs[order[-k10:]].mean()),
                                  "mean_traces": float(ntr[order[-k10:]].mean()),
                                  "mean_ms": float(lat[order[-k10:]].mean())},
                "note": "submit-to-completion on the host, 1 ms polling"}


def run_serving(args, objs, tracks, plain_value):
    """The serving loop: Poisson arrivals of flyby requests over the resident
    scenes (a scene drawn uniformly, 1-8 consecutive interior traces), served
    concurrently with footprint admission; latency is submit to result."""
    from europaraypaths_gb300 import serving
    rng = np.random.default_rng(4)
    srv = serving.Server(workers=4, device=objs[0].device)
    sids = [srv.adopt_scene(o) for o in objs]
    n_req = int(args.serve_rate * args.serve_seconds)
    gaps = rng.exponential(1.0 / args.serve_rate, n_req)
    reqs = []
    clock = CompletionClock()
    t_start = time.perf_counter()
    t_next = t_start
    for g in gaps:
        t_next += g
        dt = t_next - time.perf_counter()
        if dt > 0:
            time.sleep(dt)
        i = int(rng.integers(0, len(objs)))
        ns = tracks[i].shape[0]
        n = int(rng.integers(1, 9))
        lo = ns // 4 + int(rng.integers(0, max(ns // 2 - n, 1)))
        r = srv.submit(sids[i], tracks[i][lo:lo + n])
        reqs.append(r)
        clock.add(r)
    clock.finish(600)
    for r in reqs:
        r.result(timeout=600)
    st = srv.stats()
    st["latency_vs_size"] = clock.tail()
    srv.close(keep_scenes=True)
    st.update({"requests": n_req, "rate_req_s": args.serve_rate, "arrival_window_s": args.serve_seconds,
               "workers": 4, "request": "uniform scene of the uneven-scenes workload, 1-8 interior traces",
               "vs_plain_form": (st["pairs_per_s"] / plain_value) if (plain_value and st.get("pairs_per_s"))
               else None})
    return st


def run_serving_flybys(args, objs, tracks, plain_value):
    """The serving loop at the flyby-request load: Poisson arrivals at
    ``serve_rate`` requests/s for ``flyby_serve_seconds``; each request is a
    flyby over one of the resident uneven scenes (drawn uniformly; up to 4M
    facets) of U{50..2000} consecutive traces (capped at the scene's track).
    The server cuts requests into 16-trace steps, keeps at most 16 requests
    active, takes the next step of up to 16 of them per worker call (4
    workers, overlapping on the device) and sheds requests still queued
    after ``flyby_serve_max_wait`` seconds.  Latency is submit to result."""
    from europaraypaths_gb300 import serving
    rng = np.random.default_rng(44)
    srv = serving.Server(workers=4, device=objs[0].device, max_batch=16, step_traces=16, max_active=16,
                         max_wait=args.flyby_serve_max_wait)
    sids = [srv.adopt_scene(o) for o in objs]
    n_req = int(args.serve_rate * args.flyby_serve_seconds)
    gaps = rng.exponential(1.0 / args.serve_rate, n_req)
    reqs, offered_traces = [], 0
    clock = CompletionClock()
    t_start = time.perf_counter()
    t_next = t_start
    for g in gaps:
        t_next += g
        dt = t_next - time.perf_counter()
        if dt > 0:
            time.sleep(dt)
        i = int(rng.integers(0, len(objs)))
        ns = tracks[i].shape[0]
        n = min(int(rng.integers(50, 2001)), ns)
        lo = int(rng.integers(0, ns - n + 1))
        reqs.append((n, srv.submit(sids[i], tracks[i][lo:lo + n])))
        clock.add(reqs[-1][1])
        offered_traces += n
    t_arrivals = time.perf_counter() - t_start
    clock.finish(900)
    served_traces, shed = 0, 0
    for n, r in reqs:
        try:
            r.result(timeout=900)
            served_traces += n
        except serving.ShedError:
            shed += 1
    t_done = time.perf_counter() - t_start
    st = srv.stats()
    st["latency_vs_size"] = clock.tail()
    srv.close(keep_scenes=True)
    st.update({"requests": n_req, "rate_req_s": args.serve_rate, "arrival_window_s": t_arrivals,
               "drained_after_s": t_done, "workers": 4, "step_traces": 16, "max_active": 16,
               "max_wait_s": args.flyby_serve_max_wait,
               "offered_traces": offered_traces, "served_traces": served_traces,
               "request": "flyby over a uniform uneven scene (<= 4M facets), U{50..2000} consecutive traces",
               "served_pairs_per_s_over_plain_form": (st["pairs_per_s"] / plain_value)
               if (plain_value and st.get("pairs_per_s")) else None,
               "note": ("offered load far above one GPU's capacity (requests average ~1000 traces): the "
                        "queue-wait bound sheds what cannot start in time; latency = wait + service time "
                        "shared by up to 16 active requests, the tail being the largest requests")})
    return st


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from europaraypaths_gb300 import scenes, param_gen, traces, opcount
    from oracle import loader
    loader.lib()
    sc = scenes.large_scene()
    p = param_gen.to_rp_params(sc["params"], derive=False)
    loader.derive(p)
    track = traces.linear_track(p)
    nthreads = os.cpu_count() or 1
    times, pairs = [], []
    for k in range(args.warmup + args.steps):
        i0 = p.ns // 4 + (k * 97) % (p.ns // 2)     # interior of the track
        tr = track[i0:i0 + 1]
        t0 = time.perf_counter()
        _, counts = loader.simulate(p, sc["facets"], sc["targets"], tr, nthreads=nthreads,
                                    max_targets=args.ref_targets)
        dt = time.perf_counter() - t0
        if k >= args.warmup:
            times.append(dt)
            pairs.append(opcount.pairs(counts))
    total = float(sum(times))
    value = sum(pairs) / total
    sample = (f"each step: 1 trace of the workload, first {args.ref_targets} in-aperture targets "
              f"(FP64 C++ oracle restating the reference trace loop, {nthreads} threads)")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "sample": sample},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--traces-per-step", type=int, default=40,
                    help="traces per call: 40 x 36 target blocks x 4 facet parts = 5760 pair-kernel items, "
                         "18.95 rounds of the 304-block persistent grid")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--plain-traces", type=int, default=1, help="traces for the plain FP64 form (0 = skip)")
    ap.add_argument("--cpu-targets", type=int, default=48, help="target cap of the CPU baseline sample")
    ap.add_argument("--ref-targets", type=int, default=24, help="target cap per --impl reference step")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batch-scenes", type=int, default=64, help="scenes of the batched workload (0 = skip)")
    ap.add_argument("--batch-traces", type=int, default=8, help="interior traces per scene per batched step")
    ap.add_argument("--batch-steps", type=int, default=3)
    ap.add_argument("--serve-seconds", type=float, default=15.0, help="serving-loop arrivals window (0 = skip)")
    ap.add_argument("--serve-rate", type=float, default=20.0, help="Poisson request rate, requests/s")
    ap.add_argument("--flyby-serve-seconds", type=float, default=15.0,
                    help="arrivals window of the serving loop at flyby-request sizes (0 = skip)")
    ap.add_argument("--flyby-serve-max-wait", type=float, default=5.0,
                    help="queue-wait bound (s) of that serving run; older queued requests are shed")
    ap.add_argument("--no-io", dest="io", action="store_false", help="skip the host file-I/O measurement")
    ap.add_argument("--no-focus", dest="focus", action="store_false", help="skip the azimuth-focusing measurement")
    ap.add_argument("--graph-calls", type=int, default=20,
                    help="one-trace calls timed direct and as graph replays (0 = skip)")
    ap.add_argument("--spec-traces", type=int, default=4,
                    help="traces per step of the specular-mode and ttype-0 runs (0 = skip)")
    ap.add_argument("--spec-steps", type=int, default=3)
    ap.add_argument("--flyby-traces", type=int, default=32,
                    help="traces per step of the flyby-scale scene (0 = skip the flyby entry)")
    ap.add_argument("--flyby-steps", type=int, default=2)
    ap.add_argument("--flyby-facets-side", type=int, default=8000,
                    help="facets per side of the flyby scene at 2.5 m (8000: the 64M-facet scene; "
                         "2000: a 5 km square with the same band, altitude and aperture)")
    ap.add_argument("--no-flyby-plain", dest="flyby_plain", action="store_false",
                    help="skip the flyby trace in the plain FP64 form (accuracy check)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    if args.impl == "reference":
        return run_reference(args)

    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    from europaraypaths_gb300 import simulator, opcount
    sc, scene, track = build_scene(local)
    nr = scene.nr
    tps = args.traces_per_step
    batches = shard_steps(track.shape[0], tps, args.steps, args.warmup, rank, world)
    d_tracks = [torch.from_numpy(np.ascontiguousarray(track[s:s + n])).cuda() for s, n in batches]
    d_out = torch.empty((tps, nr), dtype=torch.complex64, device="cuda")
    stream = torch.cuda.Stream()
    counts = [np.zeros((tps, 2), np.int64) for _ in batches]

    simulator.set_timing(True)
    # warm-up
    for k in range(args.warmup):
        scene.simulate_device(d_tracks[k], d_out, form="fast", stream=stream, counts=counts[k])
    torch.cuda.synchronize()

    sampler = ClockSampler(local)
    sampler.start()
    stage = {"setup_ms": 0.0, "pairs_ms": 0.0, "compress_ms": 0.0, "tail_ms": 0.0, "pair_launches": 0}
    launches = 0
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for k in range(args.warmup, args.warmup + args.steps):
        scene.simulate_device(d_tracks[k], d_out, form="fast", stream=stream, counts=counts[k])
        t = simulator.last_timing()
        for key in stage:
            stage[key] += t[key]
        launches += simulator.last_launch_count()
    ev1.record(stream)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    clocks = sampler.stop()
    elapsed_ms = ev0.elapsed_time(ev1)
    timed_counts = np.concatenate(counts[args.warmup:])
    my_pairs = opcount.pairs(timed_counts)
    my_evals = opcount.target_evals(timed_counts)
    if dist is not None:
        t = torch.tensor([elapsed_ms], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed_ms = float(t.item())
        pt = torch.tensor([float(my_pairs)], dtype=torch.float64, device="cuda")
        dist.all_reduce(pt, op=dist.ReduceOp.SUM)
        total_pairs = float(pt.item())
    else:
        total_pairs = float(my_pairs)
    value = total_pairs / (elapsed_ms / 1e3)

    # ---- end to end through rp_simulate (pinned host buffers) ----
    h_tr = torch.empty((tps, 9), dtype=torch.float64).pin_memory()
    h_out = torch.empty((tps, nr), dtype=torch.complex64).pin_memory()
    e2e_pairs = 0
    t0 = time.perf_counter()
    for k in range(args.e2e_steps):
        s, n = batches[(args.warmup + k) % len(batches)]
        h_tr.copy_(torch.from_numpy(track[s:s + n]))
        c = np.zeros((tps, 2), np.int64)
        scene.simulate_host_ptrs(h_tr.data_ptr(), n, h_out.data_ptr(), form="fast", stream=stream, counts=c)
        e2e_pairs += opcount.pairs(c)
    e2e_s = time.perf_counter() - t0
    if dist is not None:
        t = torch.tensor([e2e_s], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
        pt = torch.tensor([float(e2e_pairs)], dtype=torch.float64, device="cuda")
        dist.all_reduce(pt, op=dist.ReduceOp.SUM)
        e2e_pairs = float(pt.item())
    e2e = {"value": e2e_pairs / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(9 * 8 * tps),
           "d2h_bytes_per_step": int(8 * nr * tps), "steps": args.e2e_steps,
           "call": "rp_simulate (C ABI), pinned host trace table in, host complex64 radargram out"}

    line = None
    if rank == 0:
        peaks = measured_peaks()
        sm_mhz = clocks.get("sm_mhz") or peaks.get("clocks_under_load", {}).get("sm_mhz_median") or 1455.0
        n_sm = torch.cuda.get_device_properties(local).multi_processor_count
        pairs_s = stage["pairs_ms"] / 1e3
        evals_rate = my_evals / pairs_s if pairs_s > 0 else 0.0
        clk = sm_mhz * 1e6
        fp32_peak = opcount.FP32_FMA_PER_CLK_PER_SM * n_sm * clk
        mufu_peak = opcount.MUFU_PER_CLK_PER_SM * n_sm * clk
        fp32_rate = opcount.FP32_OPS_PER_EVAL * evals_rate
        mufu_rate = opcount.MUFU_PER_EVAL * evals_rate
        roof = {"bound": "fp32", "kernel": "k_pairs32",
                "achieved": fp32_rate / 1e12, "peak": fp32_peak / 1e12,
                "unit": "T FP32 lane-operations/s",
                "frac": fp32_rate / fp32_peak if fp32_peak else None,
                # DRAM read+write of one launch from the committed ncu capture (2 traces: 353.9 + 82.5
                # MB), scaled by the traces per launch; the kernel is compute-bound (DRAM < 0.1 % of peak)
                "traffic": 436.4e6 * tps / 2.0,
                "traffic_unit": "bytes per launch (ncu, profiles/k_pairs32_large_scene.md, scaled)",
                "peak_source": (f"nominal {opcount.FP32_FMA_PER_CLK_PER_SM} FP32 lanes/clk/SM x {n_sm} SMs x "
                                f"{sm_mhz:.0f} MHz median SM clock under load; MEASURED_PEAKS.json holds HBM "
                                "and bf16 tensor peaks only, and this kernel uses neither"),
                "ops_per_eval": opcount.FP32_OPS_PER_EVAL,
                "sfu": {"achieved": mufu_rate / 1e12, "peak": mufu_peak / 1e12, "unit": "T MUFU/s",
                        "frac": mufu_rate / mufu_peak if mufu_peak else None,
                        "ops_per_eval": opcount.MUFU_PER_EVAL},
                "issue": {"achieved": opcount.INSTR_PER_EVAL * evals_rate / 1e12,
                          "peak": opcount.ISSUE_PER_CLK_PER_SM * n_sm * clk / 1e12,
                          "unit": "T thread-instructions/s",
                          "frac": (opcount.INSTR_PER_EVAL * evals_rate) / (opcount.ISSUE_PER_CLK_PER_SM * n_sm * clk),
                          "instr_per_eval": opcount.INSTR_PER_EVAL},
                "peak_kind": "nominal (no FP32 entry in MEASURED_PEAKS.json)",
                # the reference chain's op count per target leg (two legs per evaluation):
                # the rate the pair kernel delivers in the reference's own arithmetic
                "algorithmic": {
                    "achieved": 2 * opcount.REF_FMA_PER_TARGET_LEG * evals_rate / 1e12,
                    "peak": fp32_peak / 1e12, "unit": "T FP32 FMA-class ops/s (reference chain)",
                    "frac": (2 * opcount.REF_FMA_PER_TARGET_LEG * evals_rate) / fp32_peak if fp32_peak else None,
                    "ops_per_target_leg": opcount.REF_FMA_PER_TARGET_LEG,
                    "sfu_achieved": 2 * opcount.REF_SFU_PER_TARGET_LEG * evals_rate / 1e12,
                    "sfu_peak": mufu_peak / 1e12,
                    "sfu_frac": (2 * opcount.REF_SFU_PER_TARGET_LEG * evals_rate) / mufu_peak if mufu_peak else None,
                    "note": "above 1: hoisted incident terms and the outbound leg's reuse of the inbound "
                            "evaluation; frac above is the instruction-level fraction"},
                "pair_kernel_ms_per_launch": stage["pairs_ms"] / max(stage["pair_launches"], 1),
                "pair_evals_per_s": evals_rate,
                "pair_evals_per_launch": my_evals / max(stage["pair_launches"], 1),
                "mean_counts_per_trace": [float(timed_counts[:, 0].mean()), float(timed_counts[:, 1].mean())],
                "stage_ms": {k: stage[k] for k in ("setup_ms", "pairs_ms", "compress_ms", "tail_ms")},
                "hbm_peak_gbs": peaks.get("hbm_gbs")}
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": WORKLOAD, "traces_per_step": tps, "form": "fast (FP32 split precision)",
                           "l2": "inputs larger than L2: 384 MB resident facet store, ~55 MB of facet "
                                 "records per trace per step",
                           "parallelism": f"replicas over trace ranges x{world}"},
                "e2e": e2e, "roofline": roof, "clocks": clocks, "gpu_launches": launches}
        if args.plain_traces > 0 and world == 1:
            ptr = torch.from_numpy(np.ascontiguousarray(track[1000:1000 + args.plain_traces])).cuda()
            pout = torch.empty((args.plain_traces, nr), dtype=torch.complex128, device="cuda")
            pc = np.zeros((args.plain_traces, 2), np.int64)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            scene.simulate_device(ptr, pout, form="plain", stream=stream, counts=pc, complex128=True)
            e1.record(stream)
            torch.cuda.synchronize()
            pv = opcount.pairs(pc) / (e0.elapsed_time(e1) / 1e3)
            line["plain_form"] = {"value": pv, "unit": UNIT, "traces": args.plain_traces,
                                  "fast_over_plain": value / pv if pv else None}
            line["accuracy"] = accuracy_vs_plain(scene, ptr, pout, pc, stream)
        roof["pair_cfg"] = {f"degree_{d}": simulator.autotune_query(False, d) for d in (0, 3, 4, 5, 6)
                            if simulator.autotune_query(False, d) >= 0}
        if not args.no_cpu_baseline and world == 1:
            line["cpu_baseline"] = cpu_baseline(sc, scene, track, args.cpu_targets, 1000)
        if args.spec_traces > 0 and world == 1:
            for key, kw in (("specular", {"specular": True}), ("ttype0", {"ttype0": True})):
                try:
                    line[key] = run_mode(args, sc, track, stream, value, **kw)
                except Exception as e:
                    line[key] = {"error": f"{type(e).__name__}: {e}"}
            try:
                line["direct"] = run_direct(args, sc, track, stream)
            except Exception as e:
                line["direct"] = {"error": f"{type(e).__name__}: {e}"}
        if args.graph_calls > 0 and world == 1:
            try:
                line["graph"] = run_graph(args, scene, track)
            except Exception as e:
                line["graph"] = {"error": f"{type(e).__name__}: {e}"}
        if args.flyby_traces > 0 and world == 1:
            try:
                line["flyby"] = run_flyby(args, stream)
            except Exception as e:
                line["flyby"] = {"error": f"{type(e).__name__}: {e}"}
        if args.focus and world == 1:
            try:
                line["focus"] = run_focus()
            except Exception as e:
                line["focus"] = {"error": f"{type(e).__name__}: {e}"}
        if args.io and world == 1:
            try:
                line["io"] = run_io()
            except Exception as e:
                line["io"] = {"error": f"{type(e).__name__}: {e}"}
        if world == 1 and (args.batch_scenes > 0 or args.serve_seconds > 0 or args.flyby_serve_seconds > 0):
            scene.close()
            specs, objs, tracks, t_build = batch_workload(args, local)
            if args.batch_scenes > 0:
                try:
                    line["batch"] = run_batch(args, objs, tracks, stream)
                    line["batch"]["setup_s"] = t_build
                    # the pair stage against the headline's (pairs per ms of
                    # the pair stage on both sides)
                    b = line["batch"]
                    bp = b["pairs_per_step"] / (b["stage_ms_per_step"]["pairs_ms"] / 1e3)
                    rs = line["roofline"]
                    hp = line["value"] * line["ms_per_step"] / (rs["stage_ms"]["pairs_ms"] / args.steps)
                    b["pair_stage"] = {"pairs_per_s": bp, "headline_pair_stage_pairs_per_s": hp,
                                       "over_headline": bp / hp,
                                       "note": "headline at its traces per call; the batch's 60 MHz "
                                               "evaluations (degree-6 sinc) cost 17% more instructions"}
                except Exception as e:       # reported in the line; the headline stands
                    line["batch"] = {"error": f"{type(e).__name__}: {e}"}
            plain = line.get("plain_form", {}).get("value")
            if args.serve_seconds > 0:
                try:
                    line["serving"] = run_serving(args, objs, tracks, plain)
                except Exception as e:
                    line["serving"] = {"error": f"{type(e).__name__}: {e}"}
            if args.flyby_serve_seconds > 0:
                try:
                    line["serving_flybys"] = run_serving_flybys(args, objs, tracks, plain)
                except Exception as e:
                    line["serving_flybys"] = {"error": f"{type(e).__name__}: {e}"}
            for o in objs:
                o.close()
        print(json.dumps(line), flush=True)
    scene.close()
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
