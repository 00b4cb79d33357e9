"""Benchmark: track-steps/s and events/s of the EM-shower stepping loop.

Default workload: c3, the CMS-like detector (1300 events of 50 e-/gamma
primaries, 3.8 T, 2^21 track slots). The timed steps transport every event
of the configuration once: step k transports the k-th batch of
max(65, ceil(1300 / steps)) consecutive events to completion. Prints one
JSON line on rank 0:

* value / events_per_s: the batched, autotuned, action-sorted
  mixed-precision path (the headline);
* fp64_plain: the plain FP64 path (no action sort, default launches) on the
  same events, and events_per_s_vs_fp64_plain;
* served: the same events streamed through the continuous-batching server
  as Poisson arrivals at each offered rate, with p50/p99 latency, and
  served_events_per_s_vs_fp64_plain;
* mixed_vs_fp64_edep: per-volume deposition of the two paths, paired by
  batch; gpu_vs_cpu_edep: the CPU baseline's sample events transported on
  the GPU (FP64 and mixed) against the CPU run, paired by event;
* roofline, cpu_baseline (with the restatement's calibration against the
  reference's own host stepper), clocks, e2e, and the c2 calorimeter line.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload c3]
                  [--precision mixed|double] [--track-order 0-7] [--no-fp64]
  python bench.py --impl reference ...   # CPU path of the reference loop

Timing: W untimed warm-up steps, then K timed steps; each timed step is
bracketed by CUDA events on the stepper's stream ('value', inputs staged on
the device first) and by a host clock around the whole public-API call with
host buffers ('e2e': primaries copied host->device and the tally copied
device->host inside the timed region). L2 is flushed (a 256 MiB write)
between timed steps. SM clocks are sampled with nvidia-smi during the timed
region. Under torchrun each rank transports its own events (weak scaling);
the time is the max over ranks.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

import numpy as np  # noqa: E402

from celeritas_gb300.workloads import (  # noqa: E402
    WORKLOADS, make_primaries, physics_args, step_batches)


MAX_STEPS = 20000


def load_peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """Samples nvidia-smi SM clocks and throttle reasons in the background."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []
        self.active = False  # keep only samples taken inside timed regions

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            if self.active:
                self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            tok = [t.strip() for t in line.split(",")]
            if len(tok) < 9:
                continue
            try:
                sm.append(float(tok[1]))
                smax = float(tok[2])
            except ValueError:
                continue
            for name, val in zip(names, tok[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def port_over_reference(name):
    """Track-step rate of the CPU restatement over the reference's own host
    stepper on the same events and cores, measured where the reference
    sources exist (oracle/calibrate_port.py) and committed beside it."""
    path = os.path.join(REPO, "oracle", "port_over_reference.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        d = json.load(f)
    ratio = d.get("port_over_reference", {}).get(name)
    return None if ratio is None else {"ratio": ratio, "machine": d.get("machine"),
                                       "command": d.get("command")}


def cpu_baseline(wl, threads, target_seconds=15.0, events=None, tallies=False):
    """Time the oracle's CPU restatement on the host cores (bounded sample).

    The sample is the first 'events' events of the workload (sized to about
    'target_seconds' from a short probe when not given). With 'tallies' the
    per-event deposition of every detector is returned too (array
    [events, detectors], rows in event order)."""
    import oracle
    from celeritas_gb300 import physics_file
    from celeritas_gb300.primaries import write_primaries_text

    # The restatement with the host C library's elementary functions: the
    # reference's own CPU path calls them, and this build reproduces the
    # unmodified reference bit for bit
    exe = oracle.build_port(libm="system")
    # Events distributed over threads (celer-sim with one stream per
    # thread). A CPU stepper visits every slot each step, so each thread gets
    # 4096 slots (enough for one shower of the workload): a CPU-favourable
    # setting rather than the GPU's slot count per stream
    slots = 4096
    per_event = max(1, wl["num_primaries"] // wl["events"])
    if events is None:
        # Calibrate on a short sample, then size the sample to target_seconds
        probe = cpu_baseline(wl, threads, events=threads)
        steps_per_event = probe["value"] / probe["events_per_s"]
        events = int(target_seconds * probe["value"] / max(steps_per_event, 1.0))
        events = max(threads, min(events, 20000))
    prim = make_primaries(wl, num=events * per_event)
    if per_event == 1:
        prim["event"] = np.arange(events)
    with tempfile.TemporaryDirectory() as tmp:
        ptxt = os.path.join(tmp, "p.txt")
        ttxt = os.path.join(tmp, "t.txt")
        write_primaries_text(ptxt, prim)
        extra = ["--event-tallies", ttxt] if tallies else []
        res = subprocess.run([exe, "bench", physics_file(wl["physics"]), wl["geometry"], ptxt,
                              str(slots), str(wl["seed"]), "--threads", str(threads)]
                             + extra + physics_args(wl),
                             capture_output=True, text=True, check=True)
        table = np.loadtxt(ttxt, ndmin=2) if tallies else None
    tok = res.stdout.split()
    nev, steps, sec = int(tok[4]), int(tok[6]), float(tok[8])
    out = {
        "value": steps / sec,
        "unit": "track-steps/s",
        "events_per_s": nev / sec,
        "cores": threads,
        "kind": "port",
        "sample": f"first {nev} events of the workload ({per_event} primaries each, "
                  f"{steps} track-steps) on {threads} threads, {slots} slots per thread "
                  f"stepper, host C library's elementary functions, {sec:.2f} s",
    }
    name = next((k for k, v in WORKLOADS.items() if v is wl), None)
    cal = port_over_reference(name) if name else None
    if cal:
        # The reference's own Stepper<host> ran 1/ratio as fast as the
        # restatement on the same events and cores where it could be built
        out["port_over_reference"] = cal["ratio"]
        out["reference_estimate"] = out["value"] / cal["ratio"]
        out["calibration"] = f"{cal['machine']}: {cal['command']}"
    if tallies:
        order = np.argsort(table[:, 0], kind="stable")
        out["_events"] = prim
        out["_tallies"] = table[order, 1:]
    return out


def run_reference(args, wl):
    """CPU path of the reference loop on the host cores (oracle restatement)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    vals, evs = [], []
    base = None
    # Size each step's sample to ~8 s of CPU work from a short probe
    probe = cpu_baseline(wl, threads, events=threads)
    steps_per_event = probe["value"] / probe["events_per_s"]
    events = int(8.0 * probe["value"] / max(steps_per_event, 1.0))
    events = max(threads, min(events, 20000))
    for i in range(args.warmup + args.steps):
        r = cpu_baseline(wl, threads, events=events)
        if i >= args.warmup:
            vals.append(r["value"])
            evs.append(r["events_per_s"])
            base = r
    value = float(np.mean(vals))
    line = {
        "impl": "reference",
        "metric": "track-steps/s",
        "value": value,
        "unit": "track-steps/s",
        "events_per_s": float(np.mean(evs)),
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": None,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": wl["description"], "name": args.workload},
        "cpu_baseline": {"value": value, "unit": "track-steps/s", "cores": threads,
                         "kind": base["kind"], "sample": base["sample"],
                         "port_over_reference": base.get("port_over_reference")},
        "e2e": {"value": value, "unit": "track-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


DTYPES = {"mixed": "f32 physics + f64 positions/geometry/field/tally", "double": "f64"}


def make_params(wl, precision, track_order, **options):
    """CoreParams of a workload through the public API."""
    import celeritas_gb300 as gb

    gb.load_library(precision=precision)
    return gb.Params(gb.physics_file(wl["physics"]), wl["geometry"],
                     field_tesla=wl["field"], msc=wl["msc"], track_order=track_order,
                     precision=precision,
                     reentrant_looping=wl.get("reentrant_looping", False),
                     rz_field=gb.field_map_file(wl["geometry"]) if wl.get("rz_field") else None,
                     **options)


def measure(args, wl, precision, stream_cls, dist, rank, local_rank, clocks,
            track_order=None, tuning=None, steps=None, warmup=None, actions=True):
    """Time one precision's stepping loop: device and end-to-end throughput,
    per-step tallies, and per-action times for the roofline. Timed step k
    transports the k-th batch of the workload (step_batches). 'tuning' is a
    launch configuration (gbx_stepper_set_tuning settings)."""
    import torch

    import celeritas_gb300 as gb
    from celeritas_gb300 import roofline, sharding

    steps = args.steps if steps is None else steps
    warmup = args.warmup if warmup is None else warmup
    track_order = args.track_order if track_order is None else track_order
    params = make_params(wl, precision, track_order)
    labels = params.action_labels()
    stepper = gb.Stepper(params, wl["slots"], seed=wl["seed"] + rank)
    if tuning:
        stepper.set_tuning(**tuning)
    stream = stream_cls(stepper.stream_handle())
    batches, warm = step_batches(wl, rank, steps)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")

    def finish(res):
        # A shower of this workload ends in a few hundred steps; a run that
        # hits the cap has a track that never terminates
        res += stepper.run(max_steps=MAX_STEPS, batch=64)
        if res[-1].alive or res[-1].queued:
            raise RuntimeError(f"transport did not finish in {MAX_STEPS} steps")
        return res

    for _ in range(warmup):
        finish([stepper.step(warm)])
    torch.cuda.synchronize()

    dev_ms, e2e_s, track_steps, iterations, tallies, events = [], [], [], [], [], 0
    for prim in batches:
        flush.zero_()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        clocks.active = True
        t0 = time.perf_counter()
        stepper.clear_energy_deposition()
        stepper.insert_primaries(prim)  # host -> device copy of primaries
        start = torch.cuda.Event(enable_timing=True)
        stop = torch.cuda.Event(enable_timing=True)
        start.record(stream)
        res = finish([stepper.step()])
        stop.record(stream)
        edep = stepper.energy_deposition()  # device -> host tally
        torch.cuda.synchronize()
        e2e_s.append(time.perf_counter() - t0)
        clocks.active = False
        dev_ms.append(start.elapsed_time(stop))
        track_steps.append(sum(r.active for r in res))
        iterations.append(len(res))
        tallies.append(edep)
        events += len(np.unique(prim["event"]))

    per_action, dom = {}, None
    if actions:
        # Per-action device times over one more (untimed) transport, stepped
        # eagerly so that each step's action ranges can be read back
        stepper.set_action_times(True)
        processed = {lab: 0 for lab in labels}
        res = [stepper.step(batches[0])]
        while True:
            along, post = stepper.sorted_action_sizes()
            active = res[-1].active
            for aid, lab in enumerate(labels):
                if lab.startswith("along-step"):
                    processed[lab] += int(along[aid])
                elif lab in roofline.MODEL_ACTIONS or lab in ("geo-boundary", "tracking-cut"):
                    processed[lab] += int(post[aid])
                else:
                    processed[lab] += active
            if not (res[-1].alive or res[-1].queued) or len(res) >= MAX_STEPS:
                break
            res.append(stepper.step())
        ms, launches = stepper.action_times()
        stepper.set_action_times(False)

        real_bytes = 4 if precision == "mixed" else 8
        for aid, lab in enumerate(labels):
            if launches[aid] == 0:
                continue
            nl = int(launches[aid])
            proc = processed[lab]
            idle = 0 if lab.startswith(("along-step", "sort-")) else wl["slots"] * nl - proc
            b_proc, b_idle = roofline.bytes_per_slot(lab, real_bytes)
            per_action[lab] = {"ms_per_launch": ms[aid] / nl,
                               "bytes_per_launch": (proc * b_proc + max(idle, 0) * b_idle) / nl,
                               "processed_per_launch": proc / nl,
                               "launches": nl}
        dom = max(per_action,
                  key=lambda lab: per_action[lab]["ms_per_launch"] * per_action[lab]["launches"])
    total_ms = float(np.sum(dev_ms))
    total_e2e = float(np.sum(e2e_s))
    total_steps = float(np.sum(track_steps))
    # Slowest rank's times, all ranks' track-steps and tallies (no-op for one
    # process); the per-step tallies stay per rank for the comparisons
    red = sharding.reduce_run(dist, "cuda", total_ms, total_e2e, total_steps,
                              tallies=np.sum(tallies, axis=0))
    total_ms, total_e2e, total_steps = red["time_ms"], red["e2e_s"], red["track_steps"]
    world = max(1, int(os.environ.get("WORLD_SIZE", "1")))
    out = {
        "precision": precision,
        "value": total_steps / (total_ms / 1e3),
        "e2e": total_steps / total_e2e,
        "ms_per_step": total_ms / steps,
        "events_per_s": events * world / (total_ms / 1e3),
        "events_per_s_e2e": events * world / total_e2e,
        "events": events * world,
        "track_order": track_order,
        "track_steps_per_step": int(np.mean(track_steps)),
        "iterations_per_step": int(np.mean(iterations)),
        "tallies": np.array(tallies),
        "total_tallies": red["tallies"],
        "per_action": per_action,
        "dominant": dom,
        "kernels_per_step": stepper.step_kernels(),
        "iterations": iterations,
        "h2d": int(np.mean([len(b) for b in batches])) * 80,
        "d2h": len(tallies[0]) * 8 + 16 * 64,
        "detectors": params.detector_labels(),
    }
    del stepper, params
    return out


def measure_vs_cpu(wl, rank, cpu, labels=None):
    """Per-event, per-detector deposition of the CPU restatement's sample
    events transported again on the GPU (FP64 and mixed, action-sorted,
    per-event tallies), each compared with the CPU run event by event."""
    import celeritas_gb300 as gb

    prim, ref = cpu["_events"], cpu["_tallies"]
    events = np.unique(prim["event"])
    out = {"events": int(len(events)), "cpu": "the cpu_baseline sample (same primaries, "
           "independent random streams)"}
    for precision in ("double", "mixed"):
        params = make_params(wl, precision, 7, event_tallies=True)
        st = gb.Stepper(params, wl["slots"], seed=wl["seed"] + 17 + rank)
        res = [st.step(prim)] + st.run(max_steps=MAX_STEPS, batch=64)
        if res[-1].alive or res[-1].queued:
            raise RuntimeError("transport did not finish")
        gpu = st.event_detector_energy_deposition(0, int(events.max()) + 1)[events]
        out["fp64" if precision == "double" else "mixed"] = compare_paired(gpu, ref, labels)
        del st, params
    return out


def measure_served(args, wl, rank, tuning=None):
    """Served form: every event of the workload streamed through the
    continuous-batching server (mixed precision, action-sorted, per-track
    streams), arriving as a Poisson process at each offered rate in
    'args.served_rates' (events/s). An event is admitted when it has arrived
    and its footprint fits; its tracks join the running step loop, so the
    events in flight overlap on the device. Latency = completion - arrival
    on the host clock."""
    import celeritas_gb300 as gb
    from celeritas_gb300 import serving

    params = make_params(wl, "mixed", args.track_order, rng_per_track=True,
                         event_tallies=True)
    stepper = gb.Stepper(params, wl["slots"], seed=wl["seed"] + rank)
    if tuning:
        stepper.set_tuning(**tuning)
    per_event = wl["num_primaries"] // wl["events"]
    num_events = wl["events"]
    # The stepper's initializer queue (16 x slots) bounds the tracks pending
    server = serving.EventServer({wl["geometry"]: stepper},
                                 {wl["geometry"]: 16 * wl["slots"]}, 1 << 16)
    allp = make_primaries(wl, rank)

    def requests(first, arrivals):
        out = []
        for k, t in enumerate(arrivals):
            p = allp[k * per_event:(k + 1) * per_event].copy()
            p["event"] = first + k
            out.append(serving.Request(first + k, wl["geometry"], p, float(t)))
        return out

    warm = 64
    server.serve(requests(0, np.zeros(warm)))  # warm-up: graphs captured
    runs = []
    first = warm
    for i, rate in enumerate(args.served_rates):
        rng = np.random.default_rng(1000 + 7 * i + 7919 * rank)
        arrivals = np.cumsum(rng.exponential(1.0 / rate, num_events))
        summary = server.serve(requests(first, arrivals))
        summary["offered_rate"] = rate
        summary["arrivals"] = "Poisson"
        runs.append(summary)
        first += num_events
    del server, stepper, params
    return {"primaries_per_event": per_event, "rates": runs,
            "events_per_s": max(r["events_per_s"] for r in runs)}


def tune_workload(wl, precision, rank):
    """Launch configuration for a workload from the autotuner: charged
    along-step block size, persistent kernel and sort threshold, tuned on the
    transport time of the workload's calibration events (its slot count is
    fixed by the workload)."""
    import celeritas_gb300 as gb
    from celeritas_gb300 import autotune

    gb.load_library(precision=precision)
    params = gb.Params(gb.physics_file(wl["physics"]), wl["geometry"],
                       field_tesla=wl["field"], msc=wl["msc"], track_order=7,
                       precision=precision, rng_per_track=True,
                       reentrant_looping=wl.get("reentrant_looping", False),
                       rz_field=gb.field_map_file(wl["geometry"]) if wl.get("rz_field") else None)
    # Calibration events drawn with another beam seed than the timed ones
    prim = make_primaries(wl, rank, num=wl["tune_primaries"], seed_offset=77)
    t0 = time.perf_counter()
    best, trials = autotune.autotune(
        lambda slots: gb.Stepper(params, slots, seed=wl["seed"] + rank), prim,
        slot_counts=(wl["slots"],))
    best.pop("slots", None)
    report = {"settings": best, "calibration_primaries": int(len(prim)),
              "trials": len(trials), "seconds": round(time.perf_counter() - t0, 1)}
    del params
    return best, report


def measure_step_output(args, wl, rank, batch=8):
    """Cost of the step output (every detector hit with all step data) on the
    mixed path. A transport without the output and one that reads the hits
    back every 'batch' steps into the stepper's host buffers are timed by the
    host clock; the step-gather-post action (tally plus the hit kernels) is
    timed per launch with CUDA events, with and without the output."""
    import torch

    import celeritas_gb300 as gb
    from celeritas_gb300 import sharding

    gb.load_library(precision="mixed")
    params = gb.Params(gb.physics_file(wl["physics"]), wl["geometry"],
                       field_tesla=wl["field"], msc=wl["msc"], track_order=args.track_order,
                       precision="mixed",
                       reentrant_looping=wl.get("reentrant_looping", False),
                       rz_field=gb.field_map_file(wl["geometry"]) if wl.get("rz_field") else None)
    labels = params.action_labels()
    gather = labels.index("step-gather-post")
    st = gb.Stepper(params, wl["slots"], seed=wl["seed"] + rank)
    prim = step_batches(wl, rank, 1)[0][0]
    capacity = (batch + 1) * wl["slots"]  # every slot hitting in every step

    def transport(read):
        hits = 0
        res = [st.step(prim)]
        while res[-1].alive or res[-1].queued:
            res += st.run(max_steps=batch, batch=batch)
            if read:
                hits += len(st.read_step_output(copy=False)["step"])
        if read:
            hits += len(st.read_step_output(copy=False)["step"])
        return sum(r.active for r in res), hits

    def timed(read):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        steps, hits = transport(read)
        torch.cuda.synchronize()
        return time.perf_counter() - t0, steps, hits

    def gather_ms(read):
        st.set_action_times(True)
        transport(read)
        ms, launches = st.action_times()
        st.set_action_times(False)
        return float(ms[gather] / max(launches[gather], 1))

    transport(read=False)  # warm-up
    off_s, steps, _ = timed(read=False)
    off_gather = gather_ms(read=False)
    st.set_step_output("all", True, capacity=capacity)
    transport(read=True)  # warm-up: graph capture with the hit kernels
    on_s, steps_on, hits = timed(read=True)
    on_gather = gather_ms(read=True)
    bytes_per_hit = 4 * 7 + 8 * 16  # 7 integers, 16 doubles
    out = {
        "read_every_steps": batch, "selection": "all", "nonzero_energy_deposition": True,
        "track_steps_per_transport": int(steps_on),
        "hits_per_transport": int(hits),
        "bytes_per_hit": bytes_per_hit,
        "transport_s_without": off_s,
        "transport_s_with_reads": on_s,
        "hits_per_s": hits / on_s,
        "hit_bytes_per_s": hits * bytes_per_hit / on_s,
        "gather_post_ms_without": off_gather,
        "gather_post_ms_with": on_gather,
        "timing": "host clock around each transport (synchronized); gather-post per "
                  "launch from CUDA events of an eager transport",
    }
    st.set_step_output(capacity=0)
    del st, params
    return out


def measure_primary_generation(wl, rank, reps=5):
    """Staging one batch of primaries for the next step: generated on the
    device (PrimaryGenerator options: delta energy, box position, isotropic
    direction) against built on the host and inserted (host->device copy),
    host clock around each call with the stream synchronized. The primaries
    are 1 keV electrons, which stop in their first step."""
    import torch

    import celeritas_gb300 as gb
    from celeritas_gb300.primaries import PRIMARY_DTYPE

    gb.load_library(precision="mixed")
    params = gb.Params(gb.physics_file(wl["physics"]), wl["geometry"], precision="mixed")
    st = gb.Stepper(params, wl["slots"], seed=rank)
    n = wl["slots"]
    lo, hi = np.array([-1.0, -1.0, -6.0]), np.array([1.0, 1.0, -5.0])
    energy = 1e-3  # 1 keV: stopped in the first step, so draining is quick

    def host_batch():
        rng = np.random.default_rng(0)
        p = np.zeros(n, dtype=PRIMARY_DTYPE)
        p["pdg"] = 11
        p["energy"] = energy
        p["pos"] = lo + (hi - lo) * rng.random((n, 3))
        mu = 2 * rng.random(n) - 1
        phi = 2 * np.pi * rng.random(n)
        s = np.sqrt(1 - mu * mu)
        p["dir"] = np.stack([s * np.cos(phi), s * np.sin(phi), mu], axis=1)
        return p

    def drain():
        st.step()
        st.kill_active()
        st.run(max_steps=100000)

    host_s, dev_s = [], []
    for rep in range(reps + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st.insert_primaries(host_batch())
        st.synchronize()
        t1 = time.perf_counter()
        drain()
        st.generate_primaries(pdg=11, energy=energy, position=("box", tuple(lo) + tuple(hi)),
                              direction=("isotropic", ()), num_events=1, primaries_per_event=n,
                              first_event=rep + 1, seed=rep)
        st.synchronize()
        t2 = time.perf_counter()
        drain()
        if rep:
            host_s.append(t1 - t0)
            dev_s.append(t2 - t1)
    del st, params
    return {"primaries": n, "host_build_and_insert_ms": 1e3 * float(np.median(host_s)),
            "device_generate_ms": 1e3 * float(np.median(dev_s)),
            "h2d_bytes_saved": n * 80}


def compare_tallies(mixed, fp64):
    """Per-layer energy deposition of the mixed build against FP64, with
    errors from the scatter of the independent timed transports."""
    n = min(len(mixed), len(fp64))
    mm, dm = mixed.mean(axis=0), fp64.mean(axis=0)
    var = mixed.var(axis=0, ddof=1) / len(mixed) + fp64.var(axis=0, ddof=1) / len(fp64)
    used = var > 0
    chi2 = float((((mm - dm) ** 2)[used] / var[used]).sum())
    dof = int(used.sum())
    try:
        from scipy import stats

        p = float(stats.chi2.sf(chi2, dof))
    except ImportError:
        p = None
    big = dm > 1e-3 * dm.max()
    rel = np.abs(mm - dm)[big] / dm[big]
    return {"transports": int(n), "total_rel_diff": float(abs(mm.sum() - dm.sum()) / dm.sum()),
            "layer_chi2": chi2, "layer_dof": dof, "layer_p": p,
            "max_layer_rel_diff": float(rel.max()), "mean_layer_rel_diff": float(rel.mean())}


def compare_paired(a, b, labels=None):
    """Per-volume deposition of two runs over the same inputs (rows: the
    same batch or event in both, random streams independent), as paired
    differences: for each volume the mean difference over the rows and its
    standard error from their scatter give a Student t, turned into the
    normal deviate of the same tail probability; the sum of their squares is
    the chi-square over the volumes. Also the relative difference of the
    total with its standard error, and per-volume relative differences of
    volumes above 1e-3 of the largest."""
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    n = len(a)
    d = a - b
    mean_d = d.mean(axis=0)
    se = d.std(axis=0, ddof=1) / np.sqrt(n)
    used = se > 0
    from scipy import stats

    t = mean_d[used] / se[used]
    z = stats.norm.isf(stats.t.sf(np.abs(t), n - 1))
    chi2 = float((z ** 2).sum())
    dof = int(used.sum())
    ref = b.mean(axis=0)
    tot_d = d.sum(axis=1)
    out = {"rows": int(n), "chi2": chi2, "dof": dof,
           "p": float(stats.chi2.sf(chi2, dof)) if dof else None,
           "total_rel_diff": float(tot_d.mean() / b.sum(axis=1).mean()),
           "total_rel_sigma": float(tot_d.std(ddof=1) / np.sqrt(n) / b.sum(axis=1).mean())}
    big = ref > 1e-3 * ref.max()
    rel = mean_d[big] / ref[big]
    out["mean_abs_volume_rel_diff"] = float(np.abs(rel).mean())
    out["max_abs_volume_rel_diff"] = float(np.abs(rel).max())
    if labels is not None:
        worst = np.argsort(-np.where(used, np.abs(mean_d) / np.where(used, se, 1), 0))[:3]
        out["largest_deviations"] = [
            {"volume": labels[i], "rel_diff": float(mean_d[i] / ref[i]) if ref[i] else None,
             "t": float(mean_d[i] / se[i]) if se[i] else None} for i in worst]
    return out


def run_gb300(args, wl):
    import torch

    from celeritas_gb300.build import build

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    if rank == 0:
        for prec in {args.precision, "double"}:
            build(precision=prec)
    if dist:
        dist.barrier()

    # Event batches (c3): the headline is the batched, autotuned mixed path
    # beside the plain FP64 path (no action sort) on the same events; other
    # workloads compare with the action-sorted FP64 path
    batched = bool(wl.get("events_per_step"))
    precisions = [args.precision] + (["double"] if args.precision != "double"
                                     and not args.no_fp64 and not batched else [])
    results = {}
    tuning, tuning_report = None, None
    if wl.get("tune_primaries") and not args.no_tune:
        tuning, tuning_report = tune_workload(wl, precisions[0], rank)
    ES = torch.cuda.ExternalStream
    with ClockSampler(local_rank) as clocks:
        for prec in precisions:
            results[prec] = measure(args, wl, prec, ES, dist, rank, local_rank, clocks,
                                    tuning=tuning if prec == precisions[0] else None)
        if args.plain or batched:
            # The plain FP64 path: no action sort, default launch settings
            results["plain"] = measure(args, wl, "double", ES, dist, rank, local_rank,
                                       clocks, track_order=0, actions=False)
        clocks_summary = clocks.summary()
    head = results[precisions[0]]
    errors = {}

    def optional(name, fn):
        """A secondary measurement: its failure is reported in the line
        instead of losing the headline"""
        try:
            return fn()
        except Exception as e:  # noqa: BLE001
            errors[name] = f"{type(e).__name__}: {e}"
            return None

    served = None
    if batched and args.served_rates:
        served = optional("served", lambda: measure_served(args, wl, rank, tuning=tuning))
    c2 = None
    if batched and args.c2_steps and args.workload != "c2":
        c2 = optional("c2", lambda: measure_c2(args, dist, rank, local_rank))
    cpu = None
    if not args.no_cpu_baseline and rank == 0:
        cpu = optional("cpu_baseline",
                       lambda: cpu_baseline(wl, os.cpu_count() or 1, tallies=True))

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    dom = head["dominant"]
    act = head["per_action"][dom]
    peak, peak_kind = load_peaks()
    achieved = act["bytes_per_launch"] / (act["ms_per_launch"] / 1e3) / 1e9
    traffic = read_traffic(dom, act["processed_per_launch"], head["precision"],
                           args.workload)
    line = {
        "metric": "track-steps/s",
        "value": head["value"],
        "unit": "track-steps/s",
        "events_per_s": head["events_per_s"],
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": head["ms_per_step"],
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": DTYPES[head["precision"]],
        "data": "synthetic",
        "config": {"workload": wl["description"], "name": args.workload,
                   "precision": head["precision"],
                   "track_order": args.track_order,
                   "events_timed": head["events"],
                   "track_steps_per_step": head["track_steps_per_step"],
                   "iterations_per_step": head["iterations_per_step"],
                   "l2": "flushed (256 MiB write) between timed steps",
                   "parallelism": f"events sharded over {world} GPU(s)",
                   "reentrant_looping": bool(wl.get("reentrant_looping", False)),
                   "tuning": tuning_report},
        "e2e": {"value": head["e2e"], "unit": "track-steps/s",
                "events_per_s": head["events_per_s_e2e"],
                "h2d_bytes_per_step": head["h2d"], "d2h_bytes_per_step": head["d2h"]},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                     "peak_source": peak_kind, "launch_ms": act["ms_per_launch"],
                     "algorithmic_bytes_per_launch": act["bytes_per_launch"],
                     "actions": {k: {"ms": round(v["ms_per_launch"], 4),
                                     "GB/s": round(v["bytes_per_launch"]
                                                   / max(v["ms_per_launch"], 1e-9) / 1e6, 2)}
                                 for k, v in head["per_action"].items()}},
        "gpu_launches": int(sum(it * head["kernels_per_step"] + 2 for it in head["iterations"])),
        "clocks": clocks_summary,
    }
    labels = head["detectors"]
    if "double" in results and head["precision"] != "double":
        fp = results["double"]
        line["fp64"] = {"value": fp["value"], "e2e": fp["e2e"], "ms_per_step": fp["ms_per_step"],
                        "events_per_s": fp["events_per_s"],
                        "iterations_per_step": fp["iterations_per_step"],
                        "dominant_kernel_ms": fp["per_action"][fp["dominant"]]["ms_per_launch"]}
        line["mixed_vs_fp64_edep"] = compare_tallies(head["tallies"], fp["tallies"])
    if "plain" in results:
        pl = results["plain"]
        line["fp64_plain"] = {"value": pl["value"], "e2e": pl["e2e"],
                              "events_per_s": pl["events_per_s"],
                              "events_per_s_e2e": pl["events_per_s_e2e"],
                              "ms_per_step": pl["ms_per_step"], "track_order": 0,
                              "events_timed": pl["events"]}
        line["events_per_s_vs_fp64_plain"] = head["events_per_s"] / pl["events_per_s"]
        if batched:
            # Same events in both: paired per-batch comparison
            line["mixed_vs_fp64_edep"] = compare_paired(head["tallies"], pl["tallies"], labels)
            line["mixed_vs_fp64_edep"]["compared"] = (
                "mixed (sorted, tuned) against plain FP64, per timed batch of the same "
                "events, independent random streams")
    if served:
        line["served"] = served
        if "plain" in results:
            line["served_events_per_s_vs_fp64_plain"] = (
                served["events_per_s"] / results["plain"]["events_per_s"])
    if c2:
        line["c2"] = c2
    if args.step_output:
        line["step_output"] = measure_step_output(args, wl, rank)
    if args.primary_generation:
        line["primary_generation"] = measure_primary_generation(wl, rank)
    if cpu is not None:
        line["gpu_vs_cpu_edep"] = optional("gpu_vs_cpu_edep",
                                           lambda: measure_vs_cpu(wl, rank, cpu, labels))
        line["cpu_baseline"] = {k: v for k, v in cpu.items() if not k.startswith("_")}
    if errors:
        line["errors"] = errors
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def measure_c2(args, dist, rank, local_rank):
    """The calorimeter workload (c2) as an extra line: the mixed and the
    action-sorted FP64 paths, every step transporting all 10^4 primaries,
    with their per-layer deposition difference."""
    import torch

    wl = WORKLOADS["c2"]
    steps, warmup = args.c2_steps, 3
    ES = torch.cuda.ExternalStream
    out = {"workload": wl["description"], "steps": steps, "warmup": warmup}
    with ClockSampler(local_rank) as clocks:
        mixed = measure(args, wl, "mixed", ES, dist, rank, local_rank, clocks, track_order=7,
                        steps=steps, warmup=warmup, actions=True)
        fp64 = measure(args, wl, "double", ES, dist, rank, local_rank, clocks, track_order=7,
                       steps=max(2, steps // 2), warmup=warmup, actions=False)
        out["clocks"] = clocks.summary()
    for name, r in (("mixed", mixed), ("fp64", fp64)):
        out[name] = {"value": r["value"], "e2e": r["e2e"], "events_per_s": r["events_per_s"],
                     "ms_per_step": r["ms_per_step"], "unit": "track-steps/s"}
    out["mixed_vs_fp64_edep"] = compare_tallies(mixed["tallies"], fp64["tallies"])
    dom = mixed.get("dominant")
    if dom:
        # The dominant kernel of the mixed path on this workload: its mean
        # launch time (CUDA events over an eager transport) and its DRAM
        # traffic against the algorithmic bytes
        act = mixed["per_action"][dom]
        traffic = read_traffic(dom, act["processed_per_launch"], "mixed", "c2")
        out["dominant_kernel"] = {
            "kernel": dom, "launch_ms": act["ms_per_launch"],
            "processed_per_launch": act["processed_per_launch"],
            "algorithmic_bytes_per_launch": act["bytes_per_launch"],
            "traffic": traffic,
            "traffic_over_algorithmic": (traffic / act["bytes_per_launch"]
                                         if traffic else None)}
    return out


def run_serving(args, wl):
    """Serving benchmark (c5): the continuous-batching server at several
    Poisson arrival rates, beside the plain FP64 path serving the same
    requests one at a time in arrival order."""
    import torch

    import celeritas_gb300 as gb
    from celeritas_gb300 import serving
    from celeritas_gb300.build import build

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    if rank == 0:
        build(precision="mixed")
        build(precision="double")
    if dist:
        dist.barrier()

    fields = {"calo": (1.0, 0.0, 0.0), "cms": (0.0, 0.0, 3.8)}
    slots = wl["slots"]
    num_events = 1 << 16

    def make_steppers(precision, track_order, per_track):
        gb.load_library(precision=precision)
        out = {}
        for geo, field in fields.items():
            params = gb.Params(gb.physics_file(geo), geo, field_tesla=field, msc=True,
                               track_order=track_order, precision=precision,
                               rng_per_track=per_track, event_tallies=per_track,
                               reentrant_looping=wl.get("reentrant_looping", False))
            out[geo] = gb.Stepper(params, slots, seed=wl["seed"] + rank)
        return out

    steppers = make_steppers("mixed", 7, True)
    server = serving.EventServer(steppers, {g: 16 * slots for g in steppers}, num_events)
    next_event = 0

    def stream(rate, duration, seed):
        nonlocal next_event
        reqs = serving.make_requests(rate, duration, seed=seed + 7919 * rank,
                                     first_event=next_event)
        next_event += len(reqs)
        if next_event >= num_events:
            raise RuntimeError("serving benchmark ran out of event IDs")
        return reqs

    for i in range(args.warmup):
        server.serve(stream(200.0, 0.25, 1000 + i))
    runs = []
    with ClockSampler(local_rank) as clocks:
        clocks.active = True
        for rate in wl["rates"]:
            reqs = stream(float(rate), wl["duration"], rate)
            summary = server.serve(reqs)
            summary["rate"] = rate
            summary["requests"] = [serving.Request(r.event_id, r.geometry, r.primaries,
                                                   r.arrival) for r in reqs]
            runs.append(summary)
        clocks.active = False
    del server, steppers

    # Plain FP64 path, one request at a time in arrival order on the host
    # clock (a FIFO single server): the first 'sequential_sample' requests
    # of each rate's stream, each transported alone from when it has
    # arrived and the previous one has finished
    plain = make_steppers("double", 0, False)
    for run in runs:
        reqs = run.pop("requests")[:args.sequential_sample]
        first = reqs[0].arrival
        t0 = time.perf_counter() - first
        lat, service, last = [], [], first
        for r in reqs:
            now = time.perf_counter() - t0
            if now < r.arrival:
                time.sleep(r.arrival - now)
            start = time.perf_counter() - t0
            st = plain[r.geometry]
            res = [st.step(r.primaries)] + st.run(max_steps=MAX_STEPS, batch=64)
            if res[-1].alive or res[-1].queued:
                raise RuntimeError("plain FP64 transport did not finish")
            done = time.perf_counter() - t0
            service.append(done - start)
            lat.append(done - r.arrival)
            last = done
        lat = np.array(lat)
        run["sequential_fp64"] = {
            "requests": len(reqs), "p50_ms": float(np.percentile(lat, 50) * 1e3),
            "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "events_per_s": len(reqs) / max(last - first, 1e-9),
            "service_ms_mean": float(np.mean(service) * 1e3),
            "timing": "measured: the first requests of the same arrival stream served "
                      "one at a time by the plain FP64 path, host clock"}
    served = runs[-1]["events_per_s"]
    if dist:
        t = torch.tensor([served], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
        served = t.item()
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    line = {
        "metric": "events/s",
        "value": served,
        "unit": "events/s",
        "n_gpus": world,
        "steps": len(runs),
        "warmup": args.warmup,
        "ms_per_step": None,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": DTYPES["mixed"],
        "data": "synthetic",
        "config": {"workload": wl["description"], "name": args.workload,
                   "precision": "mixed", "track_order": 7, "rng": "per-track streams",
                   "value": "served events/s at the highest offered rate, host clock"},
        "e2e": {"value": served, "unit": "events/s",
                "h2d_bytes_per_step": None, "d2h_bytes_per_step": None},
        "serving": runs,
        "clocks": clocks.summary(),
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def run_batching(args, wl):
    """Batching benchmark (c4): uneven events all in flight in one stepper,
    launch configuration chosen by the autotuner on calibration events."""
    import torch

    import celeritas_gb300 as gb
    from celeritas_gb300 import autotune
    from celeritas_gb300.build import build
    from celeritas_gb300.workloads import make_uneven_events

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    if rank == 0:
        build(precision="mixed")
    if dist:
        dist.barrier()
    gb.load_library(precision="mixed")
    params = gb.Params(gb.physics_file(wl["physics"]), wl["geometry"],
                       field_tesla=wl["field"], msc=wl["msc"], track_order=args.track_order,
                       precision="mixed", rng_per_track=True,
                       reentrant_looping=wl.get("reentrant_looping", False),
                       rz_field=gb.field_map_file(wl["geometry"]) if wl.get("rz_field") else None)

    def make_stepper(slots):
        return gb.Stepper(params, slots, seed=wl["seed"] + rank)

    calib = make_uneven_events(wl, wl["calibration_events"], seed=1000 + rank)
    t0 = time.perf_counter()
    best, trials = autotune.autotune(make_stepper, calib)
    tune_s = time.perf_counter() - t0

    prim = make_uneven_events(wl, wl["bench_events"], seed=rank)
    nev = wl["bench_events"]

    def timed(stepper):
        for _ in range(args.warmup):
            autotune.transport(stepper, prim)
        secs, steps = [], []
        for _ in range(args.steps):
            s_, n_ = autotune.transport(stepper, prim)
            secs.append(s_)
            steps.append(n_)
        return float(np.sum(secs)), float(np.sum(steps))

    with ClockSampler(local_rank) as clocks:
        clocks.active = True
        tuned = make_stepper(best["slots"])
        tuned.set_tuning(**{k: v for k, v in best.items() if k != "slots"})
        t_tuned, n_tuned = timed(tuned)
        del tuned
        default = make_stepper(wl["slots"])
        t_def, n_def = timed(default)
        del default
        all_events = None
        if args.c4_all:
            # Every event of the workload in flight together: all primaries
            # inserted at once into the tuned stepper (the pending-track
            # queue takes the primaries waiting for slots and the
            # secondaries of the showers under way), stepped to completion
            allp = make_uneven_events(wl, wl["events"], seed=500 + rank)
            # All primaries wait in the initializer queue at first, beside the
            # secondaries of the showers under way: a queue of 2^26 (about
            # 6 GB of initializers) instead of the default 4 x slots
            params_all = gb.Params(
                gb.physics_file(wl["physics"]), wl["geometry"], field_tesla=wl["field"],
                msc=wl["msc"], track_order=args.track_order, precision="mixed",
                rng_per_track=True, reentrant_looping=wl.get("reentrant_looping", False),
                initializer_capacity=max(1 << 26, 16 * len(allp)))
            st = gb.Stepper(params_all, best["slots"], seed=wl["seed"] + rank)
            st.set_tuning(**{k: v for k, v in best.items() if k != "slots"})
            autotune.transport(st, calib)  # warm-up: graph capture
            st.synchronize()
            t_all = time.perf_counter()
            res = [st.step(allp)] + st.run(max_steps=200000, batch=64)
            st.synchronize()
            secs = time.perf_counter() - t_all
            if res[-1].alive or res[-1].queued:
                raise RuntimeError("the 4096-event transport did not finish")
            steps = sum(r.active for r in res)
            all_events = {"events": int(wl["events"]), "primaries": int(len(allp)),
                          "energy_tev": float(allp["energy"].sum() / 1e6),
                          "peak_queued_initializers": int(max(r.queued for r in res)),
                          "step_iterations": len(res),
                          "seconds": secs, "track_steps": int(steps),
                          "track_steps_per_s": steps / secs,
                          "events_per_s": wl["events"] / secs,
                          "timing": "host clock around the one transport (synchronized)"}
            del st
        clocks.active = False
    if dist:
        t = torch.tensor([t_tuned, t_def], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_tuned, t_def = t.tolist()
        n = torch.tensor([n_tuned, n_def], device="cuda", dtype=torch.float64)
        dist.all_reduce(n, op=dist.ReduceOp.SUM)
        n_tuned, n_def = n.tolist()
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    line = {
        "metric": "track-steps/s",
        "value": n_tuned / t_tuned,
        "unit": "track-steps/s",
        "events_per_s": world * nev * args.steps / t_tuned,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": t_tuned / args.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": DTYPES["mixed"],
        "data": "synthetic",
        "config": {"workload": wl["description"], "name": args.workload,
                   "precision": "mixed", "track_order": args.track_order,
                   "rng": "per-track streams", "events_per_step": nev,
                   "primaries_per_step": int(len(prim)),
                   "timing": "host clock around each transport (synchronized)"},
        "e2e": {"value": n_tuned / t_tuned, "unit": "track-steps/s",
                "h2d_bytes_per_step": int(len(prim)) * 80, "d2h_bytes_per_step": 16 * 64},
        "autotune": {"best": best, "seconds": tune_s,
                     "calibration_events": wl["calibration_events"],
                     "trials": [{"config": t.config,
                                 "track_steps_per_s": t.rate if t.seconds else None,
                                 "note": t.note} for t in trials]},
        "untuned": {"value": n_def / t_def, "events_per_s": world * nev * args.steps / t_def,
                    "slots": wl["slots"]},
        "all_events_in_flight": all_events,
        "clocks": clocks.summary(),
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def read_traffic(kernel_label, processed, precision, workload=None):
    """DRAM bytes per launch of a kernel, from the committed ncu capture.

    The capture holds one launch's DRAM bytes and the track slots that
    launch processed; the figure is scaled to this run's mean processed
    slots per launch (an action's traffic grows with the tracks it
    processes). Only captures of the same precision are used, of the same
    workload where one exists (fifth column).
    """
    path = os.path.join(REPO, "profiles", "traffic.txt")
    if not os.path.exists(path):
        return None
    fallback = None
    with open(path) as f:
        for line in f:
            tok = line.split()
            if len(tok) >= 4 and tok[0] == kernel_label and tok[1] == precision:
                value = float(tok[2]) * processed / float(tok[3])
                if len(tok) >= 5 and tok[4] == workload:
                    return value
                if fallback is None and len(tok) == 4:
                    fallback = value
    return fallback


def main():
    parser = argparse.ArgumentParser()
    parser.add_argument("--gpus", type=int, default=1)
    parser.add_argument("--steps", type=int, default=10)
    parser.add_argument("--warmup", type=int, default=3)
    parser.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    parser.add_argument("--workload", default="c3", choices=list(WORKLOADS))
    parser.add_argument("--no-cpu-baseline", action="store_true")
    parser.add_argument("--precision", default="mixed", choices=["mixed", "double"])
    parser.add_argument("--track-order", type=int, default=7,
                        help="TrackOrder (0-7): 0 none, 1 init_charge, 2-4 reindex "
                             "shuffle/status/particle type, 5-7 action sorts")
    parser.add_argument("--no-fp64", action="store_true",
                        help="skip the FP64 comparison run")
    parser.add_argument("--served-rates", default="30,200",
                        help="event batches (c3): offered Poisson rates [events/s] at "
                             "which all events of the workload are served; empty: none")
    parser.add_argument("--c2-steps", type=int, default=5,
                        help="event batches (c3): timed steps of the extra c2 line; 0: none")
    parser.add_argument("--sequential-sample", type=int, default=40,
                        help="c5: requests of each stream served one at a time by the "
                             "plain FP64 path")
    parser.add_argument("--no-c4-all", dest="c4_all", action="store_false",
                        help="c4: skip the transport of all events in flight together")
    parser.add_argument("--primary-generation", action="store_true",
                        help="also time device primary generation against host insertion")
    parser.add_argument("--step-output", action="store_true",
                        help="also time the step output (detector hits) on the mixed path")
    parser.add_argument("--no-tune", action="store_true",
                        help="skip the autotuner where the workload uses it (c3)")
    parser.add_argument("--plain", action="store_true",
                        help="also time the plain FP64 path (no action sort); always on "
                             "for event batches (c3)")
    args = parser.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    args.served_rates = [float(r) for r in args.served_rates.split(",") if r.strip()]
    wl = WORKLOADS[args.workload]
    if args.workload == "c5":
        if args.impl == "reference":
            run_reference(args, WORKLOADS["c3"])
        else:
            run_serving(args, wl)
    elif args.workload == "c4":
        if args.impl == "reference":
            run_reference(args, WORKLOADS["c3"])
        else:
            run_batching(args, wl)
    elif args.impl == "reference":
        run_reference(args, wl)
    else:
        run_gb300(args, wl)


if __name__ == "__main__":
    main()
