"""Benchmark: track-steps/s and events/s of the EM-shower stepping loop.

One benchmark step transports one batch of synthetic primaries (the
workload below) to completion through the GB300 stepper. Prints one JSON
line on rank 0.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload c1]
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

from celeritas_gb300.workloads import WORKLOADS, make_primaries, physics_args  # noqa: E402


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


def cpu_baseline(wl, threads, target_seconds=15.0, events=None):
    """Time the oracle's CPU restatement on the host cores (bounded sample)."""
    import oracle
    from celeritas_gb300 import physics_file
    from celeritas_gb300.primaries import write_primaries_text

    exe = oracle.build_port()
    # One primary per event, events distributed over threads (celer-sim with
    # one stream per thread). A CPU stepper visits every slot each step, so
    # each thread gets 4096 slots (enough for one shower of the workload):
    # a CPU-favourable setting rather than the GPU's slot count per stream
    slots = 4096
    if events is None:
        # Calibrate on a short sample, then size the sample to target_seconds
        probe = cpu_baseline(wl, threads, events=2 * threads)
        steps_per_event = probe["value"] / probe["events_per_s"]
        events = int(target_seconds * probe["value"] / max(steps_per_event, 1.0))
        events = max(2 * threads, min(events, 20000))
    prim = make_primaries(wl, num=events)
    prim["event"] = np.arange(events)
    with tempfile.TemporaryDirectory() as tmp:
        ptxt = os.path.join(tmp, "p.txt")
        write_primaries_text(ptxt, prim)
        res = subprocess.run([exe, "bench", physics_file(wl["physics"]), wl["geometry"], ptxt,
                              str(slots), str(wl["seed"]), "--threads", str(threads)]
                             + physics_args(wl),
                             capture_output=True, text=True, check=True)
    tok = res.stdout.split()
    nev, steps, sec = int(tok[4]), int(tok[6]), float(tok[8])
    return {
        "value": steps / sec,
        "unit": "track-steps/s",
        "events_per_s": nev / sec,
        "cores": threads,
        "kind": "port",
        "sample": f"first {nev} events of the workload, 1 primary each ({steps} "
                  f"track-steps) on {threads} threads, {slots} slots per thread "
                  f"stepper, {sec:.2f} s",
    }


def run_reference(args, wl):
    """CPU path of the reference loop on the host cores (oracle restatement)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    vals, evs = [], []
    base = None
    # Size each step's sample to ~8 s of CPU work from a short probe
    probe = cpu_baseline(wl, threads, events=2 * threads)
    steps_per_event = probe["value"] / probe["events_per_s"]
    events = int(8.0 * probe["value"] / max(steps_per_event, 1.0))
    events = max(2 * threads, min(events, 20000))
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
                         "kind": base["kind"], "sample": base["sample"]},
        "e2e": {"value": value, "unit": "track-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gb300(args, wl):
    import torch

    import celeritas_gb300 as gb
    from celeritas_gb300 import roofline
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
        build()
    if dist:
        dist.barrier()
    gb.load_library()

    params = gb.Params(gb.physics_file(wl["physics"]), wl["geometry"],
                       field_tesla=wl["field"], msc=wl["msc"])
    labels = params.action_labels()
    stepper = gb.Stepper(params, wl["slots"], seed=wl["seed"] + rank)
    stream = torch.cuda.ExternalStream(stepper.stream_handle())
    prim = make_primaries(wl, rank)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")

    def transport():
        return finish([stepper.step(prim)])

    def finish(res):
        # A shower of this workload ends in a few hundred steps; a run that
        # hits the cap has a track that never terminates
        res += stepper.run(max_steps=MAX_STEPS, batch=64)
        if res[-1].alive or res[-1].queued:
            raise RuntimeError(f"transport did not finish in {MAX_STEPS} steps")
        return res

    for _ in range(args.warmup):
        transport()
    torch.cuda.synchronize()

    dev_ms, e2e_s, track_steps, iterations = [], [], [], []
    with ClockSampler(local_rank) as clocks:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            if dist:
                dist.barrier()
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
            dev_ms.append(start.elapsed_time(stop))
            track_steps.append(sum(r.active for r in res))
            iterations.append(len(res))
    total_steps = float(np.sum(track_steps))
    total_ms = float(np.sum(dev_ms))
    total_e2e = float(np.sum(e2e_s))
    if dist:
        t = torch.tensor([total_ms, total_e2e], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms, total_e2e = t.tolist()
        s = torch.tensor([total_steps], device="cuda", dtype=torch.float64)
        dist.all_reduce(s, op=dist.ReduceOp.SUM)
        total_steps = s.item()
    value = total_steps / (total_ms / 1e3)
    events_per_step = wl["events"] * world
    e2e_value = total_steps / total_e2e

    # Roofline of the dominant kernel: time every action with CUDA events on
    # the stepper's stream over one more transport (not part of 'value')
    stepper.set_action_times(True)
    res = transport()
    ms, launches = stepper.action_times()
    stepper.set_action_times(False)
    active = [r.active for r in res]
    bytes_per_action = {}
    for aid, label in enumerate(labels):
        if launches[aid] == 0:
            continue
        # each action launches once per step over all slots
        nbytes = sum(roofline.launch_bytes(label, a, wl["slots"]) for a in active[:launches[aid]])
        bytes_per_action[label] = nbytes
    dom = max((lab for lab in bytes_per_action), key=lambda lab: ms[labels.index(lab)])
    dom_id = labels.index(dom)
    dom_launch_ms = ms[dom_id] / max(launches[dom_id], 1)
    dom_bytes = bytes_per_action[dom] / max(launches[dom_id], 1)
    peak, peak_kind = load_peaks()
    achieved = dom_bytes / (dom_launch_ms / 1e3) / 1e9
    traffic = read_traffic(dom, float(np.mean(active)))

    kernels_per_step = stepper.step_kernels()
    launches_timed = int(sum(it * kernels_per_step + 2 for it in iterations))

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    clk = clocks.summary()
    h2d = int(len(prim)) * 80
    d2h = len(edep) * 8 + 16 * int(np.mean(iterations)) // 64 * 64
    line = {
        "metric": "track-steps/s",
        "value": value,
        "unit": "track-steps/s",
        "events_per_s": events_per_step * args.steps / (total_ms / 1e3),
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": wl["description"], "name": args.workload,
                   "track_steps_per_step": int(np.mean(track_steps)),
                   "iterations_per_step": int(np.mean(iterations)),
                   "l2": "flushed (256 MiB write) between timed steps",
                   "parallelism": f"events sharded over {world} GPU(s)"},
        "e2e": {"value": e2e_value, "unit": "track-steps/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                     "peak_source": peak_kind,
                     "launch_ms": dom_launch_ms,
                     "action_ms_per_step": {labels[i]: ms[i] / max(launches[i], 1)
                                            for i in range(len(labels)) if launches[i]}},
        "gpu_launches": launches_timed,
        "clocks": clk,
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(wl, os.cpu_count() or 1)
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def read_traffic(kernel_label, mean_active):
    """DRAM bytes per launch of a kernel, from the committed ncu capture.

    The capture holds one launch's DRAM bytes and that launch's active track
    slots; the figure is scaled to the mean active slots per launch of this
    run (the traffic of a step action grows with the tracks it processes).
    """
    path = os.path.join(REPO, "profiles", "traffic.txt")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        for line in f:
            tok = line.split()
            if len(tok) >= 3 and tok[0] == kernel_label:
                return float(tok[1]) * mean_active / float(tok[2])
    return None


def main():
    parser = argparse.ArgumentParser()
    parser.add_argument("--gpus", type=int, default=1)
    parser.add_argument("--steps", type=int, default=10)
    parser.add_argument("--warmup", type=int, default=3)
    parser.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    parser.add_argument("--workload", default="c2", choices=list(WORKLOADS))
    parser.add_argument("--no-cpu-baseline", action="store_true")
    args = parser.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    wl = WORKLOADS[args.workload]
    if args.impl == "reference":
        run_reference(args, wl)
    else:
        run_gb300(args, wl)


if __name__ == "__main__":
    main()
