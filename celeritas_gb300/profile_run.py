"""Run one transport of a benchmark workload for a profiler.

    python -m celeritas_gb300.profile_run --workload c2 [--primaries N]
        [--max-iterations K] [--steps-log FILE] [--graph]
        [--precision double|mixed] [--track-order N] [--slots S]
        [--tuning name=value,...] [--initializer-capacity N] [--rng-per-track]

Inserts the workload's primaries, then steps (eagerly by default, so that
every kernel is its own launch) until the state empties or K iterations have
run. The steps log holds each iteration's step counters and, with an action
sort, the number of slots in each action's sorted range. Meant to be
wrapped by ncu: the launch order is fixed (one launch per step action and
iteration), so '-k <kernel> -s <n>' selects a known iteration.
"""

from __future__ import annotations

import argparse
import json
import sys

import numpy as np

from . import Params, Stepper, load_library, physics_file
from .workloads import WORKLOADS, make_primaries


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="c2", choices=list(WORKLOADS))
    ap.add_argument("--primaries", type=int, default=None)
    ap.add_argument("--max-iterations", type=int, default=20000)
    ap.add_argument("--steps-log", default=None)
    ap.add_argument("--graph", action="store_true")
    ap.add_argument("--precision", default="double", choices=["double", "mixed"])
    ap.add_argument("--track-order", type=int, default=0)
    ap.add_argument("--slots", type=int, default=None,
                    help="track slots (default: the workload's)")
    ap.add_argument("--initializer-capacity", type=int, default=0,
                    help="pending-track queue per stepper (default: 16 per slot)")
    ap.add_argument("--rng-per-track", action="store_true",
                    help="per-track random streams (needed by partition_slots)")
    ap.add_argument("--tuning", default="",
                    help="launch settings, e.g. along_block_size=64,along_persistent=0")
    args = ap.parse_args(argv)

    wl = WORKLOADS[args.workload]
    load_library(precision=args.precision)
    params = Params(physics_file(wl["physics"]), wl["geometry"],
                    field_tesla=wl["field"], msc=wl["msc"],
                    track_order=args.track_order, precision=args.precision,
                    reentrant_looping=wl.get("reentrant_looping", False),
                    initializer_capacity=args.initializer_capacity,
                    rng_per_track=args.rng_per_track)
    stepper = Stepper(params, args.slots or wl["slots"], seed=wl["seed"],
                      use_graph=args.graph)
    if args.tuning:
        stepper.set_tuning(**{k: int(v) for k, v in
                              (kv.split("=") for kv in args.tuning.split(","))})
    prim = make_primaries(wl, num=args.primaries)
    labels = params.action_labels()
    counts = []

    def record():
        # Slots per action in this step's sorted ranges (along-step sort,
        # step-limit sort); empty without an action sort
        if args.track_order:
            along, post = stepper.sorted_action_sizes()
            counts.append({lab: int(along[i] if lab.startswith("along-step") else post[i])
                           for i, lab in enumerate(labels) if along[i] or post[i]})

    res = [stepper.step(prim)]
    record()
    while len(res) < args.max_iterations and (res[-1].alive or res[-1].queued):
        res.append(stepper.step())
        record()
    stepper.synchronize()
    rows = [[r.generated, r.queued, r.active, r.alive] for r in res]
    if args.steps_log:
        with open(args.steps_log, "w") as f:
            json.dump({"workload": args.workload, "primaries": len(prim),
                       "precision": args.precision, "track_order": args.track_order,
                       "steps": rows, "action_slots": counts}, f)
    print(f"iterations {len(res)} track-steps {sum(r[2] for r in rows)}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
