"""Speed of the CPU restatement against the reference's own host stepper.

Times ``oracle/_ref/ref_harness bench`` (the reference's Stepper<host>,
compiled from its sources) and ``oracle/_port/port_stepper bench`` (this
repository's per-slot action code compiled for the host) on the same event
subsets of the c2 and c3 workloads, one stepper per thread over all the
machine's cores, and writes the ratio of their track-step rates to
``oracle/port_over_reference.json``. Both run the reference's algorithm
(no reentrant-looping option), FP64, with 4096 slots per thread stepper,
and the host C library's elementary functions (the restatement built as
``bench.py`` times it).

The reference sources exist only where this is run (not on the GPU host),
so the ratio is measured here and committed; ``bench.py`` reports it beside
the CPU baseline that it times with the restatement.

    python oracle/calibrate_port.py [--c2-events 256] [--c3-events 16]
"""

from __future__ import annotations

import argparse
import datetime
import json
import os
import platform
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import numpy as np  # noqa: E402

import oracle  # noqa: E402
from celeritas_gb300 import physics_file  # noqa: E402
from celeritas_gb300.primaries import write_primaries_text  # noqa: E402
from celeritas_gb300.workloads import WORKLOADS, make_primaries, physics_args  # noqa: E402

OUT = os.path.join(HERE, "port_over_reference.json")


def parse(stdout: str) -> dict:
    tok = stdout.split()
    i = tok.index("bench")
    return {"threads": int(tok[i + 2]), "events": int(tok[i + 4]),
            "track_steps": int(tok[i + 6]), "seconds": float(tok[i + 8])}


def time_both(name: str, num_events: int, threads: int, slots: int = 4096) -> dict:
    wl = WORKLOADS[name]
    per_event = wl["num_primaries"] // wl["events"]
    prim = make_primaries(wl, num=num_events * per_event)
    if per_event == 1:
        prim["event"] = np.arange(len(prim))
    args = [a for a in physics_args(wl) if a != "--reentrant-looping"]
    out = {"workload": name, "events": num_events, "primaries_per_event": per_event}
    with tempfile.TemporaryDirectory() as tmp:
        ptxt = os.path.join(tmp, "p.txt")
        write_primaries_text(ptxt, prim)
        for kind, exe in (("reference", oracle.REF_BIN),
                          ("port", oracle.build_port(libm="system"))):
            cmd = [exe, "bench", physics_file(wl["physics"]), wl["geometry"], ptxt,
                   str(slots), str(wl["seed"]), "--threads", str(threads)] + args
            res = subprocess.run(cmd, capture_output=True, text=True, check=True)
            r = parse(res.stdout)
            r["track_steps_per_s"] = r["track_steps"] / r["seconds"]
            out[kind] = r
    out["port_over_reference"] = (out["port"]["track_steps_per_s"]
                                  / out["reference"]["track_steps_per_s"])
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--c2-events", type=int, default=256)
    ap.add_argument("--c3-events", type=int, default=16)
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    args = ap.parse_args()
    if oracle.build_reference(oracle.reference_path()) is None:
        raise SystemExit("reference sources not found; set CELERITAS_REFERENCE")
    runs = [time_both("c2", args.c2_events, args.threads),
            time_both("c3", args.c3_events, args.threads)]
    result = {
        "what": "track-step rate of the CPU restatement (oracle/port) over the "
                "reference's own Stepper<host> (oracle/_ref), same events, same "
                "thread count, 4096 slots per thread stepper, FP64",
        "machine": f"{platform.machine()}, {args.threads} threads",
        "compiler": "g++ -O2 -ffp-contract=off (both)",
        "when": datetime.date.today().isoformat(),
        "command": "python oracle/calibrate_port.py "
                   f"--c2-events {args.c2_events} --c3-events {args.c3_events}",
        "runs": runs,
        "port_over_reference": {r["workload"]: round(r["port_over_reference"], 3)
                                for r in runs},
    }
    with open(OUT, "w") as f:
        json.dump(result, f, indent=1)
        f.write("\n")
    print(json.dumps(result["port_over_reference"]))


if __name__ == "__main__":
    main()
