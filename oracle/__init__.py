"""CPU oracle for the stepping loop (test and baseline infrastructure).

Two checkers live here:

* ``ref/``  - a recipe that compiles the reference's own host stepping loop
  (Stepper<MemSpace::host>, FP64, ORANGE, XORWOW) from its sources and a
  harness that prints per-step track counts and per-volume energy
  deposition. It needs the reference sources, so it only builds where they
  are present; its outputs are committed as golden fixtures under
  ``tests/golden/``.
* ``port/`` - a CPU restatement of the same loop that runs the GB300 path's
  per-slot action functions on the host, validated against the golden
  fixtures; it is the CPU baseline where the reference cannot be built and
  the per-action checker for the GPU kernels.

Only tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU baseline use
this package. The shipped GB300 path never calls it.
"""

from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
PORT_DIR = os.path.join(HERE, "_port")
PORT_BIN = os.path.join(PORT_DIR, "port_stepper")
REF_BIN = os.path.join(HERE, "_ref", "ref_harness")
REFERENCE_DEFAULT = "/root/reference"


def _port_sources():
    srcs = [os.path.join(HERE, "port", "port_stepper.cc"),
            os.path.join(REPO, "celeritas_gb300", "csrc", "host", "HostParams.cc")]
    deps = list(srcs)
    for root, _d, files in os.walk(os.path.join(REPO, "celeritas_gb300", "csrc")):
        deps += [os.path.join(root, f) for f in files if f.endswith((".hh", ".cc"))]
    return srcs, deps


def build_port(force: bool = False) -> str:
    """Compile the CPU restatement with g++ (no FMA contraction)."""
    os.makedirs(PORT_DIR, exist_ok=True)
    srcs, deps = _port_sources()
    if (not force and os.path.exists(PORT_BIN)
            and os.path.getmtime(PORT_BIN) >= max(os.path.getmtime(d) for d in deps)):
        return PORT_BIN
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-pthread",
           "-o", PORT_BIN + ".tmp"] + srcs
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle port build failed:\n" + res.stderr[-4000:])
    os.replace(PORT_BIN + ".tmp", PORT_BIN)
    return PORT_BIN


def build_reference(reference: str = REFERENCE_DEFAULT, jobs: int = 8) -> str | None:
    """Compile the reference harness if the reference sources are present."""
    if not os.path.isdir(os.path.join(reference, "src", "celeritas")):
        return None
    cmd = ["make", "-C", os.path.join(HERE, "ref"), f"-j{jobs}", f"REF={reference}"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("reference oracle build failed:\n" + res.stdout[-4000:]
                           + res.stderr[-4000:])
    return REF_BIN


#: Columns of a 'hit' line of the oracle programs (--hits): the step
#: iteration, then DetectorStepOutput's fields (src/celeritas/user/
#: DetectorSteps.hh:49-80) with positions and directions as three columns
HIT_COLUMNS = ("step", "detector", "track_id", "event_id", "parent_id", "track_step_count",
               "particle", "step_length", "energy_deposition",
               "pre_time", "pre_x", "pre_y", "pre_z", "pre_u", "pre_v", "pre_w", "pre_energy",
               "post_time", "post_x", "post_y", "post_z", "post_u", "post_v", "post_w",
               "post_energy")
HIT_INT_COLUMNS = 7


def parse_run_output(text: str) -> dict:
    """Parse 'step', 'total_steps', 'edep', 'action' and 'hit' lines of a run."""
    steps, edep, actions, hits = [], {}, {}, []
    total = iters = None
    seconds = None
    for line in text.splitlines():
        tok = line.split()
        if not tok:
            continue
        if tok[0] == "step":
            steps.append(tuple(int(t) for t in tok[2:6]))
        elif tok[0] == "edep":
            edep[tok[1]] = float(tok[2])
        elif tok[0] == "action":
            actions[int(tok[1])] = tok[2]
        elif tok[0] == "total_steps":
            total, iters = int(tok[1]), int(tok[3])
        elif tok[0] == "seconds":
            seconds = float(tok[1])
        elif tok[0] == "hit":
            hits.append([int(t) for t in tok[1:1 + HIT_INT_COLUMNS]]
                        + [float(t) for t in tok[1 + HIT_INT_COLUMNS:]])
    return {"steps": steps, "edep": edep, "actions": actions,
            "total_steps": total, "iterations": iters, "seconds": seconds,
            "hits": hits}


def run_port(physics: str, primaries_txt: str, slots: int, seed: int = 0,
             geometry: str = "calo", extra=()) -> dict:
    """Run the CPU restatement and parse its output."""
    exe = build_port()
    cmd = [exe, "run", physics, geometry, primaries_txt, str(slots), str(seed), *extra]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle port failed: " + res.stderr[-2000:])
    return parse_run_output(res.stdout)


def run_reference(physics: str, primaries_txt: str, slots: int, seed: int = 0,
                  geometry: str = "calo", extra=()) -> dict:
    """Run the reference harness (requires build_reference)."""
    cmd = [REF_BIN, "run", physics, geometry, primaries_txt, str(slots), str(seed), *extra]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("reference harness failed: " + res.stderr[-2000:])
    return parse_run_output(res.stdout)
