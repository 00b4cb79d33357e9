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

Both come in two forms: with the host C library's elementary functions
(exp, log, sin, cos, ...) and with correctly rounded ones ("pinned": the
reference through ``ref/pinned_libm.cc``, the restatement through the GB300
build's own ``gbx/Libm.hh``). The FP64 GPU path uses the correctly rounded
functions, so its bit-for-bit parity is checked against the pinned fixtures
(``tests/golden/pinned/``); the host C library's fixtures check the
restatement against the unmodified reference.

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
#: The restatement with the host C library's elementary functions instead of
#: the GB300 build's correctly rounded ones (reproduces REF_BIN)
PORT_SYSLIBM_BIN = os.path.join(PORT_DIR, "port_stepper_syslibm")
#: The restatement with the implicit background navigated by solving every
#: surface (the reference's search), instead of the GB300 path's ordered
#: walks; only its 'geo-rays' mode is used, to check those walks
PORT_GEOSCAN_BIN = os.path.join(PORT_DIR, "port_stepper_geoscan")
#: The restatement that runs every field chord query in full and counts the
#: queries the surface-free ball of the GB300 path would have answered, and
#: any it would have answered wrongly
PORT_BALLCHECK_BIN = os.path.join(PORT_DIR, "port_stepper_ballcheck")
REF_BIN = os.path.join(HERE, "_ref", "ref_harness")
#: The reference harness linked with correctly rounded elementary functions
REF_PINNED_BIN = os.path.join(HERE, "_ref", "ref_harness_pinned")
#: Which libm an oracle program uses: "pinned" (correctly rounded, as the
#: GB300 FP64 build) or "system" (the host C library)
LIBMS = ("pinned", "system")


def reference_path() -> str:
    """Root of the reference's source tree: $CELERITAS_REFERENCE if set,
    else the default location of the sources."""
    return os.environ.get("CELERITAS_REFERENCE", "/root/reference")


def _port_sources():
    srcs = [os.path.join(HERE, "port", "port_stepper.cc"),
            os.path.join(REPO, "celeritas_gb300", "csrc", "host", "HostParams.cc")]
    deps = list(srcs)
    for root, _d, files in os.walk(os.path.join(REPO, "celeritas_gb300", "csrc")):
        deps += [os.path.join(root, f) for f in files if f.endswith((".hh", ".cc"))]
    return srcs, deps


def build_port(force: bool = False, libm: str = "pinned", geo_scan: bool = False,
               check_ball: bool = False) -> str:
    """Compile the CPU restatement with g++ (no FMA contraction), with the
    correctly rounded elementary functions of the GB300 build ("pinned") or
    the host C library's ("system"); with geo_scan, the background is
    navigated by solving every surface; with check_ball, every field chord
    query runs in full and the surface-free ball's answers are counted."""
    if libm not in LIBMS:
        raise ValueError(f"libm must be one of {LIBMS}")
    exe = PORT_BIN if libm == "pinned" else PORT_SYSLIBM_BIN
    if geo_scan:
        exe = PORT_GEOSCAN_BIN
    if check_ball:
        exe = PORT_BALLCHECK_BIN
    os.makedirs(PORT_DIR, exist_ok=True)
    srcs, deps = _port_sources()
    if (not force and os.path.exists(exe)
            and os.path.getmtime(exe) >= max(os.path.getmtime(d) for d in deps)):
        return exe
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-pthread",
           "-o", exe + ".tmp"] + srcs
    if libm == "system":
        cmd.insert(1, "-DGBX_SYSTEM_LIBM")
    if geo_scan:
        cmd.insert(1, "-DGBX_GEO_SCAN_BACKGROUND")
    if check_ball:
        cmd.insert(1, "-DGBX_CHECK_SAFE_BALL")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle port build failed:\n" + res.stderr[-4000:])
    os.replace(exe + ".tmp", exe)
    return exe


def build_reference(reference: str | None = None, jobs: int = 8) -> str | None:
    """Compile the reference harness if the reference sources are present."""
    reference = reference or reference_path()
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
             geometry: str = "calo", extra=(), libm: str = "pinned") -> dict:
    """Run the CPU restatement and parse its output."""
    exe = build_port(libm=libm)
    cmd = [exe, "run", physics, geometry, primaries_txt, str(slots), str(seed), *extra]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle port failed: " + res.stderr[-2000:])
    return parse_run_output(res.stdout)


def run_reference(physics: str, primaries_txt: str, slots: int, seed: int = 0,
                  geometry: str = "calo", extra=(), libm: str = "system") -> dict:
    """Run the reference harness (requires build_reference), linked with the
    host C library ("system") or with correctly rounded elementary functions
    ("pinned")."""
    exe = REF_BIN if libm == "system" else REF_PINNED_BIN
    cmd = [exe, "run", physics, geometry, primaries_txt, str(slots), str(seed), *extra]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("reference harness failed: " + res.stderr[-2000:])
    return parse_run_output(res.stdout)


#: Fields of an 'int' line of the 'interact' mode, after the input index
#: and the model label
INTERACT_FIELDS = ("st", "act", "mat", "E", "dir", "edep", "nsec", "rng")


def write_interaction_inputs(path: str, inputs) -> None:
    """Write interaction inputs, one per line: model label, PDG, energy
    [MeV], position (3) [cm], direction (3), element component."""
    with open(path, "w") as f:
        for model, pdg, e, pos, d, elcomp in inputs:
            f.write(f"{model} {int(pdg)} {float(e)!r} "
                    + " ".join(repr(float(v)) for v in (*pos, *d))
                    + f" {int(elcomp)}\n")


def parse_interact_output(text: str) -> list[dict]:
    """Parse the 'pre', 'int' and 'sec' lines of the 'interact' mode: per
    input, the pre-step's results (step limit and its action, sampled MFP,
    macroscopic and per-process cross sections, range), the track after its
    interaction (status, step-limit action, material, energy, direction,
    deposition, random state) and its secondaries (PDG, energy, direction;
    PDG 0 for one killed by a cutoff)."""
    out: list[dict] = []
    pre: dict[int, dict] = {}

    def vec(t):
        return [float(v) for v in t.strip("()").split(",")]

    for line in text.splitlines():
        tok = line.split()
        if not tok:
            continue
        if tok[0] == "pre":
            kv = dict(t.split("=", 1) for t in tok[2:])
            pre[int(tok[1])] = {"action": int(kv["act"]), "step": float(kv["len"]),
                                "mfp": float(kv["mfp"]), "macro_xs": float(kv["macro"]),
                                "range": float(kv["range"]),
                                "xs": [float(v) for v in kv["xs"].split(",")]}
        elif tok[0] == "int":
            kv = dict(t.split("=", 1) for t in tok[3:])
            assert int(tok[1]) == len(out)
            out.append({"model": tok[2], "pre_step": pre[int(tok[1])],
                        "status": int(kv["st"]),
                        "action": int(kv["act"]), "material": int(kv["mat"]),
                        "energy": float(kv["E"]), "direction": vec(kv["dir"]),
                        "edep": float(kv["edep"]), "num_secondaries": int(kv["nsec"]),
                        "rng": [int(w) for w in kv["rng"].split(",")],
                        "secondaries": []})
        elif tok[0] == "sec":
            kv = dict(t.split("=", 1) for t in tok[3:])
            out[int(tok[1])]["secondaries"].append(
                {"pdg": int(kv["pdg"]), "energy": float(kv["E"]),
                 "direction": vec(kv["dir"])})
    return out


def parse_along_output(text: str) -> list[dict]:
    """Parse the 'along' lines of the 'along' mode: per input, the track after
    its along-step and discrete selection (status, step limit's action, the
    action after selection and the element component it chose or -1, step
    length, position, direction, energy, local deposition, random state)."""
    out: list[dict] = []

    def vec(t):
        return [float(v) for v in t.strip("()").split(",")]

    for line in text.splitlines():
        tok = line.split()
        if tok and tok[0] == "along":
            kv = dict(t.split("=", 1) for t in tok[2:])
            assert int(tok[1]) == len(out)
            out.append({"status": int(kv["st"]), "action": int(kv["act"]),
                        "selected": int(kv["sel"]), "element": int(kv["el"]),
                        "step": float(kv["len"]), "position": vec(kv["pos"]),
                        "direction": vec(kv["dir"]), "energy": float(kv["E"]),
                        "edep": float(kv["edep"]),
                        "rng": [int(w) for w in kv["rng"].split(",")]})
    return out


def run_interactions(program: str, physics: str, geometry: str, inputs_txt: str,
                     seed: int = 0, extra=(), libm: str = "pinned",
                     mode: str = "interact") -> list[dict]:
    """One interaction ('interact') or one along-step ('along') per input,
    through the reference's own actions (program "reference", requires
    build_reference) or the restatement's (program "port"), with the host C
    library's or correctly rounded elementary functions."""
    if program == "reference":
        exe = REF_BIN if libm == "system" else REF_PINNED_BIN
    else:
        exe = build_port(libm=libm)
    cmd = [exe, mode, physics, geometry, inputs_txt, str(seed), *extra]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"{program} {mode} failed: " + res.stderr[-2000:])
    parse = parse_interact_output if mode == "interact" else parse_along_output
    return parse(res.stdout)


def port_libm(function: str, x, libm: str = "pinned"):
    """The restatement's FP64 elementary function 'function' (the GB300
    build's correctly rounded one, or the host C library's) on the host, for
    every element of x (numpy array of doubles)."""
    import numpy as np

    exe = build_port(libm=libm)
    x = np.asarray(x, dtype=np.float64).ravel()
    text = "".join(f"{float(v).hex()}\n" for v in x)
    res = subprocess.run([exe, "libm", function], input=text, capture_output=True,
                         text=True, check=True)
    return np.array([float.fromhex(t) for t in res.stdout.split()], dtype=np.float64)
