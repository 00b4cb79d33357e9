"""celer-sim's input, set-up and transport loop over the GB300 stepper.

The reference's application layer reads a JSON ``RunnerInput``
(app/celer-sim/RunnerInput.hh:41-141, read by RunnerInputIO.json.cc:37-140),
builds the problem (``Runner::build_core_params``, app/celer-sim/Runner.cc:
281-446) and transports each event with a ``Transporter``
(app/celer-sim/Transporter.cc:84-179): insert the primaries, step until no
track is alive or queued, abort with ``kill_active`` at ``max_steps``, and
record the track counts and times of every step. This module reads the same
keys and does the same with the GB300 library:

* ``RunnerInput.from_json``: the keys the stepping loop uses --
  ``geometry_file`` (a built-in name, ``calo`` or ``cms``, or a geometry
  file), ``physics_file`` (the synthetic physics input of this package, in
  place of a ROOT/Geant4 export), ``event_file`` (primaries as text lines
  ``pdg energy x y z dx dy dz time event``) or ``primary_options``
  (``PrimaryGeneratorOptions``, sampled on the device), ``seed``,
  ``num_track_slots``, ``max_steps``, ``initializer_capacity``,
  ``secondary_stack_factor``, ``use_device``, ``action_times``,
  ``merge_events``, ``warm_up``, ``field`` [tesla], ``field_options``,
  ``brem_combined``, ``track_order``, ``simple_calo``,
  ``write_track_counts``, ``write_step_times``; required and deprecated keys
  as the reference has them. Keys for what this build does not run (Geant4
  physics options, optical physics, MC-truth and diagnostic output, step
  limiter) are rejected with a message.
* GB300 options under the same object: ``precision`` (``double`` or
  ``mixed``), ``msc`` (multiple scattering, default on),
  ``rng_per_track``, ``reentrant_looping``, ``rz_field_file``.
* ``Runner``: parameters and one stepper; ``Runner.run()`` transports the
  events (all together with ``merge_events``, else one after the other) and
  returns celer-sim's result layout.

Usage: ``python -m celeritas_gb300.runner input.json [-o output.json]``.
"""

from __future__ import annotations

import argparse
import dataclasses
import json
import sys
import time

import numpy as np

#: TrackOrder names (src/celeritas/Types.cc:51-63); this build runs them all
TRACK_ORDER_NAMES = {"none": 0, "init_charge": 1, "reindex_shuffle": 2,
                     "reindex_status": 3, "reindex_particle_type": 4,
                     "reindex_along_step_action": 5, "reindex_step_limit_action": 6,
                     "reindex_both_action": 7}
SUPPORTED_TRACK_ORDERS = tuple(range(8))

#: Keys renamed in the reference (old -> new, RunnerInputIO.json.cc:51-109)
DEPRECATED_KEYS = {"hepmc3_filename": "event_file", "event_filename": "event_file",
                   "geometry_filename": "geometry_file",
                   "physics_filename": "physics_file",
                   "primary_gen_options": "primary_options",
                   "max_num_tracks": "num_track_slots", "sync": "action_times",
                   "mag_field": "field"}

#: Keys of RunnerInput for outputs and physics that the GB300 stepping loop
#: does not produce or run
UNSUPPORTED_KEYS = ("physics_options", "geant_options", "optical", "mctruth_file",
                    "mctruth_filename", "mctruth_filter", "tracing_file",
                    "action_diagnostic", "step_diagnostic", "step_diagnostic_bins",
                    "step_diagnostic_maxsteps", "slot_diagnostic_prefix",
                    "file_sampling_options")

#: Keys read and not used by a device-only stepping loop
IGNORED_KEYS = ("cuda_heap_size", "cuda_stack_size", "environ", "default_stream")


class RunnerInputError(ValueError):
    """Invalid or unsupported celer-sim input."""


@dataclasses.dataclass
class RunnerInput:
    """The subset of celer-sim's RunnerInput that the stepping loop uses."""

    geometry_file: str = ""
    physics_file: str = ""
    event_file: str = ""
    primary_options: dict | None = None
    seed: int = 0
    num_track_slots: int = 0
    max_steps: int = (1 << 32) - 1
    initializer_capacity: int = 0
    secondary_stack_factor: float = 0.0
    use_device: bool = False
    action_times: bool = False
    merge_events: bool = False
    warm_up: bool = False
    field: tuple = (0.0, 0.0, 0.0)
    field_options: dict | None = None
    step_limiter: float = 0.0
    brem_combined: bool = False
    track_order: str = "none"
    simple_calo: list | None = None
    write_track_counts: bool = True
    write_step_times: bool = True
    # GB300 options
    precision: str = "double"
    msc: bool = True
    rng_per_track: bool = False
    reentrant_looping: bool = False
    rz_field_file: str = ""

    REQUIRED = ("initializer_capacity", "secondary_stack_factor", "use_device")

    @classmethod
    def from_json(cls, data) -> "RunnerInput":
        """Read from a JSON object (dict), a JSON string or a file path."""
        if isinstance(data, str):
            if data.lstrip().startswith("{"):
                data = json.loads(data)
            else:
                with open(data) as f:
                    data = json.load(f)
        data = dict(data)
        fmt = data.pop("_format", "celer-sim")
        if fmt != "celer-sim":
            raise RunnerInputError(f"input format '{fmt}' is not 'celer-sim'")
        data.pop("_version", None)
        data.pop("_units", None)
        for old, new in DEPRECATED_KEYS.items():
            if old in data:
                if new in data:
                    raise RunnerInputError(f"both '{old}' and its replacement '{new}'")
                data[new] = data.pop(old)
        for key in UNSUPPORTED_KEYS:
            if key in data:
                raise RunnerInputError(
                    f"'{key}' is not supported by the GB300 stepping loop")
        for key in IGNORED_KEYS:
            data.pop(key, None)
        names = {f.name for f in dataclasses.fields(cls)}
        unknown = sorted(set(data) - names)
        if unknown:
            raise RunnerInputError(f"unknown input keys: {', '.join(unknown)}")
        for key in cls.REQUIRED:
            if key not in data:
                raise RunnerInputError(f"missing required input '{key}'")
        if "geometry_file" not in data:
            raise RunnerInputError("missing required input 'geometry_file'")
        inp = cls(**data)
        inp.field = tuple(float(v) for v in inp.field)
        inp.validate()
        return inp

    def validate(self):
        """The reference's RunnerInput::operator bool and from_json checks,
        plus what this build runs."""
        if bool(self.primary_options) == bool(self.event_file):
            raise RunnerInputError("either a event filename or options to generate "
                                   "primaries must be provided (but not both)")
        if self.field_options and not any(self.field) and not self.rz_field_file:
            raise RunnerInputError("'field_options' cannot be specified without "
                                   "providing 'field'")
        if not (self.num_track_slots > 0 and self.max_steps > 0
                and self.initializer_capacity > 0 and self.secondary_stack_factor > 0):
            raise RunnerInputError("num_track_slots, max_steps, initializer_capacity and "
                                   "secondary_stack_factor must be positive")
        if not self.use_device:
            raise RunnerInputError("use_device must be true: the GB300 stepping loop "
                                   "runs on the device only")
        if self.step_limiter > 0:
            raise RunnerInputError("'step_limiter' is not supported by the GB300 "
                                   "stepping loop")
        order = TRACK_ORDER_NAMES.get(self.track_order)
        if order is None or order not in SUPPORTED_TRACK_ORDERS:
            raise RunnerInputError(f"unknown track order '{self.track_order}' (track_order)")
        if self.precision not in ("double", "mixed"):
            raise RunnerInputError("precision must be 'double' or 'mixed'")
        if self.rz_field_file and any(self.field):
            raise RunnerInputError("'rz_field_file' excludes 'field'")

    @property
    def track_order_id(self) -> int:
        return TRACK_ORDER_NAMES[self.track_order]


def read_event_file(path: str) -> np.ndarray:
    """Primaries of an event file: one 'pdg energy[MeV] x y z [cm] dx dy dz
    time[s] event' line per primary."""
    from .primaries import PRIMARY_DTYPE

    rows = np.loadtxt(path, ndmin=2)
    if rows.size == 0:
        return np.zeros(0, dtype=PRIMARY_DTYPE)
    if rows.shape[1] != 10:
        raise RunnerInputError(f"{path}: expected 10 columns per primary")
    p = np.zeros(len(rows), dtype=PRIMARY_DTYPE)
    p["pdg"] = rows[:, 0].astype(np.int32)
    p["energy"] = rows[:, 1]
    p["pos"] = rows[:, 2:5]
    p["dir"] = rows[:, 5:8]
    p["time"] = rows[:, 8]
    p["event"] = rows[:, 9].astype(np.uint32)
    return p


@dataclasses.dataclass
class TransporterResult:
    """Per-event result (app/celer-sim/Transporter.hh TransporterResult)."""

    initializers: list
    active: list
    alive: list
    step_times: list
    num_track_slots: int
    num_step_iterations: int = 0
    num_steps: int = 0
    num_aborted: int = 0
    max_queued: int = 0

    def to_json(self, counts: bool, times: bool) -> dict:
        out = {"num_track_slots": self.num_track_slots,
               "num_step_iterations": self.num_step_iterations,
               "num_steps": self.num_steps, "num_aborted": self.num_aborted,
               "max_queued": self.max_queued}
        if counts:
            out.update(initializers=self.initializers, active=self.active, alive=self.alive)
        if times:
            out["step_times"] = self.step_times
        return out


class Runner:
    """Problem set-up and transport (celer-sim's Runner and Transporter)."""

    def __init__(self, inp: RunnerInput):
        from . import Params, Stepper, load_library

        self.input = inp
        t0 = time.perf_counter()
        load_library(precision=inp.precision)
        self.params = Params(inp.physics_file, inp.geometry_file,
                             field_tesla=inp.field, msc=inp.msc,
                             track_order=inp.track_order_id, precision=inp.precision,
                             rng_per_track=inp.rng_per_track,
                             event_tallies=not inp.merge_events,
                             reentrant_looping=inp.reentrant_looping,
                             rz_field=inp.rz_field_file or None,
                             brem_combined=inp.brem_combined,
                             secondary_stack_factor=inp.secondary_stack_factor,
                             field_options=inp.field_options,
                             initializer_capacity=inp.initializer_capacity)
        self.stepper = Stepper(self.params, inp.num_track_slots, seed=inp.seed)
        if inp.action_times:
            self.stepper.set_action_times(True)
        self.setup_time = time.perf_counter() - t0
        self.warmup_time = 0.0
        if inp.warm_up:
            t0 = time.perf_counter()
            self.stepper.warm_up()
            self.warmup_time = time.perf_counter() - t0
        labels = self.params.detector_labels()
        if inp.simple_calo:
            missing = [v for v in inp.simple_calo if v not in labels]
            if missing:
                raise RunnerInputError(f"simple_calo volumes not in the geometry: {missing}")
            self.calo_index = [labels.index(v) for v in inp.simple_calo]
            self.calo_labels = list(inp.simple_calo)
        else:
            self.calo_index = list(range(len(labels)))
            self.calo_labels = labels

    def events(self) -> list:
        """Primaries of each event, in event order (event_file) or None per
        event (primary_options: generated on the device)."""
        inp = self.input
        if inp.event_file:
            p = read_event_file(inp.event_file)
            ids = np.unique(p["event"])
            return [(int(e), p[p["event"] == e]) for e in ids]
        return [(e, None) for e in range(int(inp.primary_options["num_events"]))]

    def _generate(self, first_event: int, num_events: int):
        opts = dict(self.input.primary_options)
        pdg = opts.get("pdg")
        pdg = list(pdg) if isinstance(pdg, (list, tuple)) else [pdg]

        def dist(value):
            if isinstance(value, dict):
                return (value["distribution"], tuple(value.get("params", ())))
            if isinstance(value, (list, tuple)):
                return ("delta", tuple(value))
            return ("delta", (float(value),))

        e_kind, e_par = dist(opts["energy"])
        if e_kind != "delta":
            raise RunnerInputError("primary_options energy: only 'delta' is defined")
        self.stepper.generate_primaries(
            pdg=pdg, energy=float(e_par[0]), position=dist(opts["position"]),
            direction=dist(opts["direction"]), num_events=num_events,
            primaries_per_event=int(opts["primaries_per_event"]),
            first_event=first_event, seed=int(opts.get("seed", 0)))

    def transport(self, primaries, first_event=0, num_events=1) -> TransporterResult:
        """One Transporter call: insert (or generate) the primaries and step
        until nothing is alive or queued; at max_steps the tracks in flight
        are killed (Transporter.cc:135-150) and counted as aborted."""
        st, inp = self.stepper, self.input
        res = TransporterResult([], [], [], [], inp.num_track_slots)
        t0 = time.perf_counter()
        if primaries is None:
            self._generate(first_event, num_events)
            r = st.step()
        else:
            r = st.step(primaries)
        res.step_times.append(time.perf_counter() - t0)

        def record(r):
            res.initializers.append(r.queued)
            res.active.append(r.active)
            res.alive.append(r.alive)
            res.num_steps += r.active
            res.max_queued = max(res.max_queued, r.queued)

        record(r)
        iters = 1
        while (r.alive or r.queued) and iters < inp.max_steps:
            batch = min(64, inp.max_steps - iters)
            t0 = time.perf_counter()
            rs = st.run(max_steps=batch, batch=batch)
            dt = (time.perf_counter() - t0) / max(len(rs), 1)
            for r in rs:
                record(r)
                res.step_times.append(dt)
            iters += len(rs)
            if not rs:
                break
        if r.alive or r.queued:
            res.num_aborted = r.alive + r.queued
            st.kill_active()
            while True:
                rs = st.run(max_steps=64, batch=64)
                if not rs or not (rs[-1].alive or rs[-1].queued):
                    break
        res.num_step_iterations = iters
        return res

    def run(self) -> dict:
        """Transport every event; celer-sim's output layout."""
        inp = self.input
        events = self.events()
        t0 = time.perf_counter()
        results = []
        if inp.merge_events:
            self.stepper.clear_energy_deposition()
            if inp.event_file:
                prim = np.concatenate([p for _, p in events])
                results.append(self.transport(prim))
            else:
                results.append(self.transport(None, 0, len(events)))
            edep = self.stepper.energy_deposition()[self.calo_index]
            calo = {"energy_deposition": {"labels": self.calo_labels,
                                          "total": edep.tolist()}}
        else:
            totals = np.zeros(len(self.calo_index))
            per_event = []
            for eid, prim in events:
                res = self.transport(prim, eid, 1)
                results.append(res)
                dep = self.stepper.event_detector_energy_deposition(eid, 1, clear=True)[0]
                per_event.append(dep[self.calo_index].tolist())
                totals += dep[self.calo_index]
            calo = {"energy_deposition": {"labels": self.calo_labels,
                                          "total": totals.tolist(),
                                          "per_event": per_event}}
        total = time.perf_counter() - t0
        out = {"_format": "celer-sim",
               "input": dataclasses.asdict(inp),
               "result": {"runner": {
                   "events": [r.to_json(inp.write_track_counts, inp.write_step_times)
                              for r in results],
                   "time": {"setup": self.setup_time, "warmup": self.warmup_time,
                            "total": total}},
                   "simple_calo": calo}}
        if inp.action_times:
            ms, launches = self.stepper.action_times()
            labels = self.params.action_labels()
            out["result"]["runner"]["time"]["actions"] = {
                labels[i]: float(ms[i]) / 1e3 for i in range(len(labels)) if launches[i]}
        return out


def main(argv=None):
    ap = argparse.ArgumentParser(description="celer-sim input on the GB300 stepping loop")
    ap.add_argument("input", help="celer-sim JSON input ('-' for standard input)")
    ap.add_argument("-o", "--output", help="write the JSON result here (default stdout)")
    args = ap.parse_args(argv)
    text = sys.stdin.read() if args.input == "-" else open(args.input).read()
    result = Runner(RunnerInput.from_json(json.loads(text))).run()
    dump = json.dumps(result, indent=1)
    if args.output:
        with open(args.output, "w") as f:
            f.write(dump + "\n")
    else:
        print(dump)


if __name__ == "__main__":
    main()
