"""Benchmark workloads of the EM-shower stepping loop and their primaries.

Five workloads. Two on the 50-layer Pb/lAr sampling calorimeter that the
reference's benchmark problems use (world box 60 x 60 x 60 cm of vacuum;
layers of 2.3 mm Pb + 5.7 mm lAr, 40 x 40 cm, starting at z = 0):

* ``c1`` -- 100 e- at 1 GeV in one event, pencil beam along +z, no field, no
  multiple scattering, 2^16 track slots, seed 0. Small enough for the CPU.
* ``c2`` -- Urban multiple scattering and a uniform 1 T field along x;
  10^4 e-, energies log-uniform in 0.1-10 GeV, Gaussian transverse spread of
  1 cm, one primary per event with all events in flight, 2^20 track slots.

and three on the CMS-like detector (concentric shells, 3.8 T along z):
``c3`` events of 50 primaries, ``c4`` uneven events for the batching
autotuner, ``c5`` a served stream of events on both geometries.

Primaries are synthetic (seeded numpy), standing in for the reference's
PrimaryGenerator (src/celeritas/phys/PrimaryGenerator.cc).

The workloads with a magnetic field run with ``reentrant_looping``: a
field step that ends on a boundary the track re-enters at once keeps its
looping-step count, so that an electron circling in vacuum with its orbit
grazing a surface reaches the looping cut (the reference resets the count
there and such a track never ends; celer-sim stops the whole run at its
global step limit instead).
"""

from __future__ import annotations

import numpy as np

from .primaries import eta_beam, pencil_beam, spread_beam

WORKLOADS = {
    "c1": dict(geometry="calo", physics="calo", num_primaries=100, energy=1000.0,
               emax=None, sigma=0.0, pdg=11, slots=1 << 16, seed=0, events=1,
               msc=False, field=(0.0, 0.0, 0.0),
               description="calorimeter 50x(2.3mm Pb+5.7mm lAr), 100 e- @ 1 GeV "
                           "pencil beam, no field, no MSC, 2^16 track slots, FP64"),
    "c2": dict(geometry="calo", physics="calo", num_primaries=10000, energy=100.0,
               emax=1e4, sigma=1.0, pdg=11, slots=1 << 20, seed=0, events=10000,
               msc=True, field=(1.0, 0.0, 0.0),
               reentrant_looping=True,
               description="calorimeter 50x(2.3mm Pb+5.7mm lAr), Urban MSC, 1 T "
                           "uniform field along x, 10^4 e- log-uniform 0.1-10 GeV, "
                           "sigma 1 cm, 2^20 track slots"),
    # CMS-like detector (concentric shells, 3.8 T along z): 1300 events of
    # 50 primaries, e-/gamma alternating, log-uniform 1-100 GeV, uniform in
    # |eta| < 1.5 from the origin, 2^21 slots
    "c3": dict(geometry="cms", physics="cms", num_primaries=65000, energy=1000.0,
               emax=1e5, sigma=None, pdg=None, pdgs=(11, 22), eta_max=1.5, slots=1 << 21,
               seed=0, events=1300, msc=True, field=(0.0, 0.0, 3.8),
               events_per_step=65, tune_primaries=3250,
               reentrant_looping=True,
               description="CMS-like: 10 Si shells (0.3 mm, r 4-110 cm), PbWO4 barrel "
                           "(r 129-152 cm), 17 x (5 cm brass + 0.4 cm scintillator) "
                           "(r 180-295 cm), 3.8 T along z, Urban MSC; 1300 events of 50 "
                           "e-/gamma, log-uniform 1-100 GeV, |eta| < 1.5; 2^21 slots; "
                           "the timed steps transport all 1300 events in consecutive "
                           "batches of max(65, ceil(1300 / steps)) events; launch "
                           "configuration autotuned on 65 other events"),
    # c3 in the synthetic R-Z field map of the CMS-like detector (a 3.8 T
    # solenoid with soft edges and a return flux) instead of the uniform field
    "c3rz": dict(geometry="cms", physics="cms", num_primaries=65000, energy=1000.0,
                 emax=1e5, sigma=None, pdg=None, pdgs=(11, 22), eta_max=1.5, slots=1 << 21,
                 seed=0, events=1300, msc=True, field=(0.0, 0.0, 0.0), rz_field=True,
                 events_per_step=65, tune_primaries=3250, reentrant_looping=True,
                 description="CMS-like detector in an R-Z field map (3.8 T solenoid, soft "
                             "edges, return flux), Urban MSC; 1300 events of 50 e-/gamma, "
                             "log-uniform 1-100 GeV, |eta| < 1.5; 2^21 slots; the timed "
                             "steps transport all 1300 events in batches of max(65, "
                             "ceil(1300 / steps)); launch configuration autotuned on 65 "
                             "other events"),
    # Batching of uneven events: CMS-like detector, 4096 events with primaries
    # per event log-uniform in 1-1000 and energies log-uniform in
    # 0.1-100 GeV (e-/gamma alternating, |eta| < 1.5), all in flight
    # together, per-track random streams, autotuned launch configuration
    "c4": dict(geometry="cms", physics="cms", events=4096, min_primaries=1,
               max_primaries=1000, energy=100.0, emax=1e5, pdgs=(11, 22), eta_max=1.5,
               slots=1 << 21, seed=0, msc=True, field=(0.0, 0.0, 3.8),
               bench_events=64, calibration_events=8,
               reentrant_looping=True,
               description="batching: CMS-like, events with log-uniform 1-1000 "
                           "e-/gamma primaries of log-uniform 0.1-100 GeV, |eta| < 1.5, "
                           "3.8 T; one bench step = 64 of the 4096 events in flight "
                           "together, then all 4096 in flight together in one "
                           "transport; launch configuration autotuned"),
    # Serving: Poisson arrivals, Pareto(1.5) primaries per event capped at
    # 5000, CMS-like (as c3) or calorimeter (as c2) 50/50, one pool of 2^21
    # slots per geometry (2^22 in all) with queues of 16 x slots
    "c5": dict(geometry="cms+calo", slots=1 << 21, rates=(50, 200, 1000, 2000),
               duration=2.0, seed=0,
               reentrant_looping=True,
               description="serving: Poisson arrivals at 50-2000 events/s for 2 s each, "
                           "Pareto(1.5) primaries capped at 5000, CMS-like or "
                           "calorimeter 50/50, 2 x 2^21 track slots"),
}


def make_primaries(wl: dict, rank: int = 0, num: int | None = None, seed_offset: int = 0):
    """Primaries of a workload; 'rank' offsets the event IDs and the seed."""
    num = wl["num_primaries"] if num is None else num
    if wl.get("pdgs"):
        events = max(1, round(wl["events"] * num / wl["num_primaries"]))
        p = eta_beam(num, emin=wl["energy"], emax=wl["emax"], pdgs=wl["pdgs"],
                     eta_max=wl["eta_max"], seed=wl["seed"] + 1000 * rank + seed_offset,
                     num_events=events)
        p["event"] += rank * wl["events"]
        return p
    if wl["emax"] is None:
        p = pencil_beam(num, energy=wl["energy"], pdg=wl["pdg"],
                        num_events=min(wl["events"], num))
    else:
        p = spread_beam(num, emin=wl["energy"], emax=wl["emax"], sigma=wl["sigma"],
                        pdg=wl["pdg"], seed=wl["seed"] + 1000 * rank + seed_offset,
                        num_events=min(wl["events"], num))
    p["event"] += rank * wl["events"]
    return p


def step_batches(wl: dict, rank: int, steps: int):
    """Primaries of each timed bench step and of the warm-up steps.

    A workload with 'events_per_step' splits its events into consecutive
    batches of that many events, or of ceil(events / steps) where fewer
    steps would leave events out: timed step k transports batch k (modulo the
    number of batches), so that the timed steps cover every event of the
    workload once. Warm-up steps transport one batch of other events
    (another beam seed). Any other workload transports all its primaries in
    every step.
    """
    per_step = wl.get("events_per_step")
    if not per_step:
        p = make_primaries(wl, rank, num=wl.get("bench_primaries"))
        return [p] * steps, p
    per_step = max(per_step, -(-wl["events"] // max(1, steps)))
    per_event = wl["num_primaries"] // wl["events"]
    allp = make_primaries(wl, rank)
    size = per_step * per_event
    nb = -(-wl["events"] // per_step)
    batches = [allp[k * size:(k + 1) * size] for k in range(nb)]
    warm = make_primaries(wl, rank, num=size, seed_offset=55)
    return [batches[k % nb] for k in range(steps)], warm


def physics_args(wl: dict) -> list[str]:
    """Command-line physics options of the CPU oracle programs."""
    args = []
    if wl["msc"]:
        args.append("--msc")
    if wl.get("reentrant_looping"):
        args.append("--reentrant-looping")
    if wl.get("rz_field"):
        from . import field_map_file

        args += ["--rz-field", field_map_file(wl["geometry"])]
    if any(wl["field"]):
        args += ["--field"] + [repr(float(f)) for f in wl["field"]]
    return args


def make_uneven_events(wl: dict, num_events: int, first_event: int = 0, seed: int = 0):
    """Primaries of 'num_events' events of the batching workload: each event
    draws its primary count log-uniformly in [min, max] primaries."""
    rng = np.random.default_rng(wl["seed"] + 7 * seed)
    counts = np.exp(rng.uniform(np.log(wl["min_primaries"]),
                                np.log(wl["max_primaries"] + 1), num_events))
    counts = np.minimum(counts.astype(int), wl["max_primaries"])
    parts = []
    for k, n in enumerate(counts):
        p = eta_beam(int(max(n, 1)), emin=wl["energy"], emax=wl["emax"], pdgs=wl["pdgs"],
                     eta_max=wl["eta_max"], seed=int(rng.integers(1 << 31)))
        p["event"] = first_event + k
        parts.append(p)
    return np.concatenate(parts)
