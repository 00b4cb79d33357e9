"""Continuous-batching event server over GB300 steppers.

Events (requests) arrive at given times, each with its own primaries and
geometry. Every geometry has one stepper: a fixed pool of device track slots
plus a queue of track initializers. A request is admitted as soon as it has
arrived and its estimated footprint in the queue fits beside the capacity
held by the events already in flight (their estimated peaks while their
showers grow, their live tracks once past the peak); its primaries join the running step loop (continuous
batching: in-flight events keep stepping while new ones enter), and it
completes when it has no live track left (occupied slot or queued
initializer). Each stepper is driven by its own host thread, so the steppers'
CUDA streams overlap on the device; ctypes releases the GIL during calls.

Results are reproducible per event: with per-track random streams
(rng_per_track) every track's random sequence depends only on its ancestry,
so an event's energy deposition, in total and in each detector volume, is
the same alone and in any mix, up to the summation order of the device
tally (atomics).

The latency of a request is its completion time minus its arrival time, on
the host's monotonic clock.
"""

from __future__ import annotations

import dataclasses
import threading
import time
from typing import Callable, Sequence

import numpy as np


@dataclasses.dataclass
class Request:
    """One event to transport."""

    event_id: int
    geometry: str
    primaries: np.ndarray  # PRIMARY_DTYPE, 'event' set to event_id
    arrival: float  # seconds after the start of the run
    admitted: float | None = None
    completed: float | None = None
    energy_deposition: float | None = None
    #: Deposition of each detector volume [MeV], in the order of the
    #: stepper's detector labels
    detector_deposition: np.ndarray | None = None

    @property
    def latency(self) -> float | None:
        if self.completed is None:
            return None
        return self.completed - self.arrival

    def footprint(self, initializers_per_mev: float) -> float:
        """Estimated peak queued initializers of this event: the pending-track
        queue is the device memory that an event's shower fills (the
        secondary stack, secondary_stack_factor x slots as in the
        reference's PhysicsData.hh:250,501-502, takes at most two
        secondaries per track and step and cannot overflow at factor 3)."""
        return float(self.primaries["energy"].sum()) * initializers_per_mev


@dataclasses.dataclass
class ServerOptions:
    #: Steps per graph-replayed batch between admissions and completion checks
    steps_per_batch: int = 16
    #: Estimated peak queue footprint per MeV of primary energy (the c3
    #: events peak at about 0.26 pending tracks per MeV)
    initializers_per_mev: float = 0.35
    #: Capacity held for an event past its peak, per live track
    past_peak_margin: float = 1.25
    #: Fraction of the initializer queue that admitted events may fill
    queue_fill: float = 0.7
    #: Cap on primaries inserted in one step
    max_primaries_per_insert: int = 1 << 16
    #: Stop after this many seconds even if requests are unfinished
    timeout: float = 600.0


class GeometryLane:
    """One stepper serving the requests of one geometry (runs in a thread)."""

    def __init__(self, stepper, queue_capacity: int, num_events: int,
                 options: ServerOptions, clock: Callable[[], float]):
        self.stepper = stepper
        self.capacity = queue_capacity
        self.num_events = num_events
        self.opt = options
        self.clock = clock
        self.requests: list[Request] = []
        self.error: BaseException | None = None
        self.steps = 0
        self.track_steps = 0

    def run(self):
        try:
            self._run()
        except BaseException as e:  # reported by the server after join
            self.error = e

    def _run(self):
        pending = sorted(self.requests, key=lambda r: r.arrival)
        in_flight: dict[int, Request] = {}
        # Queue capacity held for each event in flight: its estimated peak
        # footprint while its live-track count grows, then (past the peak of
        # its shower) its live tracks, which only shrink from there
        reserved: dict[int, float] = {}
        last_live: dict[int, int] = {}
        queued = 0
        deadline = self.opt.timeout
        while pending or in_flight:
            now = self.clock()
            if now > deadline:
                raise TimeoutError("serving run exceeded its time limit")
            # Admission: arrived requests whose footprint fits beside the
            # capacity held by the events in flight and beside the tracks
            # actually queued, in arrival order
            batch = []
            nprim = 0
            limit = self.opt.queue_fill * self.capacity
            held = sum(reserved.values())
            while pending and pending[0].arrival <= now:
                r = pending[0]
                need = r.footprint(self.opt.initializers_per_mev)
                if in_flight and max(held, queued) + need > limit:
                    break
                if nprim + len(r.primaries) > self.opt.max_primaries_per_insert and batch:
                    break
                pending.pop(0)
                r.admitted = now
                in_flight[r.event_id] = r
                reserved[r.event_id] = need
                held += need
                queued += need
                batch.append(r.primaries)
                nprim += len(r.primaries)
            if not in_flight:
                # Idle until the next arrival
                wait = pending[0].arrival - self.clock()
                if wait > 0:
                    time.sleep(min(wait, 0.01))
                continue
            if batch:
                res = [self.stepper.step(np.concatenate(batch))]
            else:
                res = []
            res += self.stepper.run(max_steps=self.opt.steps_per_batch,
                                    batch=self.opt.steps_per_batch)
            self.steps += len(res)
            self.track_steps += sum(r.active for r in res)
            if res:
                queued = res[-1].queued
            # Completion: events with no live track
            live = self.stepper.event_live(self.num_events)
            now = self.clock()
            for eid in in_flight:
                n = int(live[eid])
                if n < last_live.get(eid, 0):
                    reserved[eid] = min(reserved[eid], self.opt.past_peak_margin * n)
                else:
                    reserved[eid] = max(reserved[eid], float(n))
                last_live[eid] = n
            done = [eid for eid in in_flight if live[eid] == 0]
            for eid in done:
                reserved.pop(eid, None)
                last_live.pop(eid, None)
            if done:
                edep = self.stepper.event_energy_deposition(self.num_events)
                lo, hi = min(done), max(done)
                per_det = self.stepper.event_detector_energy_deposition(lo, hi - lo + 1)
                for eid in done:
                    r = in_flight.pop(eid)
                    r.completed = now
                    r.energy_deposition = float(edep[eid])
                    r.detector_deposition = per_det[eid - lo].copy()


class EventServer:
    """Serve requests over one stepper per geometry."""

    def __init__(self, steppers: dict, queue_capacity: dict, num_events: int,
                 options: ServerOptions | None = None):
        self.steppers = steppers
        self.queue_capacity = queue_capacity
        self.num_events = num_events
        self.opt = options or ServerOptions()

    def serve(self, requests: Sequence[Request]) -> dict:
        t0 = time.perf_counter()

        def clock():
            return time.perf_counter() - t0

        lanes = {g: GeometryLane(st, self.queue_capacity[g], self.num_events,
                                 self.opt, clock)
                 for g, st in self.steppers.items()}
        for r in requests:
            if r.event_id >= self.num_events:
                raise ValueError(f"event ID {r.event_id} beyond {self.num_events}")
            lanes[r.geometry].requests.append(r)
        threads = [threading.Thread(target=lane.run, daemon=True) for lane in lanes.values()]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        for lane in lanes.values():
            if lane.error is not None:
                raise lane.error
        wall = clock()
        return summarize(requests, wall,
                         sum(l.track_steps for l in lanes.values()))


def summarize(requests: Sequence[Request], wall: float, track_steps: int = 0) -> dict:
    """Latency percentiles and throughput of a served run."""
    lat = np.array([r.latency for r in requests if r.latency is not None])
    done = len(lat)
    first = min(r.arrival for r in requests) if requests else 0.0
    last = max((r.completed for r in requests if r.completed is not None), default=first)
    span = max(last - first, 1e-9)
    return {
        "events": len(requests),
        "completed": done,
        "p50_ms": float(np.percentile(lat, 50) * 1e3) if done else None,
        "p99_ms": float(np.percentile(lat, 99) * 1e3) if done else None,
        "mean_ms": float(lat.mean() * 1e3) if done else None,
        "events_per_s": done / span,
        "wall_s": wall,
        "track_steps": int(track_steps),
    }


def sequential_latencies(arrivals: Sequence[float], service: Sequence[float]) -> np.ndarray:
    """FIFO single-server latencies: each event starts when it has arrived
    and the previous one has finished, and takes its own service time."""
    order = np.argsort(arrivals, kind="stable")
    lat = np.zeros(len(arrivals))
    free = -np.inf
    for i in order:
        start = max(arrivals[i], free)
        free = start + service[i]
        lat[i] = free - arrivals[i]
    return lat


#: Request mix of the serving benchmark: Poisson arrivals, Pareto(alpha=1.5)
#: primaries per event capped at 5000, geometry CMS-like or calorimeter 50/50
def make_requests(rate: float, duration: float, seed: int = 0, first_event: int = 0,
                  max_primaries: int = 5000, alpha: float = 1.5) -> list[Request]:
    from .primaries import eta_beam, spread_beam

    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    eid = first_event
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            break
        n = int(min(max_primaries, np.floor(1.0 / rng.uniform() ** (1.0 / alpha))))
        geometry = "cms" if rng.uniform() < 0.5 else "calo"
        pseed = int(rng.integers(1 << 31))
        if geometry == "cms":
            p = eta_beam(n, emin=1000.0, emax=1e5, pdgs=(11, 22), seed=pseed)
        else:
            p = spread_beam(n, emin=100.0, emax=1e4, sigma=1.0, pdg=11, seed=pseed)
        p["event"] = eid
        out.append(Request(eid, geometry, p, t))
        eid += 1
    return out
