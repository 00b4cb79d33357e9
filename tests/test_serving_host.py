"""Host logic of the event server, with a stand-in stepper (no GPU).

The stand-in gives every event a number of track-steps proportional to its
primary energy and retires one unit of work per live track per step, which
is enough to exercise admission, continuous batching, completion detection
and the latency bookkeeping of celeritas_gb300.serving.
"""

import numpy as np
import pytest

from celeritas_gb300 import serving
from celeritas_gb300.primaries import PRIMARY_DTYPE


class FakeResult:
    def __init__(self, active, queued, alive):
        self.generated = 0
        self.active = active
        self.queued = queued
        self.alive = alive


class FakeStepper:
    """Each primary MeV becomes 'work' units; each step retires up to
    'slots' units across events in arrival order."""

    def __init__(self, slots=1000, num_events=64):
        self.slots = slots
        self.work = np.zeros(num_events)
        self.edep = np.zeros(num_events)
        self.inserted = []

    def _step(self):
        budget = self.slots
        active = 0
        for eid in np.nonzero(self.work > 0)[0]:
            take = min(self.work[eid], budget)
            self.work[eid] -= take
            self.edep[eid] += take
            budget -= take
            active += take
            if budget <= 0:
                break
        rest = self.work.sum()
        return FakeResult(int(active), int(rest), int(min(rest, self.slots)))

    def step(self, primaries=None):
        if primaries is not None:
            self.inserted.append(primaries.copy())
            for p in primaries:
                self.work[p["event"]] += p["energy"]
        return self._step()

    def run(self, max_steps, batch):
        out = []
        for _ in range(max_steps):
            r = self._step()
            out.append(r)
            if not (r.alive or r.queued):
                break
        return out

    def event_live(self, n):
        return (self.work[:n] > 0).astype(np.uint32)

    def event_energy_deposition(self, n, clear=False):
        return self.edep[:n].copy()

    def event_detector_energy_deposition(self, first, n, clear=False):
        # One detector volume holding the whole deposition
        return self.edep[first:first + n, None].copy()


def request(eid, geometry, energies, arrival):
    p = np.zeros(len(energies), dtype=PRIMARY_DTYPE)
    p["energy"] = energies
    p["event"] = eid
    return serving.Request(eid, geometry, p, arrival)


def test_all_requests_complete_with_their_energy():
    reqs = [request(i, "calo" if i % 2 else "cms", [100.0 * (i + 1)], 0.001 * i)
            for i in range(20)]
    server = serving.EventServer({"calo": FakeStepper(), "cms": FakeStepper()},
                                 {"calo": 10**6, "cms": 10**6}, num_events=64)
    summary = server.serve(reqs)
    assert summary["completed"] == 20
    for r in reqs:
        assert r.latency is not None and r.latency >= 0
        assert r.admitted >= r.arrival
        assert r.energy_deposition == pytest.approx(100.0 * (r.event_id + 1))
    assert summary["p99_ms"] >= summary["p50_ms"] >= 0


def test_admission_waits_for_queue_space():
    # Each event's footprint (0.3 per MeV) alone fills most of the queue
    reqs = [request(i, "calo", [3000.0], 0.0) for i in range(4)]
    st = FakeStepper(slots=50)
    opts = serving.ServerOptions(queue_fill=0.9)
    server = serving.EventServer({"calo": st}, {"calo": 1000}, num_events=8, options=opts)
    server.serve(reqs)
    # Admitted one at a time: each insertion holds a single event
    assert [len(batch) for batch in st.inserted] == [1, 1, 1, 1]
    admitted = sorted(r.admitted for r in reqs)
    completed = sorted(r.completed for r in reqs)
    assert all(a >= c for a, c in zip(admitted[1:], completed[:-1]))


def test_event_ids_beyond_capacity_rejected():
    server = serving.EventServer({"calo": FakeStepper()}, {"calo": 10**6}, num_events=4)
    with pytest.raises(ValueError):
        server.serve([request(7, "calo", [1.0], 0.0)])


def test_sequential_latencies_fifo():
    lat = serving.sequential_latencies([0.0, 0.5, 0.6], [1.0, 0.2, 0.1])
    np.testing.assert_allclose(lat, [1.0, 0.7, 0.7])


def test_request_mix_statistics():
    reqs = serving.make_requests(rate=500.0, duration=4.0, seed=3)
    n = len(reqs)
    assert 1700 < n < 2300  # Poisson with mean 2000
    sizes = np.array([len(r.primaries) for r in reqs])
    assert sizes.min() >= 1 and sizes.max() <= 5000
    # Pareto(1.5) from 1: P(N >= 10) = 10^-1.5 ~ 3.2%
    assert 0.015 < (sizes >= 10).mean() < 0.06
    frac_cms = np.mean([r.geometry == "cms" for r in reqs])
    assert 0.45 < frac_cms < 0.55
    assert all(int(r.primaries["event"][0]) == r.event_id for r in reqs)
