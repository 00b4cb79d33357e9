"""Continuous-batching event server on the GB300 (serving configuration).

Per-track random streams make every event's result independent of the
events it shares the device with: each event is served alone, then all are
served together as one stream of arrivals, and each event's energy
deposition, in total and in every detector volume, must agree to 1e-12
relative (the device tally sums with atomics, so only the summation order
differs). Both precisions are checked.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EDEP_RTOL = 1e-12
SLOTS = 1 << 16
NUM_EVENTS = 64


@pytest.fixture(scope="module")
def gb(built_lib):
    import celeritas_gb300 as gb
    from celeritas_gb300.build import build

    gb.load_library(built_lib)
    gb.load_library(build(precision="mixed"), precision="mixed")
    return gb


def make_server(gb, precision):
    from celeritas_gb300 import serving

    steppers, capacity = {}, {}
    for geo, field in (("calo", (1.0, 0.0, 0.0)), ("cms", (0.0, 0.0, 3.8))):
        params = gb.Params(gb.physics_file(geo), geo, field_tesla=field, msc=True,
                           track_order="reindex_both_action", precision=precision,
                           rng_per_track=True, event_tallies=True)
        steppers[geo] = gb.Stepper(params, SLOTS, seed=17)
        capacity[geo] = 16 * SLOTS
    opts = serving.ServerOptions(steps_per_batch=8)
    return serving.EventServer(steppers, capacity, NUM_EVENTS, opts), steppers


def small_requests():
    from celeritas_gb300 import serving

    reqs = serving.make_requests(rate=400.0, duration=0.05, seed=5, max_primaries=8)
    for r in reqs:
        # Keep the test quick: cap primary energies at 3 GeV
        r.primaries["energy"] = np.minimum(r.primaries["energy"], 3000.0)
    assert len(reqs) >= 8
    return reqs


@pytest.mark.parametrize("precision", ["double", "mixed"])
def test_event_results_same_alone_and_in_mix(gb, precision):
    import copy

    from celeritas_gb300 import serving

    reqs = small_requests()
    # Alone: one request at a time through the same steppers
    server, _ = make_server(gb, precision)
    alone = {}
    for r in copy.deepcopy(reqs):
        r.arrival = 0.0
        server.serve([r])
        alone[r.event_id] = (r.energy_deposition, r.detector_deposition)
    # Mixed: all requests on fresh steppers, arriving together
    server, _ = make_server(gb, precision)
    mixed = copy.deepcopy(reqs)
    for r in mixed:
        r.arrival = 0.0
    summary = server.serve(mixed)
    assert summary["completed"] == len(reqs)
    for r in mixed:
        assert r.energy_deposition > 0
        total, per_volume = alone[r.event_id]
        assert r.energy_deposition == pytest.approx(total, rel=EDEP_RTOL)
        # Every detector volume's tally, not only the event's total
        np.testing.assert_allclose(r.detector_deposition, per_volume, rtol=EDEP_RTOL,
                                   atol=EDEP_RTOL * total)
        assert r.detector_deposition.sum() == pytest.approx(total, rel=EDEP_RTOL)


def test_served_stream_reports_latency(gb):
    reqs = small_requests()
    server, steppers = make_server(gb, "mixed")
    summary = server.serve(reqs)
    assert summary["completed"] == len(reqs)
    assert 0 < summary["p50_ms"] <= summary["p99_ms"]
    for r in reqs:
        assert r.admitted >= r.arrival
        assert r.completed >= r.admitted
        # Energy is conserved: deposition never exceeds the primaries' energy
        # (no positron primaries), to the FP32 rounding of the deposits
        assert 0 < r.energy_deposition <= r.primaries["energy"].sum() * (1 + 1e-5)
