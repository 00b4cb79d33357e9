"""Launch tuning and the autotuner (GB300, batching configuration).

With per-track random streams the launch configuration of a stepper changes
its speed, not its results: every event's energy deposition must be the same
under each tuning (threads per block of the charged along-step, persistent
charged kernel, action sorts on or off, charged tracks sorted by material
too, charged and neutral tracks in partitioned slot ranges) and each track
order to 1e-12
relative (the device tally sums with atomics, so only the summation order
differs). This holds in the mixed-precision build too, whose compiler may
contract multiply-adds, because sorted and unsorted orders run the same
per-action kernels. Invalid settings
are rejected without touching the stepper. The autotuner returns a valid
configuration from the candidates it measured.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EDEP_RTOL = 1e-12
SLOTS = 1 << 15
NUM_EVENTS = 6


@pytest.fixture(scope="module")
def gb(built_lib):
    import celeritas_gb300 as gb
    from celeritas_gb300.build import build

    gb.load_library(built_lib)
    gb.load_library(build(precision="mixed"), precision="mixed")
    return gb


def cms_params(gb, precision, track_order="reindex_both_action"):
    return gb.Params(gb.physics_file("cms"), "cms", field_tesla=(0.0, 0.0, 3.8), msc=True,
                     track_order=track_order, precision=precision,
                     rng_per_track=True, event_tallies=True)


def events():
    from celeritas_gb300.workloads import WORKLOADS, make_uneven_events

    wl = dict(WORKLOADS["c4"], max_primaries=12, emax=3000.0, energy=100.0)
    return make_uneven_events(wl, NUM_EVENTS, seed=3)


def per_event_edep(stepper, prim):
    from celeritas_gb300 import autotune

    autotune.transport(stepper, prim)
    return stepper.event_energy_deposition(NUM_EVENTS)


TUNINGS = [
    {},
    {"along_block_size": 64},
    {"along_block_size": 128, "along_persistent": 0},
    {"sort": 0},
    {"sort_threshold": 1 << 30},
    {"along_persistent": 1, "along_block_size": 128},
    {"sort_material": 1},
    {"sort_material": 3, "along_persistent": 0},
    {"sort_material": 2},
    {"sort_material": 1, "along_persistent": 1, "along_block_size": 128},
    {"partition_slots": 1},
    {"partition_slots": 1, "along_persistent": 0, "sort_threshold": 1 << 12},
]


@pytest.mark.parametrize("precision", ["double", "mixed"])
def test_results_independent_of_tuning(gb, precision):
    params = cms_params(gb, precision)
    prim = events()
    base = per_event_edep(gb.Stepper(params, SLOTS, seed=5), prim)
    assert np.all(base > 0)
    for tuning in TUNINGS[1:]:
        st = gb.Stepper(params, SLOTS, seed=5)
        st.set_tuning(**tuning)
        for key, value in tuning.items():
            if key != "sort_threshold":
                assert st.get_tuning(key) == value
        np.testing.assert_allclose(per_event_edep(st, prim), base, rtol=EDEP_RTOL,
                                   err_msg=str(tuning))
    for order in ("none", "reindex_along_step_action", "reindex_step_limit_action"):
        st = gb.Stepper(cms_params(gb, precision, order), SLOTS, seed=5)
        np.testing.assert_allclose(per_event_edep(st, prim), base, rtol=EDEP_RTOL,
                                   err_msg=order)


def test_invalid_tuning_rejected(gb):
    params = cms_params(gb, "mixed")
    st = gb.Stepper(params, SLOTS, seed=5)
    before = st.get_tuning("along_block_size")
    for bad in ({"along_block_size": 1024}, {"along_block_size": 96},
                {"no_such_setting": 1}):
        with pytest.raises(gb.GbxError):
            st.set_tuning(**bad)
    assert st.get_tuning("along_block_size") == before
    # The stepper still transports after the rejected settings
    assert per_event_edep(st, events()).sum() > 0
    # Partitioned slots need per-track streams: with per-slot streams the
    # slot a track lands in would change its random sequence
    shared = gb.Params(gb.physics_file("cms"), "cms", field_tesla=(0.0, 0.0, 3.8), msc=True,
                       track_order="reindex_both_action", precision="mixed")
    st = gb.Stepper(shared, SLOTS, seed=5)
    with pytest.raises(gb.GbxError):
        st.set_tuning(partition_slots=1)
    assert st.get_tuning("partition_slots") == 0


def test_autotuner_picks_a_measured_candidate(gb):
    from celeritas_gb300 import autotune

    params = cms_params(gb, "mixed")
    prim = events()
    best, trials = autotune.autotune(lambda n: gb.Stepper(params, n, seed=5), prim,
                                     slot_counts=(1 << 14, 1 << 15),
                                     block_sizes=(128, 256, 512), thresholds=(0, 1 << 30))
    measured = [t for t in trials if t.seconds]
    assert best in [t.config for t in measured]
    assert all(t.track_steps > 0 for t in measured)
    # 512 threads run in both kernel forms (registers capped at 128)
    assert not [t for t in trials if not t.seconds]
    assert {(t.config.get("along_block_size"), t.config.get("along_persistent"))
            for t in measured} >= {(512, 0), (512, 1)}
    assert best["slots"] in (1 << 14, 1 << 15)


@pytest.mark.parametrize("precision", ["double", "mixed"])
def test_large_blocks_give_the_same_results(gb, precision):
    """512-thread blocks (the register-capped kernel instances) transport
    each event as 256-thread blocks do: exactly in the FP64 build (no
    contraction, the same operations in both instances); in the mixed
    build, whose compiler contracts multiply-adds per instance, within FP32
    rounding of a deposit."""
    prim = events()
    base = None
    rtol = EDEP_RTOL if precision == "double" else 1e-6
    for persistent in (0, 1):
        for threads in (256, 512):
            st = gb.Stepper(cms_params(gb, precision), SLOTS, seed=5)
            st.set_tuning(along_block_size=threads, along_persistent=persistent)
            edep = per_event_edep(st, prim)
            if base is None:
                base = edep
            np.testing.assert_allclose(edep, base, rtol=rtol)


def test_material_sort_keeps_action_ranges(gb):
    """With the charged tracks also sorted by material, each action's range
    holds the same tracks: the per-action sizes of both sorts agree with the
    plain action sort step by step (per-track streams: the same histories)."""
    prim = events()
    sizes = []
    for material in (0, 1, 3):
        st = gb.Stepper(cms_params(gb, "mixed"), SLOTS, seed=5, use_graph=False)
        st.set_tuning(sort_material=material)
        assert st.get_tuning("sort_material") == material
        res = [st.step(prim)]
        steps = []
        for _ in range(12):
            along, post = st.sorted_action_sizes()
            steps.append((along.copy(), post.copy(), res[-1].active))
            res.append(st.step())
        sizes.append(steps)
    for other in sizes[1:]:
        for (a0, p0, n0), (a1, p1, n1) in zip(sizes[0], other):
            assert n0 == n1
            np.testing.assert_array_equal(a0, a1)
            np.testing.assert_array_equal(p0, p1)
    assert sum(a.sum() for a, _, _ in sizes[0]) > 0
