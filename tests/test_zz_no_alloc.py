"""Extend-from-secondaries with the library's static scratch (GB300).

gbx_stepper_extend_from_secondaries_static runs the end-of-step compaction
with its scan scratch in a fixed device array of the library instead of the
stepper's own allocation. Two steppers with the same seed and primaries step
action by action; at the end of each step one runs extend-from-secondaries
through gbx_stepper_launch_action and the other through the static-scratch
entry point. The resulting states must agree: every integer, index and
per-slot field bit for bit, the calorimeter tally (double atomics) to 1e-12
relative. Two steps in a row exercise the array's reuse across calls, and
the library's device-allocation count does not change during the static
calls.

This file is collected last so that it runs after the other GPU tests in the
same process as well as alone.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOTAL_RTOL = 1e-12

# StepActionOrder of each stepping action (src/corecel/sys/ActionInterface.hh:29-45):
# generate 0, start 1, pre 4, user_pre 5, along 7, pre_post 9, post 11,
# user_post 12, end 13. Actions without a step (implicit limiters) are absent.
ACTION_ORDER = {
    "extend-from-primaries": 0,
    "initialize-tracks": 1,
    "pre-step": 4,
    "step-gather-pre": 5,
    "along-step-general-linear": 7,
    "along-step-uniform-msc": 7,
    "along-step-neutral": 7,
    "physics-discrete-select": 9,
    "ioni-moller-bhabha": 11,
    "brems-sb": 11,
    "brems-rel": 11,
    "photoel-livermore": 11,
    "scat-klein-nishina": 11,
    "conv-bethe-heitler": 11,
    "annihil-2-gamma": 11,
    "geo-boundary": 11,
    "tracking-cut": 11,
    "step-gather-post": 12,
    "extend-from-secondaries": 13,
}

PER_SLOT_FIELDS = [
    "status", "track_id", "parent_id", "event_id", "num_steps", "time", "step_length",
    "post_step_action", "along_step_action", "particle_id", "energy",
    "pos_x", "pos_y", "pos_z", "dir_x", "dir_y", "dir_z", "volume", "surface",
    "surface_sense", "boundary", "material", "interaction_mfp", "energy_deposition",
    "secondaries_offset", "secondaries_count", "element", "detector", "vacancies",
    "parents", "rng",
]

INIT_DTYPE = np.dtype({
    "names": ["track_id", "parent_id", "event_id", "time", "pos", "dir", "particle_id",
              "energy", "rng_key"],
    "formats": ["<u4", "<u4", "<u4", "<f8", ("<f8", 3), ("<f8", 3), "<u4", "<f8", "<u8"],
    "offsets": [0, 4, 8, 16, 24, 48, 72, 80, 88],
    "itemsize": 96,
})

COUNTER_NAMES = ["num_vacancies", "num_initializers", "num_secondaries", "num_active",
                 "num_alive", "num_generated", "secondary_stack_size",
                 "num_pending_primaries", "error_flags"]


@pytest.fixture(scope="module")
def gb(built_lib):
    import celeritas_gb300 as gb

    gb.load_library(built_lib)
    return gb


@pytest.fixture(scope="module")
def params(gb):
    return gb.Params(gb.physics_file("calo"), "calo")


def step_sequence(labels):
    ids = [i for i, lab in enumerate(labels) if lab in ACTION_ORDER]
    return sorted(ids, key=lambda i: (ACTION_ORDER[labels[i]], i))


def one_step(stepper, labels, static_scratch):
    for aid in step_sequence(labels):
        if labels[aid] == "extend-from-secondaries" and static_scratch:
            stepper.extend_from_secondaries_static()
        else:
            stepper.launch_action(aid)
    stepper.synchronize()


def counters(st):
    return dict(zip(COUNTER_NAMES, st.get_state("counters", np.uint32)[:len(COUNTER_NAMES)]))


def assert_same_state(a, b):
    ca, cb = counters(a), counters(b)
    assert ca == cb
    assert ca["error_flags"] == 0
    for field in PER_SLOT_FIELDS:
        ra = a.get_state(field, np.uint8)
        rb = b.get_state(field, np.uint8)
        assert np.array_equal(ra, rb), field
    n = int(ca["num_initializers"])
    ia = a.get_state("initializers", np.uint8).view(INIT_DTYPE)[:n]
    ib = b.get_state("initializers", np.uint8).view(INIT_DTYPE)[:n]
    for name in INIT_DTYPE.names:
        assert np.array_equal(ia[name], ib[name]), name
    ea, eb = a.energy_deposition(), b.energy_deposition()
    np.testing.assert_allclose(ea.sum(), eb.sum(), rtol=TOTAL_RTOL)
    np.testing.assert_allclose(ea, eb, rtol=TOTAL_RTOL, atol=1e-12)


def test_initializer_layout(gb, params):
    st = gb.Stepper(params, 1024, seed=0, use_graph=False)
    assert st.state_info("initializers")[0] == INIT_DTYPE.itemsize


def test_static_scratch_matches_allocated_scratch(gb, params):
    from celeritas_gb300.primaries import pencil_beam

    labels = params.action_labels()
    assert "extend-from-secondaries" in labels
    prim = pencil_beam(8, energy=1000.0)
    ref = gb.Stepper(params, 4096, seed=11, use_graph=False)
    new = gb.Stepper(params, 4096, seed=11, use_graph=False)
    assert gb.load_library().gbx_stepper_extend_from_secondaries_static is not None
    ref.insert_primaries(prim)
    new.insert_primaries(prim)
    # Two calls in a row: the second one finds the first one's contents
    for _ in range(2):
        one_step(ref, labels, static_scratch=False)
        before = gb.device_allocations()
        one_step(new, labels, static_scratch=True)
        # The library made no device allocation during the static step
        assert gb.device_allocations() == before
        assert_same_state(ref, new)
    assert counters(new)["num_initializers"] > 0  # secondaries were created
    # Both steppers continue identically through the ordinary step
    for _ in range(3):
        assert ref.step() == new.step()
    assert_same_state(ref, new)


def test_static_scratch_rejects_large_stepper(gb, params):
    big = gb.Stepper(params, gb.STATIC_SCRATCH_MAX_SLOTS + 1, seed=0, use_graph=False)
    with pytest.raises(gb.GbxError, match="static scratch"):
        big.extend_from_secondaries_static()
    # The largest accepted size runs
    edge = gb.Stepper(params, gb.STATIC_SCRATCH_MAX_SLOTS, seed=0, use_graph=False)
    edge.extend_from_secondaries_static()
    edge.synchronize()
    c = counters(edge)
    assert c["num_vacancies"] == gb.STATIC_SCRATCH_MAX_SLOTS
    assert c["error_flags"] == 0


def test_allocation_count_sees_allocations(gb, params):
    """The counter that the no-allocation check reads does count the
    library's allocations: creating a stepper allocates its state."""
    before = gb.device_allocations()
    st = gb.Stepper(params, 1024, seed=0, use_graph=False)
    assert gb.device_allocations() > before
    st.extend_from_secondaries_static()
    st.synchronize()
