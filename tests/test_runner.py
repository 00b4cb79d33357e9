"""celer-sim input (RunnerInput) read by celeritas_gb300.runner (no GPU).

The keys, required entries, deprecated names and checks of the reference's
RunnerInputIO (app/celer-sim/RunnerInputIO.json.cc:37-140) and
RunnerInput::operator bool (app/celer-sim/RunnerInput.hh:128-137), plus the
GB300 build's limits (device only; TrackOrder none or an action sort).
"""

import json

import numpy as np
import pytest

from celeritas_gb300.runner import RunnerInput, RunnerInputError, read_event_file


def base(**kw):
    d = {"_format": "celer-sim", "geometry_file": "calo", "physics_file": "calo.txt",
         "event_file": "events.txt", "num_track_slots": 4096, "initializer_capacity": 1 << 20,
         "secondary_stack_factor": 3.0, "use_device": True}
    d.update(kw)
    return d


def test_reads_the_stepping_keys():
    inp = RunnerInput.from_json(base(seed=7, max_steps=100, field=[0, 0, 3.8],
                                     field_options={"delta_chord": 0.01},
                                     track_order="reindex_both_action",
                                     brem_combined=True, warm_up=True, action_times=True,
                                     merge_events=True, simple_calo=["pb_0"]))
    assert inp.seed == 7 and inp.max_steps == 100
    assert inp.field == (0.0, 0.0, 3.8)
    assert inp.track_order_id == 7
    assert inp.brem_combined and inp.warm_up and inp.merge_events
    assert inp.field_options == {"delta_chord": 0.01}


def test_json_string_and_deprecated_names():
    d = base()
    d["max_num_tracks"] = d.pop("num_track_slots")
    d["geometry_filename"] = d.pop("geometry_file")
    inp = RunnerInput.from_json(json.dumps(d))
    assert inp.num_track_slots == 4096 and inp.geometry_file == "calo"
    d["num_track_slots"] = 8
    with pytest.raises(RunnerInputError, match="replacement"):
        RunnerInput.from_json(d)


@pytest.mark.parametrize("key", ["initializer_capacity", "secondary_stack_factor",
                                 "use_device", "geometry_file"])
def test_required_keys(key):
    d = base()
    del d[key]
    with pytest.raises(RunnerInputError, match="missing required"):
        RunnerInput.from_json(d)


@pytest.mark.parametrize("update, match", [
    ({"use_device": False}, "device only"),
    ({"primary_options": {"pdg": 11}}, "but not both"),
    ({"field_options": {"delta_chord": 0.1}}, "without providing 'field'"),
    ({"num_track_slots": 0}, "must be positive"),
    ({"track_order": "reindex_randomly"}, "track_order"),
    ({"track_order": "sideways"}, "unknown track order"),
    ({"step_limiter": 1.0}, "step_limiter"),
    ({"physics_options": {}}, "not supported"),
    ({"optical": {}}, "not supported"),
    ({"_format": "celer-g4"}, "format"),
    ({"no_such_key": 1}, "unknown input keys"),
])
def test_rejected_inputs(update, match):
    with pytest.raises(RunnerInputError, match=match):
        RunnerInput.from_json(base(**update))


def test_ignored_environment_keys():
    inp = RunnerInput.from_json(base(cuda_heap_size=1 << 20, environ={"A": "1"},
                                     default_stream=True))
    assert inp.num_track_slots == 4096


def test_event_file(tmp_path):
    path = tmp_path / "ev.txt"
    path.write_text("11 1000 0 0 -5 0 0 1 0 3\n22 10.5 1 2 3 0 1 0 1e-9 4\n")
    p = read_event_file(str(path))
    assert list(p["pdg"]) == [11, 22]
    assert list(p["event"]) == [3, 4]
    np.testing.assert_array_equal(p["pos"][1], [1, 2, 3])
    assert p["time"][1] == 1e-9
