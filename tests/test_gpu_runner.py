"""celer-sim input on the GB300 (GPU): golden transports described as
celer-sim JSON inputs, run by celeritas_gb300.runner, give the reference's
per-step track counts (the Transporter's initializers/active/alive) and its
energy deposition; primary_options generate events on the device; warm_up
and max_steps behave as celer-sim's.
"""

import json
import os

import numpy as np
import pytest

from conftest import case_primaries, load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def runner_mod(built_lib):
    import celeritas_gb300 as gb
    from celeritas_gb300 import runner

    gb.load_library(built_lib)
    return runner


def golden_input(tmp_path, name):
    from celeritas_gb300 import physics_file
    from celeritas_gb300.primaries import write_primaries_text

    golden = load_golden(name, "pinned")
    c = golden["case"]
    ev = os.path.join(tmp_path, "events.txt")
    write_primaries_text(ev, case_primaries(c))
    geometry = c.get("geometry", "calo")
    d = {"_format": "celer-sim", "geometry_file": geometry,
         "physics_file": physics_file(c.get("physics", geometry)), "event_file": ev,
         "seed": c["seed"], "num_track_slots": c["num_track_slots"],
         "initializer_capacity": 1 << 20, "secondary_stack_factor": 3,
         "use_device": True, "msc": bool(c["msc"]), "warm_up": True}
    if any(c["field"]):
        d["field"] = c["field"]
    if c.get("field_options"):
        d["field_options"] = c["field_options"]
    if c.get("brem_combined"):
        d["brem_combined"] = True
    return golden, d


@pytest.mark.parametrize("name", ["calo_e1000_n4", "cms_fieldopt_mix_e5000_n4",
                                  "calo_brcomb_e10000_n2", "slabs_e2000_n4"])
def test_golden_case_from_celer_sim_input(runner_mod, tmp_path, name):
    golden, d = golden_input(str(tmp_path), name)
    inp = runner_mod.RunnerInput.from_json(json.dumps(d))
    run = runner_mod.Runner(inp)
    out = run.run()
    ev = out["result"]["runner"]["events"][0]
    steps = [[0, q, a, al] for q, a, al in zip(ev["initializers"], ev["active"], ev["alive"])]
    ref = [[0, s[1], s[2], s[3]] for s in golden["steps"]]
    assert steps == ref
    assert ev["num_steps"] == golden["total_steps"]
    assert ev["num_step_iterations"] == golden["iterations"]
    assert ev["num_aborted"] == 0
    calo = out["result"]["simple_calo"]["energy_deposition"]
    ref_edep = np.array([golden["edep"][k] for k in calo["labels"]])
    np.testing.assert_allclose(calo["total"], ref_edep, rtol=1e-11, atol=1e-9)


def test_max_steps_aborts_like_celer_sim(runner_mod, tmp_path):
    golden, d = golden_input(str(tmp_path), "calo_e1000_n4")
    d["max_steps"] = 20
    out = runner_mod.Runner(runner_mod.RunnerInput.from_json(d)).run()
    ev = out["result"]["runner"]["events"][0]
    assert ev["num_step_iterations"] == 20
    assert ev["num_aborted"] > 0
    assert len(ev["active"]) == 20


def test_primary_options_generate_on_device(runner_mod, tmp_path):
    from celeritas_gb300 import physics_file

    d = {"_format": "celer-sim", "geometry_file": "calo", "physics_file": physics_file("calo"),
         "primary_options": {"_format": "primary-generator", "seed": 3, "pdg": [11, 22],
                             "num_events": 3, "primaries_per_event": 4, "energy": 100.0,
                             "position": [0.0, 0.0, -5.0],
                             "direction": {"distribution": "delta", "params": [0, 0, 1]}},
         "num_track_slots": 4096, "initializer_capacity": 1 << 18,
         "secondary_stack_factor": 3.0, "use_device": True, "msc": False,
         "write_step_times": False}
    out = runner_mod.Runner(runner_mod.RunnerInput.from_json(d)).run()
    events = out["result"]["runner"]["events"]
    assert len(events) == 3
    for ev in events:
        assert ev["active"][0] == 4 and ev["num_aborted"] == 0
        assert "step_times" not in ev
    per_event = np.array(out["result"]["simple_calo"]["energy_deposition"]["per_event"])
    assert per_event.shape[0] == 3 and (per_event.sum(axis=1) > 0).all()
