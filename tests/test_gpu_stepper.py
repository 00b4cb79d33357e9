"""GPU stepping loop against the reference's golden fixtures (GB300).

Every case is transported on the device through the C ABI and compared with
the reference's own host stepping loop on the same inputs, for both sets of
fixtures: the reference linked with correctly rounded elementary functions
(the ones the FP64 device code uses, tests/golden/pinned/) and the
unmodified reference with the host C library's (tests/golden/). Per-step
track counters (generated, queued, active, alive), the number of iterations
and the total track-steps are bit-exact in every case, calorimeter and
CMS-like. The total deposited energy agrees to 1e-12 relative (the device
tally adds per-slot deposits with atomics, so the summation order differs
from the reference's slot-ordered sum); per-volume depositions agree to
1e-11 with the pinned fixtures (summation order only) and to 1e-8 with the
host library's (whose last-bit differences, carried by multiple scattering,
move a few meV across a layer boundary).
"""

import numpy as np
import pytest

from conftest import GOLDEN_CASES, case_primaries, load_golden

pytestmark = pytest.mark.gpu

EDEP_RTOL = 1e-8
TOTAL_RTOL = 1e-12


@pytest.fixture(scope="module")
def gb(built_lib):
    import celeritas_gb300 as gb

    gb.load_library(built_lib)
    return gb


@pytest.fixture(scope="module")
def calo_params(gb):
    return gb.Params(gb.physics_file("calo"), "calo")


_PARAMS = {}


def params_for(gb, case):
    """Params with the case's field and MSC options (cached per options)."""
    geometry = case.get("geometry", "calo")
    physics = case.get("physics", geometry)
    key = (geometry, tuple(case.get("field", [0, 0, 0])), bool(case.get("msc")),
           int(case.get("track_order", 0)), bool(case.get("rz_field")),
           bool(case.get("brem_combined")),
           tuple(sorted((case.get("field_options") or {}).items())))
    if key not in _PARAMS:
        _PARAMS[key] = gb.Params(gb.physics_file(physics), geometry,
                                 field_tesla=key[1], msc=key[2], track_order=key[3],
                                 rz_field=gb.field_map_file(geometry) if key[4] else None,
                                 brem_combined=key[5], field_options=dict(key[6]))
    return _PARAMS[key]


def transport(gb, params, case, use_graph=True, batch=32):
    prim = case_primaries(case)
    st = gb.Stepper(params, case["num_track_slots"], seed=case["seed"], use_graph=use_graph)
    if case.get("reseed") is not None:
        st.reseed(case["reseed"])
    res = [st.step(prim)] + st.run(max_steps=100000, batch=batch)
    return st, res


EDEP_RTOL_PINNED = 1e-11


@pytest.mark.parametrize("libm", ["pinned", "system"])
@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_matches_reference(gb, name, libm):
    golden = load_golden(name, libm)
    params = params_for(gb, golden["case"])
    st, res = transport(gb, params, golden["case"])
    steps = [[r.generated, r.queued, r.active, r.alive] for r in res]
    assert params.action_labels() == golden["actions"]
    labels = params.detector_labels()
    edep = st.energy_deposition()
    ref = np.array([golden["edep"][k] for k in labels])
    assert steps == golden["steps"]
    assert len(res) == golden["iterations"]
    assert sum(r.active for r in res) == golden["total_steps"]
    np.testing.assert_allclose(edep.sum(), ref.sum(), rtol=TOTAL_RTOL)
    rtol = EDEP_RTOL_PINNED if libm == "pinned" else EDEP_RTOL
    np.testing.assert_allclose(edep, ref, rtol=rtol, atol=1e-9)


def test_action_labels(calo_params):
    golden = load_golden("calo_e1000_n4")
    assert calo_params.action_labels() == golden["actions"]


def test_graph_replay_equals_eager(gb, calo_params):
    case = load_golden("calo_g100_n16")["case"]
    st_g, res_g = transport(gb, calo_params, case, use_graph=True, batch=7)
    st_e, res_e = transport(gb, calo_params, case, use_graph=False, batch=1)
    assert res_g == res_e
    np.testing.assert_allclose(st_g.energy_deposition(), st_e.energy_deposition(),
                               rtol=EDEP_RTOL)


def test_action_times_cover_all_kernels(gb, calo_params):
    case = load_golden("calo_ep500_n4")["case"]
    from celeritas_gb300.primaries import pencil_beam

    st = gb.Stepper(calo_params, case["num_track_slots"], seed=case["seed"])
    st.set_action_times(True)
    prim = pencil_beam(4, energy=500.0, pdg=-11)
    res = [st.step(prim)] + st.run(max_steps=10000)
    ms, launches = st.action_times()
    labels = calo_params.action_labels()
    # run() launches whole batches: steps after the state empties are no-ops
    assert len(res) <= launches[labels.index("pre-step")] < len(res) + 32
    assert ms[labels.index("along-step-general-linear")] > 0
    assert launches[labels.index("msc-range")] == 0  # implicit action
    golden = load_golden("calo_ep500_n4")
    assert [[r.generated, r.queued, r.active, r.alive] for r in res] == golden["steps"]


def test_kill_active(gb, calo_params):
    from celeritas_gb300.primaries import pencil_beam

    st = gb.Stepper(calo_params, 4096, seed=0)
    st.step(pencil_beam(4, energy=1000.0))
    for _ in range(20):
        st.step()
    st.kill_active()
    res = st.step()
    # Killed tracks are cut this step; remaining work is queued secondaries
    assert res.active > 0
    total = st.energy_deposition().sum()
    assert 0 < total <= 4000.0 + 1e-9


def test_consecutive_insertions_rejected(gb, calo_params):
    from celeritas_gb300.primaries import pencil_beam

    st = gb.Stepper(calo_params, 1024, seed=0)
    st.insert_primaries(pencil_beam(1))
    with pytest.raises(gb.GbxError, match="consecutive"):
        st.insert_primaries(pencil_beam(1))


def test_state_roundtrip(gb, calo_params):
    st = gb.Stepper(calo_params, 256, seed=5)
    rng = st.get_state("rng", np.uint32)
    assert rng.size == 6 * 256
    st.set_state("energy", np.full(256, 3.0))
    assert (st.get_state("energy", np.float64) == 3.0).all()
    with pytest.raises(gb.GbxError, match="unknown state field"):
        st.get_state("nope", np.uint8)


def test_reseed_states_match_reference(gb, calo_params):
    """gbx_stepper_reseed gives every slot the reference's reseeded XORWOW
    state (tests/golden/xorwow_reseed.json, from Stepper<host>::reseed)."""
    import json
    import os

    with open(os.path.join(os.path.dirname(__file__), "golden", "xorwow_reseed.json")) as f:
        golden = json.load(f)
    n = golden["num_track_slots"]
    st = gb.Stepper(calo_params, n, seed=golden["seed"], use_graph=False)
    for ev, expected in golden["events"].items():
        st.reseed(int(ev))
        words = st.get_state("rng", np.uint32).reshape(6, n)
        got = [[int(words[w, i]) for w in range(6)] for i in golden["slots"]]
        assert got == expected, ev


def test_reseed_restarts_event(gb, calo_params):
    """Reseeding for the same event reproduces a transport exactly; another
    event gives another history."""
    from celeritas_gb300.primaries import pencil_beam

    prim = pencil_beam(4, energy=1000.0)
    st = gb.Stepper(calo_params, 4096, seed=3)
    results = []
    for ev in (5, 5, 6):
        st.reseed(ev)
        st.clear_energy_deposition()
        res = [st.step(prim)] + st.run(max_steps=100000)
        results.append(([[r.generated, r.queued, r.active, r.alive] for r in res],
                        st.energy_deposition()))
    assert results[0][0] == results[1][0]
    np.testing.assert_allclose(results[0][1], results[1][1], rtol=1e-12)
    assert results[0][0] != results[2][0]


@pytest.mark.parametrize("precision", ["double", "mixed"])
def test_reentrant_looping_ends_grazing_orbit(gb, precision):
    """The grazing vacuum orbit of tests/test_oracle.py on the device: with
    reentrant_looping the looping cut ends the track within 200 steps."""
    from celeritas_gb300.primaries import PRIMARY_DTYPE

    p = np.zeros(1, dtype=PRIMARY_DTYPE)
    p["pdg"] = 11
    p["energy"] = 0.01845506951212883
    p["pos"][0] = (-108.25911568208411, 19.777196382226563, 179.9582562600299)
    d = np.array([-0.7892325346384539, -0.6140944603789887, 1.065034111781243e-43])
    p["dir"][0] = d / np.linalg.norm(d)
    params = gb.Params(gb.physics_file("cms"), "cms", field_tesla=(0.0, 0.0, 3.8), msc=True,
                       precision=precision, reentrant_looping=True)
    st = gb.Stepper(params, 256, seed=0)
    res = [st.step(p)] + st.run(max_steps=199)
    assert res[-1].alive == 0 and res[-1].queued == 0
    assert len(res) < 200


def test_rzmap_mixed_build(gb):
    """The R-Z map in the mixed-precision build (FP64 integration where the
    field depends on position): the golden transport's total deposition
    within the CMS-like tolerance."""
    golden = load_golden("cms_rzmap_mix_e2000_n4")
    c = golden["case"]
    params = gb.Params(gb.physics_file("cms"), "cms", msc=True, precision="mixed",
                       rz_field=gb.field_map_file("cms"), reentrant_looping=True)
    assert "along-step-rzmap-msc" in params.action_labels()
    st = gb.Stepper(params, c["num_track_slots"], seed=c["seed"])
    res = [st.step(case_primaries(c))] + st.run(max_steps=100000)
    assert res[-1].alive == 0 and res[-1].queued == 0
    ref = sum(golden["edep"].values())
    # Independent FP32 physics: the total within 2% on this small case
    np.testing.assert_allclose(st.energy_deposition().sum(), ref, rtol=0.02)


def test_combined_brems_rejects_compound_materials(gb):
    with pytest.raises(gb.GbxError, match="more than one element"):
        gb.Params(gb.physics_file("cms"), "cms", brem_combined=True)
    params = gb.Params(gb.physics_file("calo"), "calo", brem_combined=True)
    labels = params.action_labels()
    assert "brems-combined" in labels and "brems-sb" not in labels
