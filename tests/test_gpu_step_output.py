"""Step output (detector hits, StepCollector + DetectorSteps) on the GB300,
through the C ABI, against the reference's own DetectorStepOutput
(tests/golden/hits_*.json, from the reference harness's copy_steps).

The hits of the FP64 build agree with the reference's on the calorimeter and
on the CMS-like detector: the same number per step, in the same slot order,
integers exact. Floating-point data are bit-exact against the reference
linked with correctly rounded elementary functions (tests/golden/pinned/,
the functions the device uses) and agree to 1e-9 relative with the
unmodified reference, whose host C library rounds some exp/log/sin/cos
results differently in the last bit (multiple scattering carries that into
positions and depositions). Track and parent IDs are left out: on a device,
secondaries take their event's next track ID by an atomic add in whatever
order the threads arrive, in the reference's device build as here
(make_track_id, src/celeritas/track/detail/Utils.hh:108-116); only a serial
host loop numbers them in slot order.
"""

import numpy as np
import pytest

from conftest import case_primaries, load_golden

pytestmark = pytest.mark.gpu

# Against the unmodified reference (host C library)
FLOAT_RTOL = 1e-9
# Per-step column sums over the whole shower: the last-bit libm differences
# grow through ~90 multiple-scattering deflections to ~2e-9 in a direction
# component
SUM_RTOL, SUM_ATOL = 1e-7, 1e-8
# Integer columns compared: step, detector, event, track step count, particle
# (not track_id = 2 and parent_id = 4, numbered in thread order on a device)
INT_COLS = [0, 1, 3, 5, 6]


@pytest.fixture(scope="module")
def gb(built_lib):
    import celeritas_gb300 as gb

    gb.load_library(built_lib)
    return gb


def transport_with_hits(gb, case, precision="double", capacity=1 << 16, **output):
    geometry = case.get("geometry", "calo")
    params = gb.Params(gb.physics_file(geometry), geometry,
                       field_tesla=tuple(case.get("field", [0, 0, 0])),
                       msc=bool(case.get("msc")), precision=precision)
    st = gb.Stepper(params, case["num_track_slots"], seed=case["seed"])
    st.set_step_output(capacity=capacity, **output)
    res = [st.step(case_primaries(case))] + st.run(max_steps=100000, batch=32)
    return st, res, st.read_step_output()


def hit_rows(hits):
    """Hits as rows in the column order of the golden fixtures."""
    n = len(hits["step"])
    cols = [hits[k].astype(np.float64) for k in
            ("step", "detector", "track_id", "event_id", "parent_id", "track_step_count",
             "particle", "step_length", "energy_deposition", "pre_time")]
    cols += [hits["pre_pos"][:, k] for k in range(3)]
    cols += [hits["pre_dir"][:, k] for k in range(3)]
    cols += [hits["pre_energy"], hits["post_time"]]
    cols += [hits["post_pos"][:, k] for k in range(3)]
    cols += [hits["post_dir"][:, k] for k in range(3)]
    cols += [hits["post_energy"]]
    return np.stack(cols, axis=1) if n else np.zeros((0, 25))


def per_step(rows):
    steps = np.unique(rows[:, 0]).astype(int)
    out = np.zeros((len(steps), rows.shape[1] + 1))
    for i, s in enumerate(steps):
        sel = rows[rows[:, 0] == s]
        out[i, 0] = s
        out[i, 1] = len(sel)
        out[i, 2:] = sel[:, 1:].sum(axis=0)
    return out


@pytest.mark.parametrize("libm", ["pinned", "system"])
@pytest.mark.parametrize("name", ["hits_calo_msc_field_e300_n1", "hits_cms_mix_e2000_n2"])
def test_hits_match_reference(gb, name, libm):
    golden = load_golden(name, libm)
    st, res, hits = transport_with_hits(gb, golden["case"])
    assert [[r.generated, r.queued, r.active, r.alive] for r in res] == golden["steps"]
    rows = hit_rows(hits)
    assert len(rows) == golden["num_hits"]
    ref = np.array(golden["records"])
    got = rows[:len(ref)]
    np.testing.assert_array_equal(got[:, INT_COLS], ref[:, INT_COLS])
    if libm == "pinned":
        np.testing.assert_array_equal(got[:, 7:], ref[:, 7:])
    else:
        np.testing.assert_allclose(got[:, 7:], ref[:, 7:], rtol=FLOAT_RTOL, atol=1e-12)
    # Track IDs: the first hits are the primary's (ID 0, no parent)
    assert got[0, 2] == ref[0, 2] == 0
    ps, ref_ps = per_step(rows), np.array(golden["per_step"], dtype=np.float64)
    np.testing.assert_array_equal(ps[:, :2], ref_ps[:, :2])  # hits per step
    sums = [1 + c for c in INT_COLS[1:]] + list(range(8, ps.shape[1]))
    if libm == "pinned":
        # The same records, summed here and there in possibly different orders
        np.testing.assert_allclose(ps[:, sums], ref_ps[:, sums], rtol=1e-13, atol=1e-13)
    else:
        np.testing.assert_allclose(ps[:, sums], ref_ps[:, sums], rtol=SUM_RTOL, atol=SUM_ATOL)


@pytest.mark.parametrize("precision", ["double", "mixed"])
def test_hits_add_up_to_the_tally(gb, precision):
    """Summed per detector, the hits' depositions are the SimpleCalo tally
    (both keep the steps with a deposition in a detector volume)."""
    golden = load_golden("hits_cms_mix_e2000_n2")
    st, res, hits = transport_with_hits(gb, golden["case"], precision=precision,
                                        selection=["energy_deposition"])
    assert set(hits) == {"step", "detector", "track_id", "energy_deposition"}
    tally = st.energy_deposition()
    from_hits = np.bincount(hits["detector"], weights=hits["energy_deposition"],
                            minlength=len(tally))
    np.testing.assert_allclose(from_hits, tally, rtol=1e-12, atol=1e-9)
    assert (hits["energy_deposition"] > 0).all()
    # Steps in order, records of a step in slot order: step indices never
    # decrease
    assert (np.diff(hits["step"].astype(np.int64)) >= 0).all()


def test_overflow_is_reported_and_recovers(gb):
    from celeritas_gb300.primaries import pencil_beam

    # No field: the electrons reach the calorimeter from z = -5 cm
    params = gb.Params(gb.physics_file("calo"), "calo")
    st = gb.Stepper(params, 1024, seed=4)
    st.set_step_output(capacity=16)
    st.step(pencil_beam(1, energy=300.0))
    st.run(max_steps=100000, batch=32)
    with pytest.raises(gb.GbxError, match="overflowed"):
        st.read_step_output()
    # Emptied after the report
    assert len(st.read_step_output()["step"]) == 0
    # Later steps record again: a 10 MeV electron, read after every step
    recorded = 0
    res = st.step(pencil_beam(1, energy=10.0))
    while res.alive or res.queued:
        recorded += len(st.read_step_output()["step"])
        res = st.step()
    recorded += len(st.read_step_output()["step"])
    assert recorded > 0
    st.set_step_output(capacity=0)
    with pytest.raises(gb.GbxError, match="not enabled"):
        st.read_step_output()
