"""Primary generation on the device (PrimaryGenerator with
PrimaryGeneratorOptions) through the C ABI (GB300)."""

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

# TrackInitializer of the FP64 build (gbx/Data.hh)
INIT_DTYPE = np.dtype({"names": ["track_id", "parent_id", "event_id", "time", "pos", "dir",
                                 "particle_id", "energy", "rng_key"],
                       "formats": ["<u4", "<u4", "<u4", "<f8", ("<f8", 3), ("<f8", 3), "<u4",
                                   "<f8", "<u8"],
                       "offsets": [0, 4, 8, 16, 24, 48, 72, 80, 88], "itemsize": 96})


@pytest.fixture(scope="module")
def gb(built_lib):
    import celeritas_gb300 as gb

    gb.load_library(built_lib)
    return gb


@pytest.fixture(scope="module")
def calo(gb):
    return gb.Params(gb.physics_file("calo"), "calo")


def splitmix(state):
    state = (state + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
    z = state
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
    return z ^ (z >> 31)


def stream_key(seed, event, index):
    """The per-track stream key of primary 'index' of an event."""
    first = splitmix((seed << 32) | event)
    return splitmix((first + 0x9E3779B97F4A7C15 * (index + 1)) & 0xFFFFFFFFFFFFFFFF)


def test_delta_primaries_transport_as_inserted(gb, calo):
    """A delta-distributed pencil beam generated on the device is the
    golden case's beam: the transport matches the reference bit for bit."""
    golden = load_golden("calo_e1000_n4")
    c = golden["case"]
    st = gb.Stepper(calo, c["num_track_slots"], seed=c["seed"])
    st.generate_primaries(pdg=11, energy=c["energy"], position=("delta", (0, 0, c["z0"])),
                          direction=("delta", (0, 0, 1)), num_events=1,
                          primaries_per_event=c["num_primaries"])
    res = [st.step()] + st.run(max_steps=100000)
    assert [[r.generated, r.queued, r.active, r.alive] for r in res] == golden["steps"]
    edep = st.energy_deposition()
    ref = np.array([golden["edep"][k] for k in calo.detector_labels()])
    np.testing.assert_allclose(edep, ref, rtol=1e-9, atol=1e-9)


def test_box_and_isotropic_distributions(gb, calo):
    st = gb.Stepper(calo, 1 << 16, seed=3)
    lo, hi = np.array([-2.0, -1.0, -9.0]), np.array([2.0, 3.0, -5.0])
    events, per_event = 100, 600
    st.generate_primaries(pdg=[11, 22, -11], energy=250.0,
                          position=("box", tuple(lo) + tuple(hi)),
                          direction=("isotropic", ()), num_events=events,
                          primaries_per_event=per_event, first_event=7, seed=42)
    n = events * per_event
    prim = st.get_state("primaries", np.uint8).view(INIT_DTYPE)[:n]
    idx = np.arange(n)
    # Particles cycle over each event's primaries; events in order; time 0
    np.testing.assert_array_equal(prim["particle_id"], np.array([0, 2, 1])[(idx % per_event) % 3])
    np.testing.assert_array_equal(prim["event_id"], 7 + idx // per_event)
    assert (prim["energy"] == 250.0).all() and (prim["time"] == 0).all()
    # Box: inside, uniform (mean and variance of each coordinate)
    pos = prim["pos"]
    assert ((pos >= lo) & (pos < hi)).all()
    width = hi - lo
    sigma_mean = width / np.sqrt(12 * n)
    assert (np.abs(pos.mean(axis=0) - (lo + hi) / 2) < 5 * sigma_mean).all()
    np.testing.assert_allclose(pos.var(axis=0), width**2 / 12, rtol=0.03)
    # Isotropic: unit vectors, zero mean, <u_i^2> = 1/3, cos(theta) uniform
    d = prim["dir"]
    np.testing.assert_allclose(np.linalg.norm(d, axis=1), 1.0, atol=1e-12)
    assert (np.abs(d.mean(axis=0)) < 5 / np.sqrt(3 * n)).all()
    np.testing.assert_allclose((d**2).mean(axis=0), 1 / 3, atol=0.01)
    counts, _ = np.histogram(d[:, 2], bins=10, range=(-1, 1))
    chi2 = ((counts - n / 10) ** 2 / (n / 10)).sum()
    assert chi2 < 30  # 9 degrees of freedom: p ~ 4e-4
    # Per-track stream keys as for primaries inserted from the host
    for i in (0, 1, per_event, n - 1):
        assert int(prim["rng_key"][i]) == stream_key(3, 7 + i // per_event, i % per_event)


def test_invalid_options_rejected(gb, calo):
    st = gb.Stepper(calo, 1024, seed=0)
    with pytest.raises(gb.GbxError, match="invalid distribution type 'isotropic' for energy"):
        st.generate_primaries(pdg=11, energy=("isotropic", ()))
    with pytest.raises(gb.GbxError, match="invalid distribution type 'box' for direction"):
        st.generate_primaries(pdg=11, energy=10.0, direction=("box", (0,) * 6))
    with pytest.raises(gb.GbxError, match="no particle with PDG code 2212"):
        st.generate_primaries(pdg=2212, energy=10.0)
    st.generate_primaries(pdg=11, energy=10.0, num_events=2)
    st.step()
    with pytest.raises(gb.GbxError, match="event 1 already has primaries"):
        st.generate_primaries(pdg=11, energy=10.0, first_event=1)
