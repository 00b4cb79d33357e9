"""Along-step parity against the reference (CPU, no GPU).

The fixtures hold, per input, the track after one along-step computed by the
reference's own actions (the harness's 'along' mode,
tests/golden/make_golden.py): each input (particle, energy, position,
direction) is a primary of its own event, and the reference runs
extend-from-primaries, initialize-tracks, pre-step, step-gather-pre and the
along-step action (Urban multiple scattering, uniform-field Runge-Kutta
propagation with boundary search, energy loss with fluctuations). The inputs
place e-/e+ of 10 keV to 100 GeV and photons in every material of the
calorimeter and of the CMS-like detector (3.8 T), at points just inside
boundaries too, with isotropic directions; the steps end on every kind of
limit (range, multiple scattering, boundary, discrete interaction,
propagation limit in the field).

After the along-step the reference runs physics-discrete-select, which for
steps ended by the discrete-interaction limit samples the process, applies
the integral-approach rejection and selects the model and element component.

The CPU restatement runs the GB300 path's along-step and selection code (the
source the device kernels compile) on the same inputs and must give, bit
for bit, the step limit's action, the selected action and element, step
length, position, direction, energy, local deposition, status and random
state.
"""

import os

import pytest

from conftest import load_golden

import oracle
from celeritas_gb300 import geometry_path, physics_file

CASES = ["along_cms_msc_field", "along_calo_msc", "along_calo_msc_field"]


def run(golden, libm, tmp_path):
    c = golden["case"]
    txt = os.path.join(tmp_path, "inputs.txt")
    oracle.write_interaction_inputs(txt, golden["inputs"])
    extra = (["--msc"] if c["msc"] else []) + (
        ["--field"] + [repr(float(f)) for f in c["field"]] if any(c["field"]) else [])
    return oracle.run_interactions("port", physics_file(c["geometry"]),
                                   geometry_path(c["geometry"]), txt, c["seed"],
                                   extra=extra, libm=libm, mode="along")


@pytest.mark.parametrize("libm", oracle.LIBMS)
@pytest.mark.parametrize("name", CASES)
def test_along_step_matches_reference(built_port, name, libm, tmp_path):
    golden = load_golden(name, libm)
    got = run(golden, libm, tmp_path)
    assert len(got) == len(golden["results"])
    for inp, g, r in zip(golden["inputs"], got, golden["results"]):
        assert g == r, f"pdg {inp[1]} E {inp[2]} MeV at {inp[3]} along {inp[4]}"


def test_steps_end_on_every_kind_of_limit():
    """The inputs exercise every step limit of the along-step, and discrete
    selection picks every model and the integral-approach rejection."""
    actions = set()
    selected = set()
    for name in CASES:
        golden = load_golden(name, "pinned")
        ref_actions = load_golden("cms_mix_e10000_n4" if "cms" in name
                                  else "calo_msc_field_e5000_n2", "pinned")["actions"]
        actions |= {ref_actions[r["action"]] for r in golden["results"]}
        selected |= {ref_actions[r["selected"]] for r in golden["results"]
                     if ref_actions[r["action"]] == "physics-discrete-select"}
    assert {"eloss-range", "msc-range", "geo-boundary", "physics-discrete-select",
            "geo-propagation-limit"} <= actions
    assert selected == {"physics-integral-rejected", "ioni-moller-bhabha", "brems-sb",
                        "brems-rel", "photoel-livermore", "scat-klein-nishina",
                        "conv-bethe-heitler", "annihil-2-gamma"}


@pytest.mark.skipif(not (os.path.exists(oracle.REF_BIN) and os.path.exists(oracle.REF_PINNED_BIN)),
                    reason="the compiled reference is not present")
@pytest.mark.parametrize("libm", oracle.LIBMS)
def test_random_inputs_against_live_reference(built_port, libm, tmp_path):
    """Fresh inputs beyond the fixtures: 500 along-steps (and discrete
    selections) of e-, e+ and photons, log-uniform 1 keV-100 GeV, at random
    points of the CMS-like detector (radius 0-300 cm, |z| < 320 cm) in 3.8 T
    with MSC, through the compiled reference and the restatement."""
    import numpy as np

    rng = np.random.default_rng(13579)
    inputs = []
    for _ in range(500):
        pdg = int(rng.choice([11, -11, 22]))
        e = float(np.exp(rng.uniform(np.log(1e-3), np.log(1e5))))
        r = float(rng.uniform(0.0, 300.0))
        phi = float(rng.uniform(0.0, 2 * np.pi))
        pos = [r * float(np.cos(phi)), r * float(np.sin(phi)), float(rng.uniform(-320, 320))]
        v = rng.normal(size=3)
        d = [float(x) for x in v / np.linalg.norm(v)]
        inputs.append(["-", pdg, e, pos, d, 0])
    txt = os.path.join(tmp_path, "inputs.txt")
    oracle.write_interaction_inputs(txt, inputs)
    args = (physics_file("cms"), geometry_path("cms"), txt, 88)
    extra = ["--msc", "--field", "0.0", "0.0", "3.8"]
    ref = oracle.run_interactions("reference", *args, extra=extra, libm=libm, mode="along")
    got = oracle.run_interactions("port", *args, extra=extra, libm=libm, mode="along")
    assert len(got) == len(ref) == len(inputs)
    for inp, g, r in zip(inputs, got, ref):
        assert g == r, inp


@pytest.mark.skipif(not (os.path.exists(oracle.REF_BIN) and os.path.exists(oracle.REF_PINNED_BIN)),
                    reason="the compiled reference is not present")
@pytest.mark.parametrize("libm", oracle.LIBMS)
def test_random_calorimeter_inputs_against_live_reference(built_port, libm, tmp_path):
    """Fresh inputs in the calorimeter (1 T along x, MSC): 400 along-steps of
    e-, e+ and photons, log-uniform 1 keV-10 GeV, at random depths in the
    first 20 layers and random transverse points, random directions."""
    import numpy as np

    rng = np.random.default_rng(86420)
    inputs = []
    for _ in range(400):
        pdg = int(rng.choice([11, -11, 22]))
        e = float(np.exp(rng.uniform(np.log(1e-3), np.log(1e4))))
        pos = [float(rng.uniform(-19, 19)), float(rng.uniform(-19, 19)),
               float(rng.uniform(0.0, 16.0))]
        v = rng.normal(size=3)
        d = [float(x) for x in v / np.linalg.norm(v)]
        inputs.append(["-", pdg, e, pos, d, 0])
    txt = os.path.join(tmp_path, "inputs.txt")
    oracle.write_interaction_inputs(txt, inputs)
    args = (physics_file("calo"), geometry_path("calo"), txt, 99)
    extra = ["--msc", "--field", "1.0", "0.0", "0.0"]
    ref = oracle.run_interactions("reference", *args, extra=extra, libm=libm, mode="along")
    got = oracle.run_interactions("port", *args, extra=extra, libm=libm, mode="along")
    assert len(got) == len(ref) == len(inputs)
    for inp, g, r in zip(inputs, got, ref):
        assert g == r, inp
