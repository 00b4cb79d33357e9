"""Interactor parity against the reference (CPU, no GPU).

The fixtures hold, per input, the result of one interaction computed by the
reference's own model actions (the harness's 'interact' mode,
tests/golden/make_golden.py): each input (model, particle, energy,
position, direction, element component) is a primary that the reference's
extend-from-primaries, initialize-tracks and pre-step prepared; its
step-limit action and element component are then set as discrete selection
would set them, and only that model runs. The inputs span every model's
energy range (Klein-Nishina, Livermore photoelectric, Bethe-Heitler,
Seltzer-Berger, relativistic bremsstrahlung with LPM, Moller-Bhabha,
two-photon annihilation, combined bremsstrahlung), every element component
of the calorimeter's and the CMS-like detector's materials, and isotropic
directions.

The CPU restatement runs the GB300 path's interactor code (the same source
the device kernels compile) on the same inputs and the same random states.
The bar for interactor outputs fed the same random state is 1e-12 relative;
the FP64 code meets it bit for bit, which is what is asserted after the
tolerance check: the pre-step's results (step limit and its action, sampled
interaction MFP, macroscopic and per-process cross sections, range), then
status, step-limit action, material, outgoing energy and direction, local
deposition, every secondary (PDG, energy, direction) and the random state
after the interaction.
"""

import os

import numpy as np
import pytest

from conftest import load_golden

import oracle
from celeritas_gb300 import geometry_path, physics_file

CASES = ["interact_calo", "interact_cms", "interact_calo_brcomb"]
RTOL = 1e-12


def run(golden, libm, tmp_path):
    c = golden["case"]
    txt = os.path.join(tmp_path, "inputs.txt")
    oracle.write_interaction_inputs(txt, golden["inputs"])
    extra = ["--brem-combined"] if c["brem_combined"] else []
    return oracle.run_interactions("port", physics_file(c["geometry"]),
                                   geometry_path(c["geometry"]), txt, c["seed"],
                                   extra=extra, libm=libm)


def floats(r):
    """Every floating-point output of one interaction, flattened."""
    pre = r["pre_step"]
    out = [pre["step"], pre["mfp"], pre["macro_xs"], pre["range"], *pre["xs"]]
    out += [r["energy"], r["edep"], *r["direction"]]
    for sec in r["secondaries"]:
        out += [sec["energy"], *sec["direction"]]
    return out


@pytest.mark.parametrize("libm", oracle.LIBMS)
@pytest.mark.parametrize("name", CASES)
def test_interactors_match_reference(built_port, name, libm, tmp_path):
    golden = load_golden(name, libm)
    got = run(golden, libm, tmp_path)
    assert len(got) == len(golden["results"])
    for inp, g, r in zip(golden["inputs"], got, golden["results"]):
        where = f"{inp[0]} pdg {inp[1]} E {inp[2]} MeV element {inp[5]}"
        assert g["num_secondaries"] == r["num_secondaries"], where
        np.testing.assert_allclose(floats(g), floats(r), rtol=RTOL, atol=1e-300,
                                   err_msg=where)
        assert g == r, where


def test_inputs_cover_every_model():
    """Each model of the physics (and the combined bremsstrahlung model) has
    inputs, and each element component of the compound materials is used."""
    models = set()
    comps = set()
    for name in CASES:
        golden = load_golden(name, "pinned")
        models |= {inp[0] for inp in golden["inputs"]}
        comps |= {(golden["case"]["geometry"], r["material"], inp[5])
                  for inp, r in zip(golden["inputs"], golden["results"])}
    assert models == {"scat-klein-nishina", "photoel-livermore", "conv-bethe-heitler",
                      "brems-sb", "brems-rel", "ioni-moller-bhabha", "annihil-2-gamma",
                      "brems-combined"}
    # PbWO4 (3 components), brass and scintillator (2 each) in the CMS-like
    # detector
    for mat, n in ((2, 3), (3, 2), (4, 2)):
        assert {c for g, m, c in comps if g == "cms" and m == mat} == set(range(n))


def test_reference_conserves_energy():
    """The reference's own results conserve energy (a check of the fixtures):
    outgoing + deposited + secondaries = incoming, with the pair's rest mass
    for conversion and the positron's for annihilation."""
    electron_mass = 0.51099895  # [MeV], the physics input's (gen_physics.py)
    for name in CASES:
        golden = load_golden(name, "pinned")
        for inp, r in zip(golden["inputs"], golden["results"]):
            model, e0 = inp[0], inp[2]
            total = r["energy"] + r["edep"] + sum(s["energy"] for s in r["secondaries"])
            if model == "conv-bethe-heitler":
                total += 2 * electron_mass
            elif model == "annihil-2-gamma":
                total -= 2 * electron_mass
            assert total == pytest.approx(e0, rel=1e-9, abs=1e-9), inp


def test_check_detects_another_random_state(built_port, tmp_path):
    """The comparison is sensitive: the same inputs with the random states of
    another seed give other results for every sampled interaction."""
    golden = load_golden("interact_calo", "pinned")
    golden = dict(golden, case=dict(golden["case"], seed=golden["case"]["seed"] + 1))
    got = run(golden, "pinned", tmp_path)
    differ = [g != r for g, r in zip(got, golden["results"])]
    assert all(differ)


@pytest.mark.skipif(not (os.path.exists(oracle.REF_BIN) and os.path.exists(oracle.REF_PINNED_BIN)),
                    reason="the compiled reference is not present")
@pytest.mark.parametrize("libm", oracle.LIBMS)
def test_random_inputs_against_live_reference(built_port, libm, tmp_path):
    """Fresh inputs beyond the fixtures: 600 interactions drawn at random
    (model, log-uniform energy inside the model's range, CMS-like material
    point, element component, direction), through the compiled reference
    and the restatement."""
    rng = np.random.default_rng(24680)
    points = [((4.01, 0.0, 0.0), 1), ((140.0, 0.0, 0.0), 3), ((182.0, 0.0, 0.0), 2),
              ((185.2, 0.0, 0.0), 2)]
    models = [("scat-klein-nishina", 22, 1e-3, 1e6, False),
              ("photoel-livermore", 22, 1e-3, 10.0, False),
              ("conv-bethe-heitler", 22, 1.05, 1e5, True),
              ("brems-sb", 11, 0.1, 1000.0, True), ("brems-sb", -11, 0.1, 1000.0, True),
              ("brems-rel", 11, 1000.0, 1e6, True), ("brems-rel", -11, 1000.0, 1e6, True),
              ("ioni-moller-bhabha", 11, 3.0, 1e5, False),
              ("ioni-moller-bhabha", -11, 3.0, 1e5, False),
              ("annihil-2-gamma", -11, 1e-3, 1e5, False)]
    inputs = []
    for _ in range(600):
        model, pdg, lo, hi, by_element = models[rng.integers(len(models))]
        pos, ncomp = points[rng.integers(len(points))]
        e = float(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        v = rng.normal(size=3)
        d = [float(x) for x in v / np.linalg.norm(v)]
        elcomp = int(rng.integers(ncomp)) if by_element else 0
        inputs.append([model, pdg, e, list(pos), d, elcomp])
    txt = os.path.join(tmp_path, "inputs.txt")
    oracle.write_interaction_inputs(txt, inputs)
    args = (physics_file("cms"), geometry_path("cms"), txt, 77)
    ref = oracle.run_interactions("reference", *args, libm=libm)
    got = oracle.run_interactions("port", *args, libm=libm)
    assert len(got) == len(ref) == len(inputs)
    for inp, g, r in zip(inputs, got, ref):
        assert g == r, inp


@pytest.mark.skipif(not (os.path.exists(oracle.REF_BIN) and os.path.exists(oracle.REF_PINNED_BIN)),
                    reason="the compiled reference is not present")
@pytest.mark.parametrize("libm", oracle.LIBMS)
def test_random_combined_brems_against_live_reference(built_port, libm, tmp_path):
    """Fresh inputs for the combined bremsstrahlung model: 300 e-/e+ of
    log-uniform 50 keV-1 TeV (both sides of its 1 GeV switch) in Pb and lAr,
    random directions."""
    rng = np.random.default_rng(11235)
    inputs = []
    for _ in range(300):
        pdg = int(rng.choice([11, -11]))
        e = float(np.exp(rng.uniform(np.log(0.05), np.log(1e6))))
        pos = [(0.0, 0.0, 0.1), (0.0, 0.0, 0.5)][int(rng.integers(2))]
        v = rng.normal(size=3)
        d = [float(x) for x in v / np.linalg.norm(v)]
        inputs.append(["brems-combined", pdg, e, list(pos), d, 0])
    txt = os.path.join(tmp_path, "inputs.txt")
    oracle.write_interaction_inputs(txt, inputs)
    args = (physics_file("calo"), geometry_path("calo"), txt, 55)
    ref = oracle.run_interactions("reference", *args, extra=["--brem-combined"], libm=libm)
    got = oracle.run_interactions("port", *args, extra=["--brem-combined"], libm=libm)
    assert len(got) == len(ref) == len(inputs)
    for inp, g, r in zip(inputs, got, ref):
        assert g == r, inp
