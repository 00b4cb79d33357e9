"""The CPU oracle against the reference's golden fixtures (no GPU).

The golden fixtures were produced by the reference's own host stepping loop
(tests/golden/make_golden.py), once linked with the host C library's
elementary functions (tests/golden/) and once with correctly rounded ones
(tests/golden/pinned/, the functions of the GB300 FP64 path). The CPU
restatement built with the same functions must reproduce each set bit for
bit: every per-step counter, the number of iterations, the total
track-steps and every per-volume energy deposition.
"""

import json
import os
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN_CASES, case_options, case_primaries, case_problem, load_golden

import oracle
from celeritas_gb300 import physics_file
from celeritas_gb300.primaries import write_primaries_text


def run_case(golden, libm="pinned"):
    c = golden["case"]
    physics, geometry = case_problem(c)
    prim = case_primaries(c)
    with tempfile.TemporaryDirectory() as tmp:
        ptxt = os.path.join(tmp, "p.txt")
        write_primaries_text(ptxt, prim)
        return oracle.run_port(physics, ptxt, c["num_track_slots"], c["seed"],
                               geometry=geometry, extra=case_options(c), libm=libm)


@pytest.mark.parametrize("libm", oracle.LIBMS)
@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_port_matches_reference(built_port, name, libm):
    golden = load_golden(name, libm)
    out = run_case(golden, libm)
    assert [list(s) for s in out["steps"]] == golden["steps"]
    assert out["total_steps"] == golden["total_steps"]
    assert out["iterations"] == golden["iterations"]
    assert out["edep"] == golden["edep"]  # bit-exact FP64


@pytest.mark.parametrize("name", GOLDEN_CASES + ["hits_calo_msc_field_e300_n1",
                                                 "hits_cms_mix_e2000_n2"])
def test_reference_counters_independent_of_libm(name):
    """The reference's own results with the host C library and with
    correctly rounded elementary functions: identical per-step counters in
    every case; total deposition equal to 1e-11 relative and per-volume
    depositions to 1e-8 (last-bit differences of the functions, carried by
    multiple scattering, move a few meV across a layer boundary)."""
    system, pinned = load_golden(name, "system"), load_golden(name, "pinned")
    assert system["steps"] == pinned["steps"]
    total = sum(system["edep"].values())
    assert sum(pinned["edep"].values()) == pytest.approx(total, rel=1e-11)
    for k, v in system["edep"].items():
        assert pinned["edep"][k] == pytest.approx(v, rel=1e-8, abs=1e-9)


FIELD_CASES = [n for n in GOLDEN_CASES if "field" in n or n.startswith("cms")]


@pytest.mark.parametrize("name", FIELD_CASES)
def test_reentrant_looping_inert_in_normal_transport(built_port, name):
    """The reentrant_looping option only changes tracks that loop and then
    hit a surface they re-enter at once; in the golden transports (fields of
    1-3.8 T, calorimeter and CMS-like) the results stay the reference's."""
    golden = load_golden(name, "pinned")
    c = golden["case"]
    physics, geometry = case_problem(c)
    prim = case_primaries(c)
    with tempfile.TemporaryDirectory() as tmp:
        ptxt = os.path.join(tmp, "p.txt")
        write_primaries_text(ptxt, prim)
        out = oracle.run_port(physics, ptxt, c["num_track_slots"], c["seed"],
                              geometry=geometry,
                              extra=case_options(c) + ["--reentrant-looping"])
    assert [list(s) for s in out["steps"]] == golden["steps"]
    assert out["edep"] == golden["edep"]


def test_reentrant_looping_ends_grazing_orbit(built_port):
    """An 18 keV electron in the CMS-like detector's vacuum just outside the
    last silicon shell, moving perpendicular to the 3.8 T field: its 0.12 mm
    orbit grazes the shell's outer cylinder every few steps, each graze is a
    reentrant boundary step (back into the vacuum), and the reference's
    looping cut, which resets its count on every non-looping step, never
    ends the track (the compiled reference agrees where it is built). With
    reentrant_looping the looping cut ends it."""
    from celeritas_gb300.primaries import PRIMARY_DTYPE

    p = np.zeros(1, dtype=PRIMARY_DTYPE)
    p["pdg"] = 11
    p["energy"] = 0.01845506951212883
    p["pos"][0] = (-108.25911568208411, 19.777196382226563, 179.9582562600299)
    d = np.array([-0.7892325346384539, -0.6140944603789887, 1.065034111781243e-43])
    p["dir"][0] = d / np.linalg.norm(d)
    base = ["--msc", "--field", "0", "0", "3.8", "--steps", "200"]
    runs = {}
    with tempfile.TemporaryDirectory() as tmp:
        ptxt = os.path.join(tmp, "p.txt")
        write_primaries_text(ptxt, p)
        for name, extra in (("reference", []), ("reentrant", ["--reentrant-looping"])):
            runs[name] = oracle.run_port(physics_file("cms"), ptxt, 256, 0, geometry="cms",
                                         extra=base + extra, libm="system")
        if os.path.exists(oracle.REF_BIN):
            runs["compiled"] = oracle.run_reference(physics_file("cms"), ptxt, 256, 0,
                                                    geometry="cms", extra=base)
    # Still alive after 200 steps with the reference's looping logic
    assert runs["reference"]["steps"][-1][3] == 1
    if "compiled" in runs:
        assert runs["compiled"]["steps"] == runs["reference"]["steps"]
    # Ended by the looping cut with the option
    assert runs["reentrant"]["steps"][-1][3] == 0
    assert runs["reentrant"]["iterations"] < 200


def test_action_labels_match_reference(built_port):
    golden = load_golden("calo_e1000_n4")
    out = run_case(golden)
    assert [out["actions"][i] for i in sorted(out["actions"])] == golden["actions"]


def test_geometry_matches_orange(built_port):
    """Surfaces and volumes built by the GB300 host code equal ORANGE's."""
    golden = load_golden("calo_geometry")
    res = subprocess.run([built_port, "geo", physics_file("calo"), "calo"],
                         capture_output=True, text=True, check=True)
    surfs, vols = [], []
    for line in res.stdout.splitlines():
        tok = line.split()
        if tok[0] == "surf":
            surfs.append((int(tok[3]), float(tok[5])))
        elif tok[0] == "volume":
            vols.append(tok[2])
    assert [(s["type"], s["position"]) for s in golden["surfaces"]] == surfs
    assert golden["volumes"] == vols


def test_energy_conservation_bound(built_port):
    """Deposited energy never exceeds the primaries' kinetic energy."""
    golden = load_golden("calo_e1000_n4")
    edep = np.array(list(golden["edep"].values()))
    assert 0 < edep.sum() <= 4 * 1000.0
    assert (edep >= 0).all()


def test_port_reseed_matches_reference(built_port):
    """Stepper::reseed: the restatement's XORWOW states after reseeding
    equal the reference's for events up to 2^40 (jumps of up to 4^31
    subsequences of 2^67 draws)."""
    with open(os.path.join(os.path.dirname(__file__), "golden", "xorwow_reseed.json")) as f:
        golden = json.load(f)
    from celeritas_gb300.primaries import pencil_beam

    with tempfile.TemporaryDirectory() as tmp:
        ptxt = os.path.join(tmp, "p.txt")
        write_primaries_text(ptxt, pencil_beam(1, energy=10.0))
        for ev, expected in golden["events"].items():
            res = subprocess.run(
                [built_port, "run", physics_file("calo"), "calo", ptxt,
                 str(golden["num_track_slots"]), str(golden["seed"]), "--reseed", ev,
                 "--dump-rng", str(golden["num_track_slots"]), "--steps", "1", "--quiet"],
                capture_output=True, text=True, check=True)
            words = {}
            for line in res.stdout.splitlines():
                tok = line.split()
                if tok and tok[0] == "rng":
                    words[int(tok[1])] = [int(t) for t in tok[2:8]]
            assert [words[i] for i in golden["slots"]] == expected, ev


HIT_CASES = ["hits_calo_msc_field_e300_n1", "hits_cms_mix_e2000_n2"]


def hit_summary(hits):
    """Per-step hit count and column sums, as the golden fixtures hold them."""
    per_step = {}
    for h in hits:
        row = per_step.setdefault(h[0], [h[0], 0] + [0] * (len(h) - 1))
        row[1] += 1
        for k, v in enumerate(h[1:]):
            row[2 + k] += v
    return [per_step[k] for k in sorted(per_step)]


@pytest.mark.parametrize("libm", oracle.LIBMS)
@pytest.mark.parametrize("name", HIT_CASES)
def test_port_hits_match_reference(built_port, name, libm):
    """Step output: every step's detector hits (the reference's
    DetectorStepOutput via its own copy_steps) are reproduced bit for bit,
    in the same order, by the restatement's has_step_hit/write_step_hit."""
    golden = load_golden(name, libm)
    c = golden["case"]
    geometry = c.get("geometry", "calo")
    prim = case_primaries(c)
    with tempfile.TemporaryDirectory() as tmp:
        ptxt = os.path.join(tmp, "p.txt")
        write_primaries_text(ptxt, prim)
        out = oracle.run_port(physics_file(geometry), ptxt, c["num_track_slots"], c["seed"],
                              geometry=geometry, extra=case_options(c) + ["--hits"],
                              libm=libm)
    assert [list(s) for s in out["steps"]] == golden["steps"]
    assert len(out["hits"]) == golden["num_hits"]
    assert out["hits"][:len(golden["records"])] == golden["records"]
    assert hit_summary(out["hits"]) == golden["per_step"]
    assert out["edep"] == golden["edep"]


def test_combined_brems_rejects_compound_materials(built_port):
    """The combined bremsstrahlung model has no per-element cross sections:
    like the reference (PhysicsParams.cc:660-668), building it for the
    CMS-like detector, whose PbWO4, brass and scintillator hold several
    elements, fails."""
    from celeritas_gb300.primaries import pencil_beam

    with tempfile.TemporaryDirectory() as tmp:
        ptxt = os.path.join(tmp, "p.txt")
        write_primaries_text(ptxt, pencil_beam(1, energy=100.0))
        res = subprocess.run([built_port, "run", physics_file("cms"), "cms", ptxt, "256", "0",
                              "--brem-combined", "--steps", "1"],
                             capture_output=True, text=True)
    assert res.returncode != 0
    assert "more than one element" in res.stderr


@pytest.mark.skipif(not (os.path.exists(oracle.REF_BIN) and os.path.exists(oracle.REF_PINNED_BIN)),
                    reason="the compiled reference is not present")
@pytest.mark.parametrize("draw", range(4))
def test_random_transports_against_live_reference(built_port, draw):
    """Fresh problems beyond the fixtures, drawn at random: geometry, track
    order, seed, slots, and the beam (CMS-like e-/e+/gamma mixtures in 3.8 T
    with MSC, or a calorimeter pencil beam with MSC and a 1 T field or
    none), transported by the compiled reference and the restatement, per
    step and per volume, with both libm variants."""
    from celeritas_gb300.primaries import eta_beam, pencil_beam

    rng = np.random.default_rng(97531 + draw)
    order = int(rng.integers(8))
    seed = int(rng.integers(1 << 20))
    slots = int(rng.choice([256, 1024, 4096]))
    energy = float(np.exp(rng.uniform(np.log(1.0), np.log(3000.0))))
    if draw % 2 == 0:
        geometry = "cms"
        pdgs = tuple(int(p) for p in rng.permutation([11, -11, 22]))
        prim = eta_beam(3, emin=energy, emax=2 * energy, pdgs=pdgs,
                        seed=int(rng.integers(1000)))
        extra = ["--msc", "--field", "0.0", "0.0", "3.8"]
    else:
        geometry = "calo"
        prim = pencil_beam(3, energy=energy, pdg=int(rng.choice([11, -11, 22])))
        extra = ["--msc"] + (["--field", "1.0", "0.0", "0.0"] if draw % 4 == 1 else [])
    extra += ["--track-order", str(order)]
    with tempfile.TemporaryDirectory() as tmp:
        ptxt = os.path.join(tmp, "p.txt")
        write_primaries_text(ptxt, prim)
        for libm in oracle.LIBMS:
            ref = oracle.run_reference(physics_file(geometry), ptxt, slots, seed,
                                       geometry=geometry, extra=extra, libm=libm)
            got = oracle.run_port(physics_file(geometry), ptxt, slots, seed,
                                  geometry=geometry, extra=extra, libm=libm)
            assert got["steps"] == ref["steps"], (libm, order, seed, energy)
            assert got["total_steps"] == ref["total_steps"]
            assert got["edep"] == ref["edep"]
