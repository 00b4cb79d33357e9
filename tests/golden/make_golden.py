"""Generate the golden fixtures of the stepping loop from the reference.

Runs the reference's own host stepping loop (oracle/ref, compiled from the
reference sources) on the committed synthetic physics input and records,
per case: the ordered action labels, the per-step StepperResult counters
(generated, queued, active, alive), the total track-steps and the energy
deposition per calorimeter volume; for the hit cases, the reference's
DetectorStepOutput of every step (the first records in full, per-step counts
and column sums). Also records the ORANGE surface data of the calorimeter
geometry and reseeded XORWOW states.

Also records, per interaction case, one interaction per input through the
reference's own model actions (the harness's 'interact' mode), and per
along-step case one along-step per input (its 'along' mode).

Usage (where the reference sources are present):
    python tests/golden/make_golden.py [--reference /path/to/reference]
    python tests/golden/make_golden.py --libm pinned   # fixtures under pinned/
    python tests/golden/make_golden.py --cases --hit-cases --interactions interact_cms
    python tests/golden/make_golden.py --cases --hit-cases --interactions --along

With --libm pinned the reference runs with correctly rounded exp, log, sin,
cos, tanh, log1p, expm1 and cbrt (oracle/ref/pinned_libm.cc), the elementary
functions of the GB300 build's FP64 path.
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

import oracle  # noqa: E402
from celeritas_gb300 import field_map_file, geometry_path, physics_file  # noqa: E402
from celeritas_gb300.primaries import eta_beam, pencil_beam, write_primaries_text  # noqa: E402

# name: primaries (pdg, energy [MeV], count), track slots, seed, msc, field [T]
CASES = {
    "calo_e1000_n4": dict(pdg=11, energy=1000.0, num=4, slots=65536, seed=0),
    "calo_e1000_n4_slots512": dict(pdg=11, energy=1000.0, num=4, slots=512, seed=0),
    "calo_g100_n16": dict(pdg=22, energy=100.0, num=16, slots=4096, seed=7),
    "calo_ep500_n4": dict(pdg=-11, energy=500.0, num=4, slots=4096, seed=3),
    "calo_e1000_n100": dict(pdg=11, energy=1000.0, num=100, slots=65536, seed=0),
    "calo_e10000_n2": dict(pdg=11, energy=10000.0, num=2, slots=65536, seed=0),
    "calo_msc_e1000_n4": dict(pdg=11, energy=1000.0, num=4, slots=65536, seed=0, msc=True),
    "calo_field_e1000_n4": dict(pdg=11, energy=1000.0, num=4, slots=65536, seed=0,
                                field=[1.0, 0.0, 0.0]),
    "calo_msc_field_e5000_n2": dict(pdg=11, energy=5000.0, num=2, slots=65536, seed=11,
                                    msc=True, field=[1.0, 0.0, 0.0]),
    "calo_msc_field_ep2000_n2": dict(pdg=-11, energy=2000.0, num=2, slots=8192, seed=5,
                                     msc=True, field=[1.0, 0.0, 0.0]),
    # Action-sorted track orders (TrackOrder 5, 6, 7)
    "calo_sorted_both_e1000_n4": dict(pdg=11, energy=1000.0, num=4, slots=65536, seed=0,
                                      track_order=7),
    "calo_sorted_post_g100_n16": dict(pdg=22, energy=100.0, num=16, slots=4096, seed=7,
                                      track_order=6),
    "calo_msc_field_sorted_along_e2000_n2": dict(pdg=11, energy=2000.0, num=2, slots=65536,
                                                 seed=3, msc=True, field=[1.0, 0.0, 0.0],
                                                 track_order=5),
    # CMS-like detector: shells about z, 3.8 T along z, Urban MSC; e-/gamma
    # from the origin, uniform in |eta| < 1.5
    "cms_mix_e10000_n4": dict(geometry="cms", beam="eta", pdgs=[11, 22], energy=10000.0,
                              num=4, slots=65536, seed=0, beam_seed=1, msc=True,
                              field=[0.0, 0.0, 3.8]),
    "cms_mix_logu_n6": dict(geometry="cms", beam="eta", pdgs=[22, 11], energy=1000.0,
                            emax=30000.0, num=6, slots=65536, seed=4, beam_seed=2, msc=True,
                            field=[0.0, 0.0, 3.8]),
    "cms_sorted_both_mix_e5000_n4": dict(geometry="cms", beam="eta", pdgs=[11, 22],
                                         energy=5000.0, num=4, slots=16384, seed=9,
                                         beam_seed=3, msc=True, field=[0.0, 0.0, 3.8],
                                         track_order=7),
    # R-Z field map (along-step-rzmap-msc) of the CMS-like detector
    "cms_rzmap_mix_e2000_n4": dict(geometry="cms", beam="eta", pdgs=[11, 22], energy=2000.0,
                                   num=4, slots=4096, seed=3, beam_seed=8, msc=True,
                                   rz_field=True),
    # Combined bremsstrahlung model (RunnerInput::brem_combined): SB below
    # 1 GeV, relativistic with LPM above, one "brems-combined" action
    "calo_brcomb_e10000_n2": dict(pdg=11, energy=10000.0, num=2, slots=65536, seed=1,
                                  brem_combined=True),
    "calo_brcomb_msc_field_ep3000_n2": dict(pdg=-11, energy=3000.0, num=2, slots=16384,
                                            seed=6, msc=True, field=[1.0, 0.0, 0.0],
                                            brem_combined=True),
    "calo_brcomb_sorted_both_e2000_n4": dict(pdg=11, energy=2000.0, num=4, slots=65536,
                                             seed=2, track_order=7, brem_combined=True),
    # Field-driver options other than the defaults (RunnerInput's
    # field_options, FieldDriverOptions members in native units)
    "cms_fieldopt_mix_e5000_n4": dict(geometry="cms", beam="eta", pdgs=[11, 22],
                                      energy=5000.0, num=4, slots=16384, seed=12, beam_seed=9,
                                      msc=True, field=[0.0, 0.0, 3.8],
                                      field_options={"delta_chord": 0.01, "max_substeps": 20,
                                                     "epsilon_step": 1e-6, "safety": 0.8}),
    # Geometries read from files (celeritas_gb300/data/*.geo): boxes of
    # different sizes with a gap, and shells about z not centred on z = 0
    "slabs_e2000_n4": dict(geometry="slabs.geo", physics="calo", pdg=11, energy=2000.0,
                           num=4, slots=16384, seed=3, msc=True, z0=-10.0),
    "tracker_mix_e3000_n4": dict(geometry="tracker.geo", physics="cms", beam="eta",
                                 pdgs=[11, 22], energy=3000.0, num=4, slots=16384, seed=5,
                                 beam_seed=4, msc=True, field=[0.0, 0.0, 3.8]),
    # Charge partition of new tracks' slots (TrackOrder init_charge = 1):
    # neutral and charged tracks fill the two ends of the vacancies, and no
    # secondary takes its dead parent's slot
    "calo_initcharge_msc_field_e2000_n4": dict(pdg=11, energy=2000.0, num=4, slots=4096,
                                               seed=3, msc=True, field=[1.0, 0.0, 0.0],
                                               track_order=1),
    "calo_initcharge_g100_n16": dict(pdg=22, energy=100.0, num=16, slots=1024, seed=7,
                                     track_order=1),
    "cms_initcharge_mix_e5000_n4": dict(geometry="cms", beam="eta", pdgs=[11, 22],
                                        energy=5000.0, num=4, slots=16384, seed=2,
                                        beam_seed=6, msc=True, field=[0.0, 0.0, 3.8],
                                        track_order=1),
    # Thread -> slot reindexing orders (reindex_shuffle = 2, reindex_status = 3,
    # reindex_particle_type = 4): the visiting order changes, the physics
    # does not (the same counters as the unsorted runs of the same problems)
    "calo_shuffle_msc_e1000_n4": dict(pdg=11, energy=1000.0, num=4, slots=65536, seed=0,
                                      msc=True, track_order=2),
    "calo_status_g100_n16": dict(pdg=22, energy=100.0, num=16, slots=4096, seed=7,
                                 track_order=3),
    "cms_particle_mix_e10000_n4": dict(geometry="cms", beam="eta", pdgs=[11, 22],
                                       energy=10000.0, num=4, slots=65536, seed=0,
                                       beam_seed=1, msc=True, field=[0.0, 0.0, 3.8],
                                       track_order=4),
    # Edge cases at the bottom of the energy range: electrons below the
    # 1 keV tracking cut (killed in their first along-step), positrons that
    # stop and annihilate at rest, photons just above the pair threshold,
    # and a log-uniform 1 keV-10 MeV e-/gamma mixture in the CMS-like field
    "calo_e0.0005_n64": dict(pdg=11, energy=0.0005, num=64, slots=256, seed=1),
    "calo_ep0.01_n64": dict(pdg=-11, energy=0.01, num=64, slots=256, seed=2, msc=True),
    "calo_g1.1_n64": dict(pdg=22, energy=1.1, num=64, slots=1024, seed=3),
    "cms_lowe_mix_n64": dict(geometry="cms", beam="eta", pdgs=[11, 22], energy=0.001,
                             emax=10.0, num=64, slots=1024, seed=4, beam_seed=11,
                             msc=True, field=[0.0, 0.0, 3.8]),
    # The top of the CMS-like beam's energy range (100 GeV)
    "cms_mix_e100000_n2": dict(geometry="cms", beam="eta", pdgs=[11, 22], energy=1e5,
                               num=2, slots=65536, seed=5, beam_seed=12, msc=True,
                               field=[0.0, 0.0, 3.8]),
    # Stepper::reseed(event 7) before the first step
    "calo_reseed7_msc_e1000_n4": dict(pdg=11, energy=1000.0, num=4, slots=4096, seed=2,
                                      msc=True, reseed=7),
}

# Step output (detector hits of every step, StepCollector/DetectorSteps):
# the first HIT_RECORDS records in full, and per step the number of hits and
# the sum of every column
HIT_CASES = {
    "hits_calo_msc_field_e300_n1": dict(pdg=11, energy=300.0, num=1, slots=1024, seed=4,
                                        msc=True, field=[1.0, 0.0, 0.0]),
    "hits_cms_mix_e2000_n2": dict(geometry="cms", beam="eta", pdgs=[11, 22], energy=2000.0,
                                  num=2, slots=4096, seed=6, beam_seed=5, msc=True,
                                  field=[0.0, 0.0, 3.8]),
}
HIT_RECORDS = 150

# Interactor parity: one interaction per input, through the reference's own
# model actions (the 'interact' mode of the harness), on tracks that its
# extend-from-primaries, initialize-tracks and pre-step prepared; inputs span
# each model's energy range, every element component of each material and
# isotropic directions. Per case: geometry, physics, seed, combined brems,
# and the material points (position, number of element components)
INTERACTION_CASES = {
    "interact_calo": dict(geometry="calo", seed=0,
                          points=[((0.0, 0.0, 0.1), 1), ((0.0, 0.0, 0.5), 1)]),
    "interact_cms": dict(geometry="cms", seed=1,
                         points=[((4.01, 0.0, 0.0), 1), ((140.0, 0.0, 0.0), 3),
                                 ((182.0, 0.0, 0.0), 2), ((185.2, 0.0, 0.0), 2)]),
    "interact_calo_brcomb": dict(geometry="calo", seed=2, brem_combined=True,
                                 points=[((0.0, 0.0, 0.1), 1), ((0.0, 0.0, 0.5), 1)]),
}
# Energies [MeV] per model and particle, inside each model's range (the
# electron production cut is at most 1.02 MeV here, so Moller scattering
# needs more than 2.04 MeV)
INTERACTION_ENERGIES = {
    ("scat-klein-nishina", 22): [0.005, 0.05, 0.5, 5.0, 50.0, 5e3, 5e5],
    ("photoel-livermore", 22): [0.002, 0.02, 0.087, 0.089, 0.3, 3.0],
    ("conv-bethe-heitler", 22): [1.1, 2.0, 10.0, 100.0, 1e4, 8e4],
    ("brems-sb", 11): [0.1, 1.0, 10.0, 100.0, 999.0],
    ("brems-sb", -11): [0.1, 1.0, 10.0, 100.0, 999.0],
    ("brems-rel", 11): [1001.0, 1e4, 1e5, 1e6],
    ("brems-rel", -11): [1001.0, 1e4, 1e5, 1e6],
    ("ioni-moller-bhabha", 11): [5.0, 50.0, 500.0, 5e4],
    ("ioni-moller-bhabha", -11): [5.0, 50.0, 500.0, 5e4],
    ("annihil-2-gamma", -11): [0.01, 1.0, 100.0, 1e4],
}
COMBINED_ENERGIES = [0.1, 10.0, 500.0, 999.0, 1001.0, 5e3, 1e5, 1e6]
#: Models whose interactor reads the element component
ELEMENT_MODELS = ("photoel-livermore", "conv-bethe-heitler", "brems-sb", "brems-rel",
                  "brems-combined")


def interaction_inputs(name: str) -> list:
    """Inputs of an interaction case: (model, PDG, energy, position,
    direction, element component), directions isotropic from a seeded
    generator."""
    import numpy as np

    c = INTERACTION_CASES[name]
    rng = np.random.default_rng(1000 + c["seed"])
    if c.get("brem_combined"):
        energies = {("brems-combined", pdg): COMBINED_ENERGIES for pdg in (11, -11)}
    else:
        energies = INTERACTION_ENERGIES
    out = []
    for pos, ncomp in c["points"]:
        for (model, pdg), es in energies.items():
            comps = range(ncomp) if model in ELEMENT_MODELS else [0]
            for elcomp in comps:
                for e in es:
                    v = rng.normal(size=3)
                    d = v / np.linalg.norm(v)
                    out.append([model, pdg, e, list(pos), [float(x) for x in d], elcomp])
    return out


def make_interaction_case(name: str, libm: str = "system") -> dict:
    c = INTERACTION_CASES[name]
    inputs = interaction_inputs(name)
    extra = ["--brem-combined"] if c.get("brem_combined") else []
    with tempfile.TemporaryDirectory() as tmp:
        txt = os.path.join(tmp, "inputs.txt")
        oracle.write_interaction_inputs(txt, inputs)
        results = oracle.run_interactions("reference", physics_file(c["geometry"]),
                                          geometry_path(c["geometry"]), txt, c["seed"],
                                          extra=extra, libm=libm)
    case = {"geometry": c["geometry"], "seed": c["seed"],
            "brem_combined": bool(c.get("brem_combined", False))}
    return {"case": case, "inputs": inputs, "results": results}


# Along-step parity: one along-step per input through the reference's own
# actions (the harness's 'along' mode) on tracks that its first actions
# prepared: material points and points just inside boundaries, e-/e+ from 10
# keV to 100 GeV and photons, isotropic directions
ALONG_CASES = {
    "along_cms_msc_field": dict(geometry="cms", seed=3, msc=True, field=[0.0, 0.0, 3.8],
                                points=[(4.01, 0.0, 0.0), (50.0, 0.0, 0.0),
                                        (129.0001, 0.0, 0.0), (140.0, 0.0, 0.0),
                                        (151.9999, 0.0, 0.0), (182.0, 0.0, 0.0),
                                        (185.2, 0.0, 0.0)]),
    "along_calo_msc": dict(geometry="calo", seed=4, msc=True, field=[0.0, 0.0, 0.0],
                           points=[(0.0, 0.0, 0.1), (0.0, 0.0, 0.2299), (0.0, 0.0, 0.5)]),
    "along_calo_msc_field": dict(geometry="calo", seed=5, msc=True, field=[1.0, 0.0, 0.0],
                                 points=[(0.0, 0.0, 0.1), (0.0, 0.0, 0.2299),
                                         (0.0, 0.0, 0.5)]),
}
ALONG_ENERGIES = {11: [0.01, 0.1, 1.0, 10.0, 100.0, 1e3, 1e4, 1e5],
                  -11: [0.01, 0.1, 1.0, 10.0, 100.0, 1e3, 1e4, 1e5],
                  22: [0.1, 10.0, 1e4]}
ALONG_DIRECTIONS = 2


def along_inputs(name: str) -> list:
    """Inputs of an along-step case (the interaction inputs' format, with
    '-' for the model), directions isotropic from a seeded generator."""
    import numpy as np

    c = ALONG_CASES[name]
    rng = np.random.default_rng(2000 + c["seed"])
    out = []
    for pos in c["points"]:
        for pdg, es in ALONG_ENERGIES.items():
            for e in es:
                for _ in range(ALONG_DIRECTIONS):
                    v = rng.normal(size=3)
                    d = v / np.linalg.norm(v)
                    out.append(["-", pdg, e, list(pos), [float(x) for x in d], 0])
    return out


def make_along_case(name: str, libm: str = "system") -> dict:
    c = ALONG_CASES[name]
    inputs = along_inputs(name)
    extra = (["--msc"] if c["msc"] else []) + (
        ["--field"] + [repr(float(f)) for f in c["field"]] if any(c["field"]) else [])
    with tempfile.TemporaryDirectory() as tmp:
        txt = os.path.join(tmp, "inputs.txt")
        oracle.write_interaction_inputs(txt, inputs)
        results = oracle.run_interactions("reference", physics_file(c["geometry"]),
                                          geometry_path(c["geometry"]), txt, c["seed"],
                                          extra=extra, libm=libm, mode="along")
    case = {"geometry": c["geometry"], "seed": c["seed"], "msc": c["msc"],
            "field": list(c["field"])}
    return {"case": case, "inputs": inputs, "results": results}


# Reseeded XORWOW states: seed, track slots, events, and the slots recorded
RNG_SEED = 5
RNG_SLOTS = 4096
RNG_EVENTS = [0, 1, 7, 123456789, (1 << 40) + 3]
RNG_RECORDED = list(range(32)) + [RNG_SLOTS - 1]


def case_primaries(c: dict):
    """Primaries of a golden case (the case dict as stored in a fixture)."""
    if c.get("beam", "pencil") == "eta":
        return eta_beam(c["num_primaries"] if "num_primaries" in c else c["num"],
                        emin=c["energy"], emax=c.get("emax"), pdgs=tuple(c["pdgs"]),
                        seed=c["beam_seed"])
    return pencil_beam(c["num_primaries"] if "num_primaries" in c else c["num"],
                       energy=c["energy"], pdg=c["pdg"], z0=c.get("z0", -5.0))


def case_options(c: dict) -> list[str]:
    """Command-line physics options of the oracle programs for a case."""
    opts = []
    if c.get("msc"):
        opts.append("--msc")
    field = c.get("field")
    if field and any(field):
        opts += ["--field"] + [repr(float(f)) for f in field]
    if c.get("track_order"):
        opts += ["--track-order", str(int(c["track_order"]))]
    if c.get("reseed") is not None:
        opts += ["--reseed", str(int(c["reseed"]))]
    if c.get("rz_field"):
        opts += ["--rz-field", field_map_file(c.get("geometry", "cms"))]
    if c.get("brem_combined"):
        opts.append("--brem-combined")
    for k, v in (c.get("field_options") or {}).items():
        opts += ["--field-option", k, repr(v)]
    return opts


def make_case(name: str, hits: bool = False, libm: str = "system") -> dict:
    c = (HIT_CASES if hits else CASES)[name]
    geometry = c.get("geometry", "calo")
    physics = c.get("physics", geometry)
    case = {"geometry": geometry, "energy": c["energy"],
            "num_primaries": c["num"], "num_track_slots": c["slots"],
            "seed": c["seed"], "msc": bool(c.get("msc", False)),
            "field": list(c.get("field", [0.0, 0.0, 0.0])),
            "track_order": int(c.get("track_order", 0))}
    if c.get("reseed") is not None:
        case["reseed"] = int(c["reseed"])
    if c.get("rz_field"):
        case["rz_field"] = True
    if c.get("brem_combined"):
        case["brem_combined"] = True
    if c.get("field_options"):
        case["field_options"] = dict(c["field_options"])
    if physics != geometry:
        case["physics"] = physics
    if c.get("beam", "pencil") == "eta":
        case.update(beam="eta", pdgs=list(c["pdgs"]), emax=c.get("emax"),
                    beam_seed=c["beam_seed"])
    else:
        case.update(beam="pencil", pdg=c["pdg"], z0=c.get("z0", -5.0))
    prim = case_primaries(case)
    with tempfile.TemporaryDirectory() as tmp:
        ptxt = os.path.join(tmp, "primaries.txt")
        write_primaries_text(ptxt, prim)
        out = oracle.run_reference(physics_file(physics), ptxt, c["slots"], c["seed"],
                                   extra=case_options(c) + (["--hits"] if hits else []),
                                   geometry=geometry_path(geometry), libm=libm)
    if hits:
        per_step = {}
        for h in out["hits"]:
            row = per_step.setdefault(h[0], [h[0], 0] + [0] * (len(h) - 1))
            row[1] += 1
            for k, v in enumerate(h[1:]):
                row[2 + k] += v
        return {
            "case": case,
            "columns": list(oracle.HIT_COLUMNS),
            "steps": out["steps"],
            "edep": out["edep"],
            "num_hits": len(out["hits"]),
            "records": out["hits"][:HIT_RECORDS],
            "per_step": [per_step[k] for k in sorted(per_step)],
        }
    return {
        "case": case,
        "actions": [out["actions"][i] for i in sorted(out["actions"])],
        "steps": out["steps"],
        "total_steps": out["total_steps"],
        "iterations": out["iterations"],
        "edep": out["edep"],
    }


def rng_reseed_dump() -> dict:
    """XORWOW states of the recorded slots after Stepper::reseed, per event."""
    prim = pencil_beam(1, energy=10.0)
    out = {"seed": RNG_SEED, "num_track_slots": RNG_SLOTS, "slots": RNG_RECORDED,
           "events": {}}
    with tempfile.TemporaryDirectory() as tmp:
        ptxt = os.path.join(tmp, "primaries.txt")
        write_primaries_text(ptxt, prim)
        for ev in RNG_EVENTS:
            res = subprocess.run([oracle.REF_BIN, "run", physics_file("calo"), "calo", ptxt,
                                  str(RNG_SLOTS), str(RNG_SEED), "--reseed", str(ev),
                                  "--dump-rng", str(RNG_SLOTS), "--steps", "1"],
                                 capture_output=True, text=True, check=True)
            words = {}
            for line in res.stdout.splitlines():
                tok = line.split()
                if tok and tok[0] == "rng":
                    words[int(tok[1])] = [int(t) for t in tok[2:8]]
            out["events"][str(ev)] = [words[i] for i in RNG_RECORDED]
    return out


def geometry_dump() -> dict:
    res = subprocess.run([oracle.REF_BIN, "geo", "x", "calo"], capture_output=True,
                         text=True, check=True)
    surfaces = []
    volumes = []
    for line in res.stdout.splitlines():
        tok = line.split()
        if tok and tok[0] == "surf":
            surfaces.append({"type": int(tok[3]), "position": float(tok[5])})
        elif tok and tok[0] == "volume":
            volumes.append(tok[2])
    return {"surfaces": surfaces, "volumes": volumes}


def main():
    parser = argparse.ArgumentParser()
    parser.add_argument("--reference", default=oracle.reference_path())
    parser.add_argument("--cases", nargs="*", default=list(CASES))
    parser.add_argument("--hit-cases", nargs="*", default=list(HIT_CASES))
    parser.add_argument("--interactions", nargs="*", default=list(INTERACTION_CASES))
    parser.add_argument("--along", nargs="*", default=list(ALONG_CASES))
    parser.add_argument("--libm", choices=oracle.LIBMS, default="system",
                        help="the reference linked with the host C library's elementary "
                             "functions (fixtures here) or with correctly rounded ones "
                             "(fixtures under pinned/)")
    args = parser.parse_args()
    if oracle.build_reference(args.reference) is None:
        sys.exit("reference sources not found")
    outdir = HERE if args.libm == "system" else os.path.join(HERE, "pinned")
    os.makedirs(outdir, exist_ok=True)
    for name in args.cases:
        data = make_case(name, libm=args.libm)
        with open(os.path.join(outdir, f"{name}.json"), "w") as f:
            json.dump(data, f, indent=0)
        print(name, data["iterations"], data["total_steps"])
    for name in args.hit_cases:
        data = make_case(name, hits=True, libm=args.libm)
        with open(os.path.join(outdir, f"{name}.json"), "w") as f:
            json.dump(data, f, indent=0)
        print(name, data["num_hits"], "hits")
    for name in args.interactions:
        data = make_interaction_case(name, libm=args.libm)
        with open(os.path.join(outdir, f"{name}.json"), "w") as f:
            json.dump(data, f, indent=0)
        print(name, len(data["results"]), "interactions")
    for name in args.along:
        data = make_along_case(name, libm=args.libm)
        with open(os.path.join(outdir, f"{name}.json"), "w") as f:
            json.dump(data, f, indent=0)
        print(name, len(data["results"]), "along-steps")
    if args.libm != "system":
        return
    with open(os.path.join(HERE, "calo_geometry.json"), "w") as f:
        json.dump(geometry_dump(), f, indent=0)
    with open(os.path.join(HERE, "xorwow_reseed.json"), "w") as f:
        json.dump(rng_reseed_dump(), f, indent=0)


if __name__ == "__main__":
    main()
