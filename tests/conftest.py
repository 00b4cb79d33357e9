"""Shared test configuration: markers, golden fixtures and helpers."""

from __future__ import annotations

import json
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(REPO, "tests", "golden")
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU (sm_103a)")


def load_golden(name: str, libm: str = "system") -> dict:
    """A golden fixture of the reference linked with the host C library
    ("system", tests/golden/) or with correctly rounded elementary functions
    ("pinned", tests/golden/pinned/)."""
    folder = GOLDEN if libm == "system" else os.path.join(GOLDEN, "pinned")
    with open(os.path.join(folder, f"{name}.json")) as f:
        return json.load(f)


GOLDEN_CASES = ["calo_e1000_n4", "calo_e1000_n4_slots512", "calo_g100_n16",
                "calo_ep500_n4", "calo_e1000_n100", "calo_e10000_n2",
                "calo_msc_e1000_n4", "calo_field_e1000_n4", "calo_msc_field_e5000_n2",
                "calo_msc_field_ep2000_n2", "calo_sorted_both_e1000_n4",
                "calo_sorted_post_g100_n16", "calo_msc_field_sorted_along_e2000_n2",
                "cms_mix_e10000_n4", "cms_mix_logu_n6", "cms_sorted_both_mix_e5000_n4",
                "calo_reseed7_msc_e1000_n4", "cms_rzmap_mix_e2000_n4",
                "calo_brcomb_e10000_n2", "calo_brcomb_msc_field_ep3000_n2",
                "calo_brcomb_sorted_both_e2000_n4", "cms_fieldopt_mix_e5000_n4",
                "slabs_e2000_n4", "tracker_mix_e3000_n4",
                "calo_initcharge_msc_field_e2000_n4", "calo_initcharge_g100_n16",
                "cms_initcharge_mix_e5000_n4", "calo_shuffle_msc_e1000_n4",
                "calo_status_g100_n16", "cms_particle_mix_e10000_n4",
                "calo_e0.0005_n64", "calo_ep0.01_n64", "calo_g1.1_n64", "cms_lowe_mix_n64",
                "cms_mix_e100000_n2"]


def case_problem(case: dict) -> tuple[str, str]:
    """(physics file, geometry argument) of a golden case"""
    from celeritas_gb300 import geometry_path, physics_file

    geometry = case.get("geometry", "calo")
    return physics_file(case.get("physics", geometry)), geometry_path(geometry)


def case_primaries(case: dict):
    """Primaries of a golden case (pencil beam along z, or eta-uniform from
    the origin), as tests/golden/make_golden.py made them."""
    from celeritas_gb300.primaries import eta_beam, pencil_beam

    if case.get("beam", "pencil") == "eta":
        return eta_beam(case["num_primaries"], emin=case["energy"], emax=case.get("emax"),
                        pdgs=tuple(case["pdgs"]), seed=case["beam_seed"])
    return pencil_beam(case["num_primaries"], energy=case["energy"], pdg=case["pdg"],
                       z0=case.get("z0", -5.0))


def case_options(case: dict) -> list[str]:
    """Oracle command-line physics options for a golden case."""
    opts = []
    if case.get("msc"):
        opts.append("--msc")
    field = case.get("field") or [0, 0, 0]
    if any(field):
        opts += ["--field"] + [repr(float(f)) for f in field]
    if case.get("track_order"):
        opts += ["--track-order", str(int(case["track_order"]))]
    if case.get("reseed") is not None:
        opts += ["--reseed", str(int(case["reseed"]))]
    if case.get("rz_field"):
        from celeritas_gb300 import field_map_file

        opts += ["--rz-field", field_map_file(case.get("geometry", "cms"))]
    if case.get("brem_combined"):
        opts.append("--brem-combined")
    for k, v in (case.get("field_options") or {}).items():
        opts += ["--field-option", k, repr(v)]
    return opts


@pytest.fixture(scope="session")
def built_port():
    import oracle

    return oracle.build_port()


@pytest.fixture(scope="session")
def built_lib():
    from celeritas_gb300.build import build

    return build()
