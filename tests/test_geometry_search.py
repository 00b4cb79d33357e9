"""Ordered search of the implicit background against a solve of every surface.

In the implicit background volume the reference solves every surface and
takes the first crossing whose bumped point lies in a neighboring volume.
The GB300 path walks each kind of surface in the order the ray meets it and
stops at the current best crossing (``GeoTrackView::background_crossing``,
``gbx/Geometry.hh``); its safety distance likewise visits only the nearest
planes and cylinders. The CPU restatement is built both ways
(``-DGBX_GEO_SCAN_BACKGROUND`` restores the full solve) and runs the same
random walks (points near and on cylinders, isotropic, axis-aligned,
near-axial and near-tangent directions, step limits from 1e-6 cm to
infinity, boundary crossings and direction changes): every query's next step,
crossed surface and safety must agree to the bit.
"""

import subprocess

import pytest

import oracle
from celeritas_gb300 import physics_file


@pytest.fixture(scope="module")
def ports():
    return oracle.build_port(), oracle.build_port(geo_scan=True)


@pytest.mark.parametrize("geometry,walks", [("cms", 6000), ("calo", 4000)])
def test_ordered_walks_match_full_solve(ports, geometry, walks):
    outs = []
    for exe in ports:
        res = subprocess.run([exe, "geo-rays", physics_file(geometry), geometry,
                              str(walks), "20261204"],
                             capture_output=True, text=True, check=True)
        outs.append((res.stdout, res.stderr))
    (ordered, err), (scan, _) = outs
    background = int(err.split()[-1])
    assert background > 5000, err
    lines_o, lines_s = ordered.splitlines(), scan.splitlines()
    assert len(lines_o) == len(lines_s)
    bad = [(a, b) for a, b in zip(lines_o, lines_s) if a != b]
    assert not bad, bad[:5]


FIELD_CASES = ["calo_msc_field_e5000_n2", "calo_msc_field_ep2000_n2", "cms_mix_e10000_n4",
               "cms_mix_logu_n6", "cms_rzmap_mix_e2000_n4", "cms_fieldopt_mix_e5000_n4",
               "tracker_mix_e3000_n4"]


@pytest.mark.parametrize("name", FIELD_CASES)
def test_safe_ball_never_contradicts_full_query(name):
    """The field propagation answers a chord query without the geometry when
    the chord lies in a ball free of surfaces (``inside_safe_ball``,
    ``gbx/Field.hh``). The check build of the CPU restatement runs every
    query in full along the golden transports and counts the queries the
    ball answered and any whose full answer differs: there must be none, and
    the ball must have been used."""
    import os
    import tempfile

    from celeritas_gb300.primaries import write_primaries_text
    from conftest import case_options, case_primaries, case_problem, load_golden

    exe = oracle.build_port(check_ball=True)
    case = load_golden(name, "pinned")["case"]
    physics, geometry = case_problem(case)
    with tempfile.TemporaryDirectory() as tmp:
        ptxt = os.path.join(tmp, "p.txt")
        write_primaries_text(ptxt, case_primaries(case))
        res = subprocess.run([exe, "run", physics, geometry, ptxt,
                              str(case["num_track_slots"]), str(case["seed"]),
                              *case_options(case)],
                             capture_output=True, text=True, check=True)
    line = [ln for ln in res.stderr.splitlines() if ln.startswith("safe_ball")][-1]
    uses, mismatches = int(line.split()[2]), int(line.split()[4])
    assert mismatches == 0, line
    assert uses > 0, line
