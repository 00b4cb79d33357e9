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
