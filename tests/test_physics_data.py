"""The synthetic physics input is deterministic and well formed (no GPU)."""

import numpy as np
import pytest

from celeritas_gb300 import physics_file
from celeritas_gb300.data import gen_physics


def parse(text):
    d = {}
    for line in text.splitlines():
        tok = line.split()
        d[tok[0]] = tok[2:]
    return d


@pytest.mark.parametrize("problem", ["calo", "cms"])
def test_committed_file_is_regenerated_exactly(problem):
    with open(physics_file(problem)) as f:
        committed = f.read()
    assert gen_physics.generate(problem) == committed


def test_tables_are_log_spaced_and_nonnegative():
    d = parse(open(physics_file("calo")).read())
    for key, vals in d.items():
        if key.startswith("table.") and key.endswith(".x"):
            x = np.array(vals, dtype=float)
            ratio = x[1:] / x[:-1]
            assert np.allclose(ratio, ratio[0], rtol=1e-9), key
            y = np.array(d[key[:-2] + ".y"], dtype=float)
            assert (y >= 0).all(), key
        if ".range." in key and key.endswith(".y"):
            y = np.array(vals, dtype=float)
            assert (np.diff(y) > 0).all() and y[0] > 0, key


def test_production_cuts_are_bounded():
    d = parse(open(physics_file("calo")).read())
    for m in range(int(d["materials"][0])):
        for pdg in (11, -11, 22):
            e = float(d[f"material.{m}.cut.{pdg}"][0])
            assert 990e-6 <= e <= 10e3
