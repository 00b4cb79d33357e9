"""FP64 elementary functions of the stepping loop on the host (no GPU).

exp, log, sin, cos, tanh, log1p, expm1 and cbrt of the GB300 build
(celeritas_gb300/csrc/gbx/Libm.hh), compiled into the CPU restatement, must
return the correctly rounded double: on the committed vectors
(tests/golden/libm_cr.json: special values, thresholds, inputs that the host
C library misrounds, seeded random draws) and, where mpmath is available, on
fresh seeded random inputs against a 250-bit evaluation.
"""

import json
import math
import os
import random

import numpy as np
import pytest

import oracle
from conftest import GOLDEN

FUNCTIONS = ("exp", "log", "sin", "cos", "tanh", "log1p", "expm1", "cbrt")


def load_vectors():
    with open(os.path.join(GOLDEN, "libm_cr.json")) as f:
        d = json.load(f)
    return {fn: (np.array([float.fromhex(a) for a, _ in d[fn]]),
                 np.array([float.fromhex(b) for _, b in d[fn]])) for fn in FUNCTIONS}


def same_doubles(a, b):
    """Element-wise bit equality up to the sign of NaN."""
    a, b = np.asarray(a), np.asarray(b)
    nan = np.isnan(a) & np.isnan(b)
    return nan | ((a == b) & (np.signbit(a) == np.signbit(b)))


@pytest.mark.parametrize("fn", FUNCTIONS)
def test_host_matches_correctly_rounded_vectors(built_port, fn):
    x, y = load_vectors()[fn]
    got = oracle.port_libm(fn, x)
    bad = ~same_doubles(got, y)
    assert not bad.any(), list(zip(x[bad][:5], got[bad][:5], y[bad][:5]))


@pytest.mark.parametrize("fn", FUNCTIONS)
def test_host_correctly_rounded_random(built_port, fn):
    mpmath = pytest.importorskip("mpmath")
    from golden.make_libm_vectors import correctly_rounded, random_inputs

    mpmath.mp.prec = 250
    xs = random_inputs(fn, 1500, random.Random(hash(fn) % 1000 + 7))
    got = oracle.port_libm(fn, xs)
    ref = np.array([correctly_rounded(fn, x) for x in xs])
    bad = ~same_doubles(got, ref)
    assert not bad.any(), list(zip(np.array(xs)[bad][:5], got[bad][:5], ref[bad][:5]))


def test_system_build_uses_host_library(built_port):
    """The restatement built against the host C library reproduces that
    library (the unmodified reference's functions), not the pinned ones."""
    import ctypes

    libm = ctypes.CDLL("libm.so.6")
    libm.exp.restype = ctypes.c_double
    libm.exp.argtypes = [ctypes.c_double]
    x, _ = load_vectors()["exp"]
    x = x[np.isfinite(x)]
    got = oracle.port_libm("exp", x, libm="system")
    assert same_doubles(got, [libm.exp(float(v)) for v in x]).all()
    assert math.isfinite(got[0])
