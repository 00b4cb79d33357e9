"""FP64 elementary functions on the GB300 against the host (GPU).

The FP64 stepping loop's bit-for-bit parity needs its exp, log, sin, cos,
tanh, log1p, expm1 and cbrt to return the same doubles on the device as on
the host: the device results (through gbx_libm_evaluate) must equal the
correctly rounded vectors and the CPU restatement's host results on 2^18
seeded random inputs per function, bit for bit.
"""

import numpy as np
import pytest

import oracle
from test_libm import FUNCTIONS, load_vectors, same_doubles

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gb(built_lib):
    import celeritas_gb300 as gb

    gb.load_library(built_lib)
    return gb


@pytest.mark.parametrize("fn", FUNCTIONS)
def test_device_matches_correctly_rounded_vectors(gb, fn):
    x, y = load_vectors()[fn]
    got = gb.libm_evaluate(fn, x)
    bad = ~same_doubles(got, y)
    assert not bad.any(), list(zip(x[bad][:5], got[bad][:5], y[bad][:5]))


RANGES = {"exp": (-745.0, 709.0), "log": None, "sin": (-20.0, 20.0), "cos": (-20.0, 20.0),
          "tanh": (-25.0, 25.0), "log1p": (-0.999, 50.0), "expm1": (-45.0, 45.0),
          "cbrt": None}


@pytest.mark.parametrize("fn", FUNCTIONS)
def test_device_equals_host(gb, built_port, fn):
    rng = np.random.default_rng(FUNCTIONS.index(fn) + 100)
    n = 1 << 18
    if RANGES[fn] is None:
        # log-uniform magnitudes over the whole double range
        x = 10.0 ** rng.uniform(-300, 300, n)
        if fn == "cbrt":
            x *= rng.choice([-1.0, 1.0], n)
    else:
        lo, hi = RANGES[fn]
        x = np.concatenate([rng.uniform(lo, hi, n // 2),
                            rng.uniform(-1.0, 1.0, n // 4) * 10.0 ** rng.uniform(-12, 0, n // 4)])
        x = np.concatenate([x, rng.uniform(lo, hi, n - len(x))])
    dev = gb.libm_evaluate(fn, x)
    host = oracle.port_libm(fn, x)
    bad = ~same_doubles(dev, host)
    assert not bad.any(), list(zip(x[bad][:5], dev[bad][:5], host[bad][:5]))
