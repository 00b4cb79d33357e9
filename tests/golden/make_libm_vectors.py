"""Golden vectors of the FP64 elementary functions: correctly rounded values.

Writes tests/golden/libm_cr.json: for each function of the stepping loop's
elementary-function set (exp, log, sin, cos, tanh, log1p, expm1, cbrt), a
list of [x, f(x)] pairs as hexadecimal doubles, f(x) computed with 250-bit
arithmetic (mpmath) and rounded to nearest (including subnormal results).
The inputs are seeded random draws over each function's range plus special
values, values at the overflow and underflow thresholds, and inputs on which
the host C library's result is not correctly rounded (found by search).

    python tests/golden/make_libm_vectors.py
"""

from __future__ import annotations

import ctypes
import json
import math
import os
import random

import mpmath

HERE = os.path.dirname(os.path.abspath(__file__))
mpmath.mp.prec = 250

MP = {"exp": mpmath.exp, "log": mpmath.log, "sin": mpmath.sin, "cos": mpmath.cos,
      "tanh": mpmath.tanh, "log1p": mpmath.log1p, "expm1": mpmath.expm1,
      "cbrt": lambda v: mpmath.cbrt(v) if v >= 0 else -mpmath.cbrt(-v)}


def correctly_rounded(fn: str, x: float) -> float:
    if math.isnan(x):
        return math.nan
    special = {
        ("exp", math.inf): math.inf, ("exp", -math.inf): 0.0,
        ("log", 0.0): -math.inf, ("log", math.inf): math.inf,
        ("log1p", -1.0): -math.inf, ("log1p", math.inf): math.inf,
        ("expm1", math.inf): math.inf, ("expm1", -math.inf): -1.0,
        ("tanh", math.inf): 1.0, ("tanh", -math.inf): -1.0,
        ("cbrt", math.inf): math.inf, ("cbrt", -math.inf): -math.inf,
    }
    if (fn, x) in special:
        return special[(fn, x)]
    if (fn == "log" and x < 0) or (fn == "log1p" and x < -1) or \
            (fn in ("sin", "cos") and math.isinf(x)):
        return math.nan
    if x == 0 and fn in ("sin", "tanh", "expm1", "log1p", "cbrt"):
        return x
    v = MP[fn](mpmath.mpf(x))
    if v == 0:
        return 0.0
    if abs(v) >= mpmath.mpf(2) ** 1024:
        return math.copysign(math.inf, float(mpmath.sign(v)))
    if abs(v) < mpmath.mpf(2) ** -1022:
        return float(mpmath.nint(v * mpmath.mpf(2) ** 1074)) * 2.0 ** -1074
    return float(v)


def random_inputs(fn: str, n: int, rng: random.Random) -> list[float]:
    draw = {
        "exp": lambda: rng.choice([rng.uniform(-745.2, 709.8), rng.uniform(-2, 2),
                                   rng.uniform(-745.2, -708), -10 ** rng.uniform(-12, 2.8)]),
        "log": lambda: rng.choice([10 ** rng.uniform(-320, 308), rng.uniform(0.98, 1.02),
                                   10 ** rng.uniform(-12, 4)]),
        "sin": lambda: rng.choice([rng.uniform(-7, 7), rng.uniform(0, 2 * math.pi),
                                   rng.uniform(-1e5, 1e5), 10 ** rng.uniform(-10, 0)]),
        "cos": lambda: rng.choice([rng.uniform(-7, 7), rng.uniform(0, 2 * math.pi),
                                   rng.uniform(-1e5, 1e5), 10 ** rng.uniform(-10, 0)]),
        "tanh": lambda: rng.choice([rng.uniform(-25, 25), rng.uniform(-1, 1),
                                    10 ** rng.uniform(-10, 0)]),
        "log1p": lambda: rng.choice([10 ** rng.uniform(-20, 10), -rng.uniform(0, 1),
                                     rng.uniform(-0.01, 0.01)]),
        "expm1": lambda: rng.choice([rng.uniform(-50, 50), rng.uniform(-0.4, 0.4),
                                     rng.choice([-1, 1]) * 10 ** rng.uniform(-20, 0)]),
        "cbrt": lambda: rng.choice([rng.choice([-1, 1]) * 10 ** rng.uniform(-320, 308),
                                    rng.uniform(0, 10)]),
    }[fn]
    return [float(draw()) for _ in range(n)]


EDGES = {
    "exp": [0.0, -0.0, 1e-300, -1e-300, 2.0 ** -54, 709.782712893384, 709.7827128933841,
            -708.3964185322641, -745.1332191019411, -745.1332191019412, -745.2, 1e3,
            math.inf, -math.inf, math.nan],
    "log": [1.0, 2.0, 0.5, 5e-324, 2.2250738585072014e-308, 1.7976931348623157e308,
            1.0078125, 0.9921875, 1 + 2.0 ** -52, 1 - 2.0 ** -53, 0.0, math.inf, -1.0,
            math.nan],
    "sin": [0.0, -0.0, 1e-300, math.pi, math.pi / 2, 1e6, math.inf, math.nan],
    "cos": [0.0, 1e-300, math.pi, math.pi / 2, 1e6, math.inf, math.nan],
    "tanh": [0.0, -0.0, 1e-300, 22.0, -22.0, 0.35, math.inf, -math.inf, math.nan],
    "log1p": [0.0, -0.0, 1e-300, 2.0 ** -7, -2.0 ** -7, -0.5, 1e300, -1.0, -2.0,
              math.inf, math.nan],
    "expm1": [0.0, -0.0, 1e-300, 0.35, -0.35, 709.78, 709.79, -40.0, -41.0, math.inf,
              -math.inf, math.nan],
    "cbrt": [0.0, -0.0, 5e-324, -5e-324, 8.0, 27.0, -1.0, 1.7976931348623157e308,
             -9.409401804709187e307, math.inf, -math.inf, math.nan],
}


def glibc_misrounded(fn: str, rng: random.Random, want: int, tries: int) -> list[float]:
    """Inputs on which the host C library's result is not correctly rounded."""
    libm = ctypes.CDLL("libm.so.6")
    f = getattr(libm, fn)
    f.restype = ctypes.c_double
    f.argtypes = [ctypes.c_double]
    found = []
    for x in random_inputs(fn, tries, rng):
        y = f(x)
        cr = correctly_rounded(fn, x)
        if y != cr and not (math.isnan(y) and math.isnan(cr)):
            found.append(x)
            if len(found) >= want:
                break
    return found


def main():
    rng = random.Random(20261204)
    out = {"note": "[x, f(x)] as hexadecimal doubles, f correctly rounded to nearest"}
    for fn in MP:
        xs = EDGES[fn] + random_inputs(fn, 300, rng)
        xs += glibc_misrounded(fn, rng, want=20, tries=20000)
        out[fn] = [[float(x).hex(), float(correctly_rounded(fn, x)).hex()] for x in xs]
        print(fn, len(out[fn]))
    with open(os.path.join(HERE, "libm_cr.json"), "w") as f:
        json.dump(out, f, indent=0)


if __name__ == "__main__":
    main()
