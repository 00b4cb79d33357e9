"""Write LibmTables.hh: the constant tables of the elementary functions in
Libm.hh, computed with 200-bit arithmetic (mpmath) and rounded to doubles.

Every value is a mathematical constant (powers of two, logarithms, parts of
ln 2 and pi/2), so the tables can be regenerated and checked:

    python celeritas_gb300/csrc/gbx/gen_libm_tables.py
"""

from __future__ import annotations

import os

import mpmath

mpmath.mp.prec = 200
HERE = os.path.dirname(os.path.abspath(__file__))
N = 128  # table size of exp (2^(j/N)) and log (N intervals of [1, 2))


def rd(v) -> float:
    """Nearest double."""
    return float(mpmath.mpf(v))


def split(v, bits: int) -> float:
    """v rounded to 'bits' significant bits."""
    v = mpmath.mpf(v)
    if v == 0:
        return 0.0
    e = int(mpmath.floor(mpmath.log(abs(v), 2)))
    scale = mpmath.mpf(2) ** (bits - 1 - e)
    return float(mpmath.nint(v * scale) / scale)


def dd(v):
    hi = rd(v)
    lo = rd(mpmath.mpf(v) - mpmath.mpf(hi))
    return hi, lo


def h(x: float) -> str:
    return float(x).hex()


def main():
    out = []
    w = out.append
    w("// Generated by gen_libm_tables.py: constant tables of Libm.hh (do not edit).")
    w("// Values are correctly rounded doubles of the exact mathematical constants;")
    w("// pairs (hi, lo) hold a value to about 2^-106 relative.")
    w("#pragma once")
    w("")
    w("// GBX_LIBM_TABLE(name, ...) defines one table; Libm.hh expands it twice,")
    w("// as a device array and as a host array.")
    # exp: 2^(j/N) for j in [0, N) as (hi, lo)
    vals = []
    for j in range(N):
        hi, lo = dd(mpmath.mpf(2) ** (mpmath.mpf(j) / N))
        vals += [hi, lo]
    w("#define GBX_LIBM_EXP_TABLE \\")
    lines = [f"    {h(vals[2 * j])}, {h(vals[2 * j + 1])}" for j in range(N)]
    w(", \\\n".join(lines))
    w("")
    # log: interval j of [1, 2) is [1 + j/N, 1 + (j+1)/N); its center c, the
    # double nearest 1/c, and -log of that double as (hi, lo)
    vals = []
    for j in range(N):
        c = 1 + (mpmath.mpf(j) + mpmath.mpf(0.5)) / N
        inv_c = rd(1 / c)
        hi, lo = dd(-mpmath.log(mpmath.mpf(inv_c)))
        vals += [inv_c, hi, lo]
    w("#define GBX_LIBM_LOG_TABLE \\")
    lines = [f"    {h(vals[3 * j])}, {h(vals[3 * j + 1])}, {h(vals[3 * j + 2])}"
             for j in range(N)]
    w(", \\\n".join(lines))
    w("")
    # ln 2 / N in three parts (the first two of 35 bits, so that k times them
    # is exact for |k| < 2^18), ln 2 in three parts (42, 42, 53 bits: e times
    # the first two exact for |e| < 2^11), pi/2 in three parts (33, 33, 53)
    ln2n = mpmath.log(2) / N
    a = split(ln2n, 35)
    b = split(ln2n - a, 35)
    c = rd(ln2n - a - b)
    w(f"#define GBX_LIBM_LN2_N {h(a)}, {h(b)}, {h(c)}")
    ln2 = mpmath.log(2)
    a = split(ln2, 42)
    b = split(ln2 - a, 42)
    c = rd(ln2 - a - b)
    w(f"#define GBX_LIBM_LN2 {h(a)}, {h(b)}, {h(c)}")
    pio2 = mpmath.pi / 2
    a = split(pio2, 33)
    b = split(pio2 - a, 33)
    c = rd(pio2 - a - b)
    w(f"#define GBX_LIBM_PIO2 {h(a)}, {h(b)}, {h(c)}")
    w(f"#define GBX_LIBM_INV_LN2_N {h(rd(N / mpmath.log(2)))}")
    w(f"#define GBX_LIBM_TWO_OVER_PI {h(rd(2 / mpmath.pi))}")
    # Taylor coefficients as (hi, lo): 1/k! for exp, 1/k for log1p
    w("#define GBX_LIBM_INV_FACT \\")
    lines = []
    for k in range(0, 28):
        hi, lo = dd(1 / mpmath.factorial(k))
        lines.append(f"    {h(hi)}, {h(lo)}")
    w(", \\\n".join(lines))
    w("#define GBX_LIBM_INV_INT \\")
    lines = []
    for k in range(0, 28):
        hi, lo = dd(1 / mpmath.mpf(k)) if k else (0.0, 0.0)
        lines.append(f"    {h(hi)}, {h(lo)}")
    w(", \\\n".join(lines))
    w("")
    with open(os.path.join(HERE, "LibmTables.hh"), "w") as f:
        f.write("\n".join(out))


if __name__ == "__main__":
    main()
