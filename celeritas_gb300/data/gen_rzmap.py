"""Write the synthetic R-Z magnetic field map of the CMS-like detector.

A solenoid-like field on a uniform (z, r) grid, standing in for the measured
CMS map that the reference's RZMapFieldInput would read (no map ships with
the reference): Bz = 3.8 T inside r < 300 cm and |z| < 600 cm with soft
edges, a -1.2 T return flux around r = 350 cm, and Br = -(r/2) dBz/dz, the
first term of a divergence-free field about the axis.

Format: a header line 'rzmap num_z num_r min_z max_z min_r max_r' (cm), then
num_z * num_r lines 'Bz Br' in tesla, z-major with r fastest (the [Z][R]
order of RZMapFieldInput).

    python -m celeritas_gb300.data.gen_rzmap [output]
"""

from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
NUM_Z, NUM_R = 141, 81
MIN_Z, MAX_Z = -700.0, 700.0
MIN_R, MAX_R = 0.0, 400.0


def field(r, z):
    """(Bz, Br) in tesla."""
    def logistic(x):
        return 1.0 / (1.0 + np.exp(x))
    f = logistic((np.abs(z) - 600.0) / 40.0)
    dfdz = -np.sign(z) * f * (1 - f) / 40.0
    inner = logistic((r - 300.0) / 20.0)
    radial = 3.8 * inner - 1.2 * (1 - inner) * np.exp(-((r - 350.0) / 30.0) ** 2)
    bz = f * radial
    br = -0.5 * r * dfdz * radial
    return bz, br


def write(path: str):
    z = np.linspace(MIN_Z, MAX_Z, NUM_Z)
    r = np.linspace(MIN_R, MAX_R, NUM_R)
    zz, rr = np.meshgrid(z, r, indexing="ij")
    bz, br = field(rr, zz)
    with open(path, "w") as f:
        f.write(f"rzmap {NUM_Z} {NUM_R} {MIN_Z!r} {MAX_Z!r} {MIN_R!r} {MAX_R!r}\n")
        for a, b in zip(bz.ravel(), br.ravel()):
            f.write(f"{a:.10g} {b:.10g}\n")


if __name__ == "__main__":
    write(sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "cms.rzmap.txt"))
