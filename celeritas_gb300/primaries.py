"""Synthetic primary generation for the benchmark configurations.

Plays the role of the reference's PrimaryGenerator with
PrimaryGeneratorOptions (src/celeritas/phys/PrimaryGenerator.cc,
src/celeritas/phys/PrimaryGeneratorOptions.hh): seeded, reproducible
primaries with the configurations' particle types, energy spectra and beam
shapes. Primaries are a numpy structured array; ``write_primaries_text``
writes the text form read by the CPU oracle programs.
"""

from __future__ import annotations

import numpy as np

PRIMARY_DTYPE = np.dtype([
    ("pdg", np.int32),
    ("energy", np.float64),
    ("pos", np.float64, 3),
    ("dir", np.float64, 3),
    ("time", np.float64),
    ("event", np.uint32),
])


def pencil_beam(num: int, energy: float = 1000.0, pdg: int = 11,
                z0: float = -5.0, event: int = 0, num_events: int = 1) -> np.ndarray:
    """Pencil beam along +z from (0, 0, z0); events assigned round-robin."""
    p = np.zeros(num, dtype=PRIMARY_DTYPE)
    p["pdg"] = pdg
    p["energy"] = energy
    p["pos"][:, 2] = z0
    p["dir"][:, 2] = 1.0
    p["event"] = event + (np.arange(num) % max(num_events, 1))
    return p


def spread_beam(num: int, emin: float = 100.0, emax: float = 1e4,
                sigma: float = 1.0, pdg: int = 11, z0: float = -5.0,
                seed: int = 0, num_events: int = 1) -> np.ndarray:
    """Log-uniform energies in [emin, emax] MeV, Gaussian transverse spread."""
    rng = np.random.default_rng(seed)
    p = np.zeros(num, dtype=PRIMARY_DTYPE)
    p["pdg"] = pdg
    p["energy"] = np.exp(rng.uniform(np.log(emin), np.log(emax), num))
    p["pos"][:, 0] = rng.normal(0.0, sigma, num)
    p["pos"][:, 1] = rng.normal(0.0, sigma, num)
    p["pos"][:, 2] = z0
    p["dir"][:, 2] = 1.0
    p["event"] = np.arange(num) % max(num_events, 1)
    return p


def write_primaries_text(path: str, primaries: np.ndarray):
    """Write 'pdg energy x y z dx dy dz time event' lines (round-trip exact)."""
    with open(path, "w") as f:
        for p in primaries:
            vals = [repr(float(p["energy"]))]
            vals += [repr(float(v)) for v in p["pos"]]
            vals += [repr(float(v)) for v in p["dir"]]
            vals += [repr(float(p["time"])), str(int(p["event"]))]
            f.write(f"{int(p['pdg'])} " + " ".join(vals) + "\n")


def eta_beam(num: int, emin: float = 1000.0, emax: float | None = None,
             pdgs=(11, 22), eta_max: float = 1.5, seed: int = 0,
             num_events: int = 1) -> np.ndarray:
    """Primaries from the origin, directions isotropic in azimuth and uniform
    in pseudorapidity |eta| < eta_max; energies log-uniform in [emin, emax]
    MeV (fixed at emin if emax is None); particle types cycle through pdgs;
    events assigned in blocks of num / num_events."""
    rng = np.random.default_rng(seed)
    p = np.zeros(num, dtype=PRIMARY_DTYPE)
    p["pdg"] = np.array(pdgs)[np.arange(num) % len(pdgs)]
    if emax is None:
        p["energy"] = emin
    else:
        p["energy"] = np.exp(rng.uniform(np.log(emin), np.log(emax), num))
    eta = rng.uniform(-eta_max, eta_max, num)
    phi = rng.uniform(0.0, 2 * np.pi, num)
    theta = 2 * np.arctan(np.exp(-eta))
    p["dir"][:, 0] = np.sin(theta) * np.cos(phi)
    p["dir"][:, 1] = np.sin(theta) * np.sin(phi)
    p["dir"][:, 2] = np.cos(theta)
    per_event = max(1, -(-num // max(num_events, 1)))
    p["event"] = np.arange(num) // per_event
    return p
