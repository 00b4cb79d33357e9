"""Synthetic EM physics input for the stepping loop.

Geant4 (and its G4EMLOW data) is not available, so the physics tables that the
reference normally imports from Geant4 (``src/celeritas/io/ImportData.hh:55-107``)
are generated here from textbook formulas. Both the GB300 path and the CPU
oracle (the reference compiled from source) read the *same* generated file, so
"same inputs" holds by construction. Physical realism versus Geant4 is not
claimed; the tables are smooth, positive and of realistic magnitude so that
showers have realistic step counts.

Contents (the ImportData pieces the stepping loop consumes):

* elements, materials (number densities, number fractions) and production
  cuts (``ImportMaterial.hh``, ``ImportElement.hh``);
* per-process ``lambda`` / ``dedx`` / ``range`` tables on log-uniform grids,
  7 bins per decade (``ImportPhysicsTable.hh:32-51``);
* per-model micro cross sections for element selection (``ImportModel.hh``);
* Seltzer-Berger scaled DCS tables (``ImportSBTable.hh``), Livermore
  photoelectric subshell data (``ImportLivermorePE.hh``);
* Urban MSC transport cross sections (``ImportModel.hh`` ImportMscModel);
* EM and transport parameters (``ImportParameters.hh``).

File format: plain text, one record per line: ``key count v0 v1 ...``; floating
point values are written with 17 significant digits so they round-trip exactly.
The file is deterministic (no random numbers) and committed beside this script.

Usage: ``python -m celeritas_gb300.data.gen_physics`` regenerates the files.
"""

from __future__ import annotations

import math
import os

import numpy as np

# Physical constants (CODATA 2018), CGS + MeV
R_E = 2.8179403262e-13  # classical electron radius [cm]
M_E = 0.51099895000  # electron mass [MeV]
ALPHA = 1 / 137.035999084
N_A = 6.02214076e23
BARN = 1e-24  # [cm^2]
TWOPI_RE2 = 2 * math.pi * R_E * R_E

BINS_PER_DECADE = 7
E_MIN = 1e-4  # 100 eV
E_MAX = 1e8  # 100 TeV
RANGE_CUT = 0.07  # 0.7 mm production cut

ELEMENTS = {
    # name: (Z, atomic mass [amu], mean excitation energy [MeV])
    "H": (1, 1.00794, 19.2e-6),
    "C": (6, 12.0107, 81.0e-6),
    "O": (8, 15.9994, 95.0e-6),
    "Si": (14, 28.0855, 173.0e-6),
    "Ar": (18, 39.948, 188.0e-6),
    "Cu": (29, 63.546, 322.0e-6),
    "Zn": (30, 65.38, 330.0e-6),
    "W": (74, 183.84, 727.0e-6),
    "Pb": (82, 207.2, 823.0e-6),
}

# name: (density [g/cm^3], state, [(element, number fraction)])
MATERIALS = {
    "G4_Galactic": (1e-25, "gas", [("H", 1.0)]),
    "G4_Pb": (11.35, "solid", [("Pb", 1.0)]),
    "G4_lAr": (1.396, "liquid", [("Ar", 1.0)]),
    "G4_Si": (2.33, "solid", [("Si", 1.0)]),
    "G4_PbWO4": (8.28, "solid", [("Pb", 1 / 6), ("W", 1 / 6), ("O", 4 / 6)]),
    # Brass 70/30 by mass -> number fractions
    "Brass": (8.53, "solid", [("Cu", 0.70 / 63.546 / (0.70 / 63.546 + 0.30 / 65.38)),
                              ("Zn", 0.30 / 65.38 / (0.70 / 63.546 + 0.30 / 65.38))]),
    "G4_PLASTIC_SC_VINYLTOLUENE": (1.032, "solid", [("C", 9 / 19), ("H", 10 / 19)]),
}

PROBLEMS = {
    # problem name: material list (index = material id)
    "calo": ["G4_Galactic", "G4_Pb", "G4_lAr"],
    "cms": ["G4_Galactic", "G4_Si", "G4_PbWO4", "Brass", "G4_PLASTIC_SC_VINYLTOLUENE"],
}


def log_grid(emin: float, emax: float) -> np.ndarray:
    """Log-uniform grid with BINS_PER_DECADE bins per decade (endpoints exact)."""
    ndec = math.log10(emax / emin)
    nbins = max(int(round(ndec * BINS_PER_DECADE)), 2)
    e = emin * np.power(10.0, np.arange(nbins + 1) * (ndec / nbins))
    e[0], e[-1] = emin, emax
    return e


# --------------------------------------------------------------------------
# Material properties
# --------------------------------------------------------------------------
class Mat:
    def __init__(self, name):
        density, state, comp = MATERIALS[name]
        # Components in increasing element order, the order in which the
        # reference stores a material's components (and so pairs them with
        # the per-element micro cross sections)
        comp = sorted(comp, key=lambda c: ELEMENTS[c[0]][0])
        self.name, self.density, self.state = name, density, state
        self.els = [e for e, _ in comp]
        self.frac = np.array([f for _, f in comp])
        self.frac /= self.frac.sum()
        amean = sum(f * ELEMENTS[e][1] for e, f in zip(self.els, self.frac))
        self.number_density = density * N_A / amean  # atoms / cm^3
        self.n_at = self.number_density * self.frac
        self.z = np.array([ELEMENTS[e][0] for e in self.els], dtype=float)
        self.n_e = float((self.n_at * self.z).sum())
        lnI = sum(n * z * math.log(ELEMENTS[e][2]) for e, n, z in zip(self.els, self.n_at, self.z))
        self.mean_exc = math.exp(lnI / self.n_e)
        self.inv_x0 = float(sum(n * _x0_per_atom(z) for n, z in zip(self.n_at, self.z)))


def _x0_per_atom(z: float) -> float:
    """Tsai radiation-length coefficient per atom [cm^2] (PDG 34.4.2)."""
    a2 = (ALPHA * z) ** 2
    fc = a2 * (1 / (1 + a2) + 0.20206 - 0.0369 * a2 + 0.0083 * a2 * a2 - 0.002 * a2 ** 3)
    if z == 1:
        lrad, lradp = 5.31, 6.144
    else:
        lrad = math.log(184.15 * z ** (-1 / 3))
        lradp = math.log(1194.0 * z ** (-2 / 3))
    return 4 * ALPHA * R_E * R_E * (z * z * (lrad - fc) + z * lradp)


# --------------------------------------------------------------------------
# Cross sections
# --------------------------------------------------------------------------
def kn_per_electron(e):
    """Total Klein-Nishina cross section per electron [cm^2]."""
    k = np.asarray(e, dtype=float) / M_E
    out = np.empty_like(k)
    small = k < 1e-3
    ks = k[small]
    out[small] = (8 * math.pi / 3) * R_E * R_E * (1 - 2 * ks + 5.2 * ks * ks)
    kb = k[~small]
    l = np.log1p(2 * kb)
    out[~small] = TWOPI_RE2 * ((1 + kb) / kb ** 2 * (2 * (1 + kb) / (1 + 2 * kb) - l / kb)
                               + l / (2 * kb) - (1 + 3 * kb) / (1 + 2 * kb) ** 2)
    return out


def pe_shells(z: int):
    """Synthetic photoelectric subshells: list of (binding [MeV], strength [b])."""
    ryd = 13.6057e-6
    shells = [(ryd * max(z - 1, 1) ** 2, 2000.0 * (82.0 / z) ** 2)]
    if z > 2:
        shells.append((ryd * max(z - 5, 1) ** 2 / 4, 3 * shells[0][1]))
    if z > 10:
        shells.append((ryd * max(z - 13, 1) ** 2 / 9, 6 * shells[0][1]))
    return shells


def pe_shell_coeffs(binding, strength):
    """Per-shell sigma(E) = a2/E^2 + a3/E^3 [b] as 1/E polynomial coefficients."""
    c = np.zeros(6)
    c[1] = 0.3 * strength * binding ** 2
    c[2] = 0.7 * strength * binding ** 3
    return c


def pe_micro(z: int, e):
    """Total synthetic photoelectric micro cross section [b]."""
    e = np.asarray(e, dtype=float)
    out = np.zeros_like(e)
    for b, s in pe_shells(z):
        c = pe_shell_coeffs(b, s)
        inv = 1 / e
        val = inv * (c[0] + inv * (c[1] + inv * (c[2] + inv * (c[3] + inv * (c[4] + inv * c[5])))))
        out += np.where(e >= b, val, 0.0)
    return out


def bh_micro(z: float, e):
    """Synthetic pair-production micro cross section [cm^2]."""
    e = np.asarray(e, dtype=float)
    thresh = 2 * M_E
    x = np.clip(1 - thresh / e, 0, None)
    return (7 / 9) * _x0_per_atom(z) * x ** 3 * (1 - 0.5 * np.exp(-e / 20.0))


def brems_shape(e, kc):
    """Integral of the complete-screening brems DCS above kc, in units of 1/X0."""
    e = np.asarray(e, dtype=float)
    out = np.zeros_like(e)
    ok = e > kc
    ee = e[ok]
    out[ok] = (4 / 3) * np.log(ee / kc) - (4 / 3) * (ee - kc) / ee + (ee * ee - kc * kc) / (2 * ee * ee)
    return out


def moller_per_electron(t, tc):
    """Moller cross section per target electron for delta rays above tc [cm^2]."""
    out = np.zeros_like(t)
    for i, ti in enumerate(t):
        xmin, xmax = tc / ti, 0.5
        if xmin >= xmax:
            continue
        gam = ti / M_E + 1
        g2 = gam * gam
        beta2 = 1 - 1 / g2
        gg = (2 * gam - 1) / g2
        cross = ((xmax - xmin) * (1 - gg + 1 / (xmin * xmax) + 1 / ((1 - xmin) * (1 - xmax)))
                 - gg * math.log(xmax * (1 - xmin) / (xmin * (1 - xmax)))) / beta2
        out[i] = cross * TWOPI_RE2 * M_E / ti
    return out


def bhabha_per_electron(t, tc):
    """Bhabha cross section per target electron for delta rays above tc [cm^2]."""
    out = np.zeros_like(t)
    for i, ti in enumerate(t):
        xmin, xmax = tc / ti, 1.0
        if xmin >= xmax:
            continue
        gam = ti / M_E + 1
        beta2 = 1 - 1 / (gam * gam)
        y = 1 / (1 + gam)
        y2 = y * y
        y12 = 1 - 2 * y
        b1 = 2 - y2
        b2 = y12 * (3 + y2)
        y122 = y12 * y12
        b4 = y122 * y12
        b3 = b4 + y122
        cross = ((xmax - xmin) * (1 / (beta2 * xmin * xmax) + b2 - 0.5 * b3 * (xmin + xmax)
                                  + b4 * (xmin * xmin + xmin * xmax + xmax * xmax) / 3)
                 - b1 * math.log(xmax / xmin))
        out[i] = cross * TWOPI_RE2 * M_E / ti
    return out


def coll_dedx(mat: Mat, t, tc, positron: bool):
    """Restricted Berger-Seltzer collision stopping power [MeV/cm] (no density effect)."""
    tlow = 10e-3
    out = np.zeros_like(t)
    eexc2 = (mat.mean_exc / M_E) ** 2

    def raw(ti):
        tau = ti / M_E
        gam = tau + 1
        beta2 = tau * (tau + 2) / (gam * gam)
        if positron:
            d = min(tc, ti) / M_E
            y = 1 / (1 + gam)
            d2 = d * d * 0.5
            d3 = d2 * d / 1.5
            d4 = d3 * d * 0.75
            f = (math.log(2 * (tau + 2) / eexc2) + math.log(tau * d)
                 - beta2 * (tau + 2 * d - y * (3 * d2 + y * (d - d3 + y * (d2 - tau * d3 + d4)))) / tau)
        else:
            d = min(tc, 0.5 * ti) / M_E
            f = (math.log(2 * (tau + 2) / eexc2) - 1 - beta2 + math.log((tau - d) * d)
                 + tau / (tau - d) + (0.5 * d * d + (2 * tau + 1) * math.log(1 - d / tau)) / (gam * gam))
        return max(f, 0.0) * TWOPI_RE2 * M_E * mat.n_e / beta2

    ref = raw(tlow)
    for i, ti in enumerate(t):
        out[i] = raw(ti) if ti >= tlow else ref * math.sqrt(ti / tlow)
    return out


def rad_dedx(mat: Mat, t, kc):
    """Restricted radiative stopping power for photon energies below kc [MeV/cm]."""
    k = np.minimum(kc, t)
    y = k / t
    return k * (4 / 3 - (2 / 3) * y + y * y / 3) * mat.inv_x0


def csda_range(e, dedx):
    """Range = integral of 1/dedx, trapezoid in energy; low end ~ sqrt(E) scaling."""
    r = np.empty_like(e)
    r[0] = 2 * e[0] / dedx[0]
    for i in range(1, len(e)):
        r[i] = r[i - 1] + 0.5 * (e[i] - e[i - 1]) * (1 / dedx[i] + 1 / dedx[i - 1])
    return r


def find_energy(e, f, target):
    """Energy where monotonically increasing f(e) reaches target (log interp)."""
    if f[0] >= target:
        return e[0]
    for i in range(1, len(e)):
        if f[i] >= target:
            lo, hi = math.log(f[i - 1]), math.log(f[i])
            frac = (math.log(target) - lo) / (hi - lo)
            return math.exp(math.log(e[i - 1]) + frac * (math.log(e[i]) - math.log(e[i - 1])))
    return e[-1]


def production_cuts(mat: Mat):
    """Synthetic range -> energy conversion for the 0.7 mm production cut."""
    e = log_grid(1e-4, 1e4)
    de = coll_dedx(mat, e, 1e30, positron=False) + rad_dedx(mat, e, 1e30)
    rng = csda_range(e, np.maximum(de, 1e-300))
    ecut = min(max(find_energy(e, rng, RANGE_CUT), 990e-6), 10e3)
    mu = (mat.n_e * kn_per_electron(e)
          + sum(n * pe_micro(int(z), e) * BARN for n, z in zip(mat.n_at, mat.z)))
    absl = 5 / np.maximum(mu, 1e-300)
    # Absorption length is not monotonic below the lowest shell edge: take the
    # highest energy at which five absorption lengths still fit in the cut.
    below = np.nonzero(absl < RANGE_CUT)[0]
    gcut = e[below[-1]] if len(below) else e[0]
    gcut = min(max(gcut, 990e-6), 10e3)
    return {11: ecut, -11: ecut, 22: gcut}


# --------------------------------------------------------------------------
# Writer
# --------------------------------------------------------------------------
class Writer:
    def __init__(self):
        self.lines = []

    def put(self, key, values):
        if isinstance(values, (str, int, float, np.floating, np.integer)):
            values = [values]
        toks = []
        for v in values:
            if isinstance(v, str):
                assert " " not in v
                toks.append(v)
            elif isinstance(v, (int, np.integer)):
                toks.append(str(int(v)))
            else:
                toks.append(repr(float(v)))
        self.lines.append(f"{key} {len(toks)} " + " ".join(toks))

    def text(self):
        return "\n".join(self.lines) + "\n"


def generate(problem: str) -> str:
    mats = [Mat(n) for n in PROBLEMS[problem]]
    el_names = []
    for m in mats:
        for e in m.els:
            if e not in el_names:
                el_names.append(e)
    el_names.sort(key=lambda n: ELEMENTS[n][0])
    w = Writer()
    w.put("format", "gbx-physics-1")
    w.put("units", "cgs")
    w.put("problem", problem)

    # Elements
    w.put("elements", len(el_names))
    for i, n in enumerate(el_names):
        z, a, _ = ELEMENTS[n]
        w.put(f"element.{i}.name", n)
        w.put(f"element.{i}.z", z)
        w.put(f"element.{i}.a", a)

    # Materials
    cuts = []
    w.put("materials", len(mats))
    for i, m in enumerate(mats):
        w.put(f"material.{i}.name", m.name)
        w.put(f"material.{i}.state", m.state)
        w.put(f"material.{i}.temperature", 293.15)
        w.put(f"material.{i}.number_density", m.number_density)
        w.put(f"material.{i}.elements", [el_names.index(e) for e in m.els])
        w.put(f"material.{i}.fractions", m.frac)
        c = production_cuts(m)
        cuts.append(c)
        for pdg in (11, -11, 22):
            w.put(f"material.{i}.cut.{pdg}", [c[pdg], RANGE_CUT])

    # Particles (PDG, mass, charge, spin)
    parts = [("e-", 11, M_E, -1, 0.5), ("e+", -11, M_E, 1, 0.5), ("gamma", 22, 0.0, 0, 1)]
    w.put("particles", len(parts))
    for i, (n, pdg, mass, q, s) in enumerate(parts):
        w.put(f"particle.{i}", [n, pdg, mass, q, s])

    # Parameters
    w.put("em.energy_loss_fluct", 1)
    w.put("em.lpm", 1)
    w.put("em.integral_approach", 1)
    w.put("em.linear_loss_limit", 0.01)
    w.put("em.lowest_electron_energy", 0.001)
    w.put("em.msc_range_factor", 0.04)
    w.put("em.msc_safety_factor", 0.6)
    w.put("em.msc_lambda_limit", 0.1)
    w.put("trans.looping", [11, 10, 250.0, -11, 10, 250.0, 22, 10, 250.0])
    w.put("trans.max_substeps", 1000)

    egrid = log_grid(E_MIN, E_MAX)
    bhgrid = log_grid(2 * M_E, E_MAX)

    def table(key, x, y):
        w.put(key + ".x", x)
        w.put(key + ".y", y)

    for mi, m in enumerate(mats):
        # --- gamma
        table(f"table.22.compton.lambda.{mi}", egrid, m.n_e * kn_per_electron(egrid))
        pe = sum(n * pe_micro(int(z), egrid) * BARN for n, z in zip(m.n_at, m.z))
        table(f"table.22.photoelectric.lambda.{mi}", egrid, pe)
        bh = sum(n * bh_micro(z, bhgrid) for n, z in zip(m.n_at, m.z))
        table(f"table.22.conversion.lambda.{mi}", bhgrid, bh)
        w.put(f"model.22.conversion.bethe_heitler.{mi}.energy", bhgrid)
        for ei, z in enumerate(m.z):
            w.put(f"model.22.conversion.bethe_heitler.{mi}.micro.{ei}", bh_micro(z, bhgrid))
        # --- e-, e+
        ecut, gcut = cuts[mi][11], cuts[mi][22]
        for pdg in (11, -11):
            pos = pdg < 0
            # Discrete-process tables start at their production threshold
            # (cross section exactly zero there), so interpolation never gives
            # a cross section below the threshold
            ioni_grid = log_grid(ecut if pos else 2 * ecut, E_MAX)
            per_e = (bhabha_per_electron(ioni_grid, ecut) if pos
                     else moller_per_electron(ioni_grid, ecut))
            per_e[0] = 0.0
            table(f"table.{pdg}.e_ioni.lambda.{mi}", ioni_grid, m.n_e * per_e)
            dedx = coll_dedx(m, egrid, ecut, pos) + rad_dedx(m, egrid, gcut)
            dedx = np.maximum(dedx, 1e-300 if m.density < 1e-10 else 0)
            table(f"table.{pdg}.e_ioni.dedx.{mi}", egrid, dedx)
            table(f"table.{pdg}.e_ioni.range.{mi}", egrid, csda_range(egrid, dedx))
            brems_grid = log_grid(gcut, E_MAX)
            brems_xs = m.inv_x0 * brems_shape(brems_grid, gcut)
            brems_xs[0] = 0.0
            table(f"table.{pdg}.e_brems.lambda.{mi}", brems_grid, brems_xs)
            for model in ("e_brems_sb", "e_brems_lpm"):
                w.put(f"model.{pdg}.e_brems.{model}.{mi}.energy", egrid)
                for ei, z in enumerate(m.z):
                    w.put(f"model.{pdg}.e_brems.{model}.{mi}.micro.{ei}",
                          _x0_per_atom(z) * brems_shape(egrid, gcut))
            # Urban MSC: lambda_1 transport mean free path scaled by E^2
            # (screened Rutherford, Wentzel screening), "msc_xs" table
            zeff2 = float((m.n_at * m.z * (m.z + 1)).sum())
            tau = egrid / M_E
            p2 = egrid * (egrid + 2 * M_E)
            beta2 = p2 / (egrid + M_E) ** 2
            zbar = max(float((m.frac * m.z).sum()), 1.0)
            scr = 1.13 * (ALPHA * zbar ** (1 / 3) / 0.885) ** 2 * M_E * M_E / p2 * 0.25
            scr = scr * (1.13 + 3.76 * (ALPHA * zbar) ** 2 / beta2)
            sig_tr = 2 * math.pi * R_E * R_E * (M_E * M_E / (beta2 * p2)) * (
                np.log1p(1 / scr) - 1 / (1 + scr))
            lam1_inv = zeff2 * sig_tr
            table(f"msc.{pdg}.{mi}", egrid, np.maximum(lam1_inv, 1e-300) * egrid * egrid)
            del tau

    # Seltzer-Berger synthetic scaled DCS (in mb), per element
    sb_x = np.log(np.logspace(-3, 4, 57))
    sb_y = np.array([1e-12, 0.025, 0.05, 0.075, 0.1, 0.15, 0.2, 0.25, 0.3, 0.35, 0.4,
                     0.45, 0.5, 0.55, 0.6, 0.65, 0.7, 0.75, 0.8, 0.85, 0.9, 0.925, 0.95,
                     0.97, 0.99, 0.995, 0.999, 0.9995, 0.9999, 0.99995, 0.99999, 1.0])
    for n in el_names:
        z = ELEMENTS[n][0]
        le = np.log10(np.exp(sb_x))
        amp = (6.0 + 1.2 * (le + 3)) * (1 + 0.004 * (z - 29))
        shape = 4 / 3 - 4 / 3 * sb_y + sb_y * sb_y
        soft = 1 + 0.15 * (1 - sb_y) * np.exp(-((le[:, None] + 1) ** 2) / 4)
        val = amp[:, None] * shape[None, :] * soft
        w.put(f"sb.{z}.x", sb_x)
        w.put(f"sb.{z}.y", sb_y)
        w.put(f"sb.{z}.value", val.ravel())

    # Livermore photoelectric synthetic data, per element
    for n in el_names:
        z = ELEMENTS[n][0]
        shells = pe_shells(z)
        b_front, b_back = shells[0][0], shells[-1][0]
        thresh_lo = max(2 * b_front, 1e-3)
        thresh_hi = 10 * thresh_lo
        w.put(f"livermore.{z}.thresh", [thresh_lo, thresh_hi])
        ehi = np.geomspace(b_front, thresh_lo, 24)
        w.put(f"livermore.{z}.xs_hi.x", ehi)
        w.put(f"livermore.{z}.xs_hi.y", pe_micro(z, ehi) * ehi ** 3)
        if len(shells) > 1:
            elo = np.geomspace(b_back, b_front * (1 - 1e-9), 16)
            w.put(f"livermore.{z}.xs_lo.x", elo)
            w.put(f"livermore.{z}.xs_lo.y", pe_micro(z, elo) * elo ** 3)
        w.put(f"livermore.{z}.shells", len(shells))
        cum = np.zeros(6)
        for si, (b, s) in enumerate(shells):
            c = pe_shell_coeffs(b, s)
            cum = cum + c
            w.put(f"livermore.{z}.shell.{si}.binding", b)
            w.put(f"livermore.{z}.shell.{si}.param_lo", cum)
            w.put(f"livermore.{z}.shell.{si}.param_hi", cum)
            es = np.geomspace(b, thresh_lo, 12)
            inv = 1 / es
            sig = inv * (c[0] + inv * (c[1] + inv * (c[2] + inv * (c[3] + inv * (c[4] + inv * c[5])))))
            w.put(f"livermore.{z}.shell.{si}.energy", es)
            w.put(f"livermore.{z}.shell.{si}.xs", sig * es ** 3)
    return w.text()


def main():
    here = os.path.dirname(os.path.abspath(__file__))
    for prob in PROBLEMS:
        with open(os.path.join(here, f"{prob}.physics.txt"), "w") as f:
            f.write(generate(prob))


if __name__ == "__main__":
    main()
