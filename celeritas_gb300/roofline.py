"""Algorithmic bytes per track slot for each step action (HBM roofline).

Each entry counts the bytes of persistent per-slot state an action must read
and write once for one track it processes, from the sizes of the
structure-of-arrays fields it touches: a fixed part (IDs 4 B, status and
flags 1 B, FP64 positions/directions/time/step 8 B, XORWOW state 24 B read +
24 B written when the action samples) and a number of physics reals (energy,
cross sections, MFP, range, deposition, multiple-scattering state), which are
8 B in the FP64 build and 4 B in the mixed-precision build. A slot that the
launch visits but does not process costs the idle bytes (its status or
action ID). Physics tables are read-only, L2-resident and excluded, as in
the reference's sizing of the track state.

The roofline figure for a kernel is
    bytes per launch = processed * bytes_processed + idle * bytes_idle
divided by its CUDA-event launch time.
"""

from __future__ import annotations

# action label -> (fixed bytes, physics reals, idle bytes) per slot
ACTION_BYTES = {
    # reads status, particle, material, volume, rng; writes status, secondary
    # span, element, step (FP64), actions, detector | reals: energy, MFP (r/w),
    # deposition, 4 per-process XS, macro XS, range
    "pre-step": (94, 10, 1),
    # charged, straight line: status, actions, step, pos, dir, geometry
    # state, particle, material, time, steps, rng; writes pos, geometry
    # state, step, action, time, steps | reals: energy (r/w), MFP (r/w),
    # macro XS, range, deposition (r/w)
    "along-step-general-linear": (203, 8, 5),
    # as above plus the field/MSC state: looping counter (r/w) and
    # multiple-scattering range, factor, minimum limit (r/w) and true path,
    # geometric path, slope (r/w)
    "along-step-uniform-msc": (243, 17, 5),
    # the same state in an R-Z map field (the map itself is a read-only table)
    "along-step-rzmap-msc": (243, 17, 5),
    # photons: no random numbers, no energy loss | reals: energy, MFP (r/w),
    # macro XS
    "along-step-neutral": (158, 4, 5),
    # reads action, particle, material, rng; writes action, element |
    # reals: energy, macro XS, up to 4 per-process XS, MFP (w)
    "physics-discrete-select": (68, 7, 4),
    # interacting slot: particle, material, dir (r/w), element, action, rng,
    # status, secondary span, ~1.3 secondaries x 4 B ID | reals: energy
    # (r/w), deposition, ~1.3 secondaries x (energy + 3 direction)
    "model": (126, 8, 4),
    # crossing slot: pos, surface, sense, boundary, volume -> sense,
    # boundary, volume, material, status
    "geo-boundary": (45, 0, 4),
    "tracking-cut": (6, 4, 4),
    # status, detector, deposition -> one atomic add (8)
    "step-gather-post": (13, 1, 1),
    # locate (status, secondary span), scan, scatter (vacancy, initializers
    # 88 B per secondary, in-place reuse)
    "extend-from-secondaries": (120, 0, 10),
    # initializer (88 B) -> slot sim/particle/geometry/material/physics
    "initialize-tracks": (200, 4, 0),
    # action key (4) read twice, thread->slot index (4) written
    "sort-tracks-along-step": (12, 0, 12),
    "sort-tracks-post-step": (12, 0, 12),
}

MODEL_ACTIONS = {"ioni-moller-bhabha", "brems-sb", "brems-rel", "photoel-livermore",
                 "scat-klein-nishina", "conv-bethe-heitler", "annihil-2-gamma"}


def bytes_per_slot(label: str, real_bytes: int = 8) -> tuple[int, int]:
    """(bytes per processed slot, bytes per idle slot) of an action."""
    key = "model" if label in MODEL_ACTIONS else label
    fixed, nreal, idle = ACTION_BYTES.get(key, (0, 0, 0))
    return fixed + nreal * real_bytes, idle


def launch_bytes(label: str, processed: int, slots: int, real_bytes: int = 8) -> int:
    """Algorithmic bytes for one launch of an action over 'slots' slots."""
    b_proc, b_idle = bytes_per_slot(label, real_bytes)
    return processed * b_proc + (slots - processed) * b_idle
