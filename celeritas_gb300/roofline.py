"""Algorithmic bytes per track slot for each step action (HBM roofline).

Each entry counts the bytes of persistent per-slot state an action must read
and write once for one active track, from the sizes of the structure-of-arrays
fields it touches (FP64 physics layout: reals 8 B, IDs 4 B, status 1 B,
XORWOW state 24 B read + 24 B written when the action samples). Inactive
slots cost the 1-byte status (or 4-byte action ID) check only. Physics tables
are read-only, L2/shared-memory resident and excluded, as in the reference
sizing of the track state.

The roofline figure for a kernel is
    bytes per launch = active * bytes_active + inactive * bytes_idle
divided by its CUDA-event launch time.
"""

from __future__ import annotations

# action label -> (bytes per active slot, bytes per idle slot)
ACTION_BYTES = {
    # reads status, particle, material, energy, mfp, volume (29);
    # rng (48); writes status, edep, secondary span, element, per-process
    # xs (3 x 8), macro xs, range, step, actions, mfp, detector (93)
    "pre-step": (170, 1),
    # reads status, action, step, pos, dir, volume, surface, sense, boundary,
    # particle, material, energy, post action, mfp, macro xs, range, time,
    # num steps, edep (153); rng (48); writes pos, surface, sense, next
    # step/surface/sense, step, post action, time, energy, edep, status,
    # mfp, num steps (91)
    "along-step-general-linear": (292, 5),
    "along-step-neutral": (292, 5),
    # as above, plus the multiple-scattering step-limit state (range at
    # the volume entry, range factor, minimum limit: 24 B read + written)
    # and the looping-step counter (4 + 4)
    "along-step-uniform-msc": (348, 5),
    # reads post action, particle, material, energy, macro + per-process xs
    # (52); rng (48); writes mfp, post action, element (16)
    "physics-discrete-select": (116, 4),
    # interacting slot: reads particle, material, energy, dir, element,
    # surface, boundary (53); rng (48); writes energy, dir, boundary,
    # status, edep, secondary span (50); ~1.3 secondaries x 32 B (42)
    "model": (197, 4),
    # crossing slot: pos, surface, sense, boundary, volume (34) -> sense,
    # boundary, volume, material, status (11)
    "geo-boundary": (49, 4),
    "tracking-cut": (29, 4),
    # status, detector, edep (13) -> one atomic add (8)
    "step-gather-post": (21, 1),
    # locate (status, secondary span, secondaries), scan, scatter
    # (vacancy, initializers 72 B per secondary, in-place reuse ~150 B)
    "extend-from-secondaries": (120, 10),
    # initializer (72) -> slot sim/particle/geometry/material/physics (~160)
    "initialize-tracks": (232, 0),
}

MODEL_ACTIONS = {"ioni-moller-bhabha", "brems-sb", "brems-rel", "photoel-livermore",
                 "scat-klein-nishina", "conv-bethe-heitler", "annihil-2-gamma"}


def bytes_per_slot(label: str) -> tuple[int, int]:
    if label in MODEL_ACTIONS:
        return ACTION_BYTES["model"]
    return ACTION_BYTES.get(label, (0, 0))


def launch_bytes(label: str, active: int, slots: int) -> int:
    """Algorithmic bytes for one launch of an action over 'slots' slots."""
    b_active, b_idle = bytes_per_slot(label)
    return active * b_active + (slots - active) * b_idle


# Persistent per-slot state of this build's FP64 layout (bytes), for the
# per-track-step figure: read once + written once per step
STATE_BYTES_PER_SLOT = (
    1 + 4 * 4 + 8 * 2 + 4 * 2   # sim: status, ids, steps, time, step, actions
    + 4 + 8                     # particle
    + 8 * 6 + 4 * 2 + 1 * 3 + 8 + 4 + 1 + 1  # geometry
    + 4                         # material
    + 8 * 3 + 8 * 4 + 8 + 4 * 3  # physics (mfp, range, macro, per-process, edep, spans)
    + 24                        # rng
    + 4 * 3 + 4                 # init bookkeeping, detector
)
B_STEP = 2 * STATE_BYTES_PER_SLOT
