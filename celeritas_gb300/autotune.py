"""Autotuner for batched transport of many uneven events.

The launch configuration of a stepper changes its speed but not its results
when every track has its own random stream (rng_per_track): the same
calibration events then cost the same physics work under every candidate, so
their transport times compare directly. The tuner runs a coordinate descent
over

* the number of track slots (one stepper per candidate),
* threads per block of the charged along-step kernel (64, 128, 256 and 512,
  the last from kernel instances whose registers are capped at 128 per
  thread) together with its form, a persistent kernel or one thread per track
  (the best block size differs between the two forms, so they are tuned as
  pairs); a setting the stepper rejects is recorded and skipped,
* the sort threshold: action sorts only in steps that start with at least
  this many live tracks (0: always),
* the along-step sort by material within the charged tracks, and within the
  neutral ones too (off, charged, both),

keeping the best value of each parameter before tuning the next. Every
candidate first transports the calibration events once untimed (a new
setting may capture new CUDA graphs), then once timed.
"""

from __future__ import annotations

import dataclasses
import time
from typing import Callable, Sequence

import numpy as np

SLOT_COUNTS = (1 << 20, 1 << 21, 1 << 22)
BLOCK_SIZES = (64, 128, 256, 512)
THRESHOLDS = (0, 1 << 14, 1 << 17)


@dataclasses.dataclass
class Trial:
    config: dict
    seconds: float | None
    track_steps: int | None
    note: str = ""

    @property
    def rate(self) -> float:
        return self.track_steps / self.seconds if self.seconds else 0.0


def transport(stepper, primaries, max_steps: int = 20000) -> tuple[float, int]:
    """Seconds and track-steps to transport the primaries to completion."""
    stepper.synchronize()
    t0 = time.perf_counter()
    res = [stepper.step(primaries)] + stepper.run(max_steps=max_steps, batch=64)
    stepper.synchronize()
    seconds = time.perf_counter() - t0
    if res[-1].alive or res[-1].queued:
        raise RuntimeError("calibration transport did not finish")
    return seconds, sum(r.active for r in res)


def autotune(make_stepper: Callable[[int], object], primaries: np.ndarray,
             slot_counts: Sequence[int] = SLOT_COUNTS,
             block_sizes: Sequence[int] = BLOCK_SIZES,
             thresholds: Sequence[int] = THRESHOLDS,
             start: dict | None = None,
             materials: Sequence[int] = (0, 1, 3)) -> tuple[dict, list[Trial]]:
    """Tune on 'primaries'; return the best configuration and every trial."""
    trials: list[Trial] = []
    best = dict(start or {})
    best.setdefault("slots", slot_counts[len(slot_counts) // 2])

    def run(stepper, config):
        settings = {k: v for k, v in config.items() if k != "slots"}
        try:
            stepper.set_tuning(**settings)
        except RuntimeError as e:
            trials.append(Trial(dict(config), None, None, str(e)))
            return None
        transport(stepper, primaries)  # warm-up: graph capture for the setting
        seconds, steps = transport(stepper, primaries)
        trial = Trial(dict(config), seconds, steps)
        trials.append(trial)
        return trial

    # Slot count: one stepper per candidate, warmed up once
    winner = None
    for slots in slot_counts:
        stepper = make_stepper(slots)
        config = dict(best, slots=slots)
        transport(stepper, primaries)  # warm-up (graph capture, first touch)
        t = run(stepper, config)
        if t and (winner is None or t.seconds < winner.seconds):
            winner = t
        del stepper
    best = dict(winner.config)
    stepper = make_stepper(best["slots"])
    transport(stepper, primaries)

    stages = (
        [{"along_block_size": b, "along_persistent": f} for f in (1, 0) for b in block_sizes],
        [{"sort_threshold": v} for v in thresholds],
        [{"sort_material": v} for v in materials],
    )
    for candidates in stages:
        winner = None
        for settings in candidates:
            t = run(stepper, dict(best, **settings))
            if t and (winner is None or t.seconds < winner.seconds):
                winner = t
        if winner is not None:
            best = dict(winner.config)
    return best, trials
