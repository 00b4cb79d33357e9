"""The autotuner's search on the host, with a fake stepper whose transport
times are a known function of the launch configuration (no GPU)."""

from __future__ import annotations

import numpy as np

from celeritas_gb300 import autotune


class _Result:
    active, alive, queued = 100, 0, 0


class FakeStepper:
    """Transport time from a table over (slots, block, persistent, threshold);
    a setting the table marks None is rejected like an invalid block size."""

    clock = 0.0

    def __init__(self, slots, cost):
        self.slots = slots
        self.cost = cost
        self.cfg = {"along_block_size": 256, "along_persistent": 1, "sort_threshold": 0,
                    "sort_material": 0}
        self.calls = []

    def set_tuning(self, **settings):
        trial = dict(self.cfg, **settings)
        if self.cost(self.slots, trial) is None:
            raise RuntimeError(f"invalid setting {settings}")
        self.cfg = trial
        self.calls.append(dict(settings))

    def synchronize(self):
        pass

    def step(self, primaries=None):
        FakeStepper.clock += self.cost(self.slots, self.cfg)
        return _Result()

    def run(self, max_steps, batch):
        return [_Result()]


def _patch_clock(monkeypatch):
    monkeypatch.setattr(autotune.time, "perf_counter", lambda: FakeStepper.clock)


def test_block_size_and_kernel_form_tuned_together(monkeypatch):
    _patch_clock(monkeypatch)

    # The persistent kernel is best at 64 threads, one thread per track at
    # 128, and the latter is faster overall: tuning the block size with the
    # persistent kernel on and then the form would end at (64, 0)
    def cost(slots, c):
        b, f = c["along_block_size"], c["along_persistent"]
        if b == 512:
            return None
        table = {(64, 1): 1.8, (128, 1): 1.9, (256, 1): 2.0,
                 (64, 0): 1.85, (128, 0): 1.5, (256, 0): 1.7}
        thr = {0: 0.2, 1 << 14: 0.1, 1 << 17: 0.0}[c["sort_threshold"]]
        return table[(b, f)] + thr + (0.0 if slots == 1 << 21 else 0.3)

    best, trials = autotune.autotune(lambda n: FakeStepper(n, cost), np.zeros(4))
    assert best == {"slots": 1 << 21, "along_block_size": 128, "along_persistent": 0,
                    "sort_threshold": 1 << 17, "sort_material": 0}
    rejected = [t for t in trials if t.seconds is None]
    assert [t.config["along_block_size"] for t in rejected] == [512, 512]
    # Every measured candidate was timed after an untimed warm-up transport
    measured = [t for t in trials if t.seconds is not None]
    assert all(t.rate > 0 for t in measured)


def test_start_configuration_kept_when_nothing_is_faster(monkeypatch):
    _patch_clock(monkeypatch)

    def cost(slots, c):
        if c["along_block_size"] == 512:
            return None
        return 1.0  # every candidate ties: the first of each stage wins

    best, _ = autotune.autotune(lambda n: FakeStepper(n, cost), np.zeros(1),
                                slot_counts=(1 << 20,), block_sizes=(256, 512),
                                thresholds=(0, 1 << 14))
    assert best == {"slots": 1 << 20, "along_block_size": 256, "along_persistent": 1,
                    "sort_threshold": 0, "sort_material": 0}


def test_material_sort_taken_when_faster(monkeypatch):
    _patch_clock(monkeypatch)

    def cost(slots, c):
        if c["along_block_size"] == 512:
            return None
        return {0: 1.0, 1: 0.95, 3: 0.97}[c["sort_material"]]

    best, trials = autotune.autotune(lambda n: FakeStepper(n, cost), np.zeros(1),
                                     slot_counts=(1 << 20,), block_sizes=(256,),
                                     thresholds=(0,))
    assert best["sort_material"] == 1
    assert [t.config.get("sort_material") for t in trials][-3:] == [0, 1, 3]
