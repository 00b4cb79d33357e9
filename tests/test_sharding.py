"""Events sharded over ranks: the N>1 path of bench.py, run as two gloo
ranks on the CPU (one process per GPU in production, NCCL there; the
reduction is the same code with CPU buffers)."""

from __future__ import annotations

import os
import socket

import numpy as np
import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, workload, queue):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist

    from celeritas_gb300 import sharding
    from celeritas_gb300.workloads import WORKLOADS

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        wl = WORKLOADS[workload]
        prim = sharding.rank_primaries(wl, rank, num=40)
        lo, hi = sharding.event_range(wl, rank)
        mine = {"events": sorted(set(int(e) for e in prim["event"])), "lo": lo, "hi": hi,
                "energy": prim["energy"].tolist()}
        everyone = [None] * world
        dist.all_gather_object(everyone, mine)
        # Per-rank figures that make the expected reduction obvious
        tallies = np.arange(8, dtype=np.float64) * (rank + 1)
        red = sharding.reduce_run(dist, "cpu", time_ms=100.0 + 10 * rank,
                                  e2e_s=2.0 - rank, track_steps=1000.0 * (rank + 1),
                                  tallies=tallies)
        red["tallies"] = red["tallies"].tolist()
        queue.put((rank, everyone, red))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("workload", ["c2", "c3"])
def test_two_rank_sharding_and_reduction(workload):
    import torch.multiprocessing as mp

    world = 2
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, workload, queue))
             for r in range(world)]
    for p in procs:
        p.start()
    results = {}
    for _ in range(world):
        rank, everyone, red = queue.get(timeout=120)
        results[rank] = (everyone, red)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0

    everyone, _ = results[0]
    ev0, ev1 = set(everyone[0]["events"]), set(everyone[1]["events"])
    # Each rank's events lie in its own range, so no event is transported twice
    assert not ev0 & ev1
    for info in everyone:
        assert all(info["lo"] <= e < info["hi"] for e in info["events"])
    # Independent primaries: the ranks' beams are not copies of each other
    assert everyone[0]["energy"] != everyone[1]["energy"]

    for rank in range(world):
        _, red = results[rank]
        # Job time = slowest rank; throughput counts every rank's steps
        assert red["time_ms"] == pytest.approx(110.0)
        assert red["e2e_s"] == pytest.approx(2.0)
        assert red["track_steps"] == pytest.approx(3000.0)
        np.testing.assert_allclose(red["tallies"], np.arange(8) * 3.0)


def test_single_process_reduction_is_identity():
    from celeritas_gb300 import sharding

    red = sharding.reduce_run(None, "cpu", 5.0, 0.5, 123.0, np.ones(3))
    assert (red["time_ms"], red["e2e_s"], red["track_steps"]) == (5.0, 0.5, 123.0)
    np.testing.assert_array_equal(red["tallies"], np.ones(3))


@pytest.mark.parametrize("steps", [1, 3, 10, 20, 25])
def test_bench_batches_cover_every_event(steps):
    """The timed bench steps of a batched workload transport every event of
    the configuration: batches of max(65, ceil(1300 / steps)) consecutive
    events, the warm-up batch of other events."""
    import numpy as np

    from celeritas_gb300.workloads import WORKLOADS, step_batches

    wl = WORKLOADS["c3"]
    batches, warm = step_batches(wl, 0, steps)
    assert len(batches) == steps
    per_event = wl["num_primaries"] // wl["events"]
    size = max(wl["events_per_step"], -(-wl["events"] // steps))
    first = min(steps, -(-wl["events"] // size))
    events = np.concatenate([b["event"] for b in batches[:first]])
    assert len(np.unique(events)) == wl["events"]
    assert all(len(b) <= size * per_event for b in batches)
    assert len(warm) == size * per_event
    assert not np.array_equal(warm["energy"], batches[0]["energy"])
