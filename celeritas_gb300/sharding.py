"""Events sharded over ranks (one process per GPU) and the end-of-run reduction.

Events are independent: a shower's tracks interact only through its own
secondaries, and the parameters (tables, geometry) are read-only, so each rank
owns a stepper and transports its own events, as celer-sim gives each stream
its own events (app/celer-sim/celer-sim.cc:126-138). Nothing is exchanged on
the data path; the only collective is the final reduction of the timings,
track-step counts and per-detector tallies.

Rank r takes the workload's primaries with event IDs offset by
r * (events of the workload) and its beam seed offset by 1000 * r, so the
ranks' events are disjoint and their primaries independent.
"""

from __future__ import annotations

import numpy as np

from .workloads import make_primaries


def rank_primaries(wl: dict, rank: int, num: int | None = None):
    """Primaries of the events that 'rank' transports."""
    return make_primaries(wl, rank, num=num)


def event_range(wl: dict, rank: int) -> tuple[int, int]:
    """Half-open range of event IDs that 'rank' may use."""
    return rank * wl["events"], (rank + 1) * wl["events"]


def reduce_run(dist, device, time_ms: float, e2e_s: float, track_steps: float,
               tallies=None) -> dict:
    """Whole-job totals over ranks: the slowest rank's device and host times
    (the job ends when its last rank does), the summed track-steps and the
    summed per-detector energy deposition. 'dist' is torch.distributed (or
    None for one process); 'device' holds the reduction buffers (a CUDA
    device under NCCL, 'cpu' under gloo)."""
    out = {"time_ms": float(time_ms), "e2e_s": float(e2e_s),
           "track_steps": float(track_steps),
           "tallies": None if tallies is None else np.asarray(tallies, dtype=np.float64)}
    if dist is None:
        return out
    import torch

    t = torch.tensor([time_ms, e2e_s], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    out["time_ms"], out["e2e_s"] = (float(v) for v in t.tolist())
    st = torch.tensor([track_steps], device=device, dtype=torch.float64)
    dist.all_reduce(st, op=dist.ReduceOp.SUM)
    out["track_steps"] = float(st.item())
    if tallies is not None:
        tl = torch.as_tensor(np.asarray(tallies, dtype=np.float64)).to(device)
        dist.all_reduce(tl, op=dist.ReduceOp.SUM)
        out["tallies"] = tl.cpu().numpy()
    return out
