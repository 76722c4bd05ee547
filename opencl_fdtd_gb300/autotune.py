"""Tile-shape autotuner of the batched path (BatchSimulation).

A batch cuts every variant into tiles of 256 (y, z) cells times ``xchunk`` x planes and runs
them either as one launch per half-step (one block per tile) or as one persistent cooperative
launch with ``blocks_per_sm`` resident blocks per SM. The best choice depends on the mix of
grid shapes (tile count against the grid's concurrency, x-neighbour reuse against tail
imbalance), so ``tune_batch`` times each candidate on the batch itself (CUDA events around a
short run on the batch's stream, after a warm-up run), keeps the fastest, and restores the
simulations' state afterwards so tuning changes no result. Choices are remembered per
(device, storage, shapes) in memory and, when ``cache_path`` is given or
``OPENCL_FDTD_GB300_TUNE_CACHE`` names a file, in a JSON file.
"""
from __future__ import annotations

import json
import os

XCHUNKS = (2, 4, 8, 16, 32)
BLOCKS_PER_SM = (1, 2)
SCHEDULES = ("launches", "persistent")

_MEMO: dict = {}


def _key(batch) -> str:
    import torch
    name = torch.cuda.get_device_name(batch.device)
    shapes = ";".join("x".join(str(s) for s in sim.shape) for sim in batch.sims)
    return "%s|%s|%s" % (name, batch.storage, shapes)


def _load(path):
    if path and os.path.exists(path):
        try:
            with open(path) as f:
                return json.load(f)
        except (OSError, ValueError):
            return {}
    return {}


def _snapshot(batch):
    st = []
    for sim in batch.sims:
        st.append(({k: getattr(sim, k).clone() for k in ("E", "H")},
                   [[(u.clone(), v.clone()) for u, v in sim.psi[f]] for f in ("E", "H")],
                   sim.steps_run))
    extra = [t.clone() for t in batch._e16 + batch._h16 + batch._eexp + batch._hexp]
    series = [s.clone() if s is not None else None for s in batch.series]
    return st, extra, series, batch.step_counter(), batch.steps_run


def _restore(batch, snap):
    st, extra, series, step, steps_run = snap
    for sim, (fields, psi, sr) in zip(batch.sims, st):
        for k, t in fields.items():
            getattr(sim, k).copy_(t)
        for f, pairs in zip(("E", "H"), psi):
            for (u, v), (u0, v0) in zip(sim.psi[f], pairs):
                u.copy_(u0)
                v.copy_(v0)
        sim.steps_run = sr
    for t, t0 in zip(batch._e16 + batch._h16 + batch._eexp + batch._hexp, extra):
        t.copy_(t0)
    for s, s0 in zip(batch.series, series):
        if s is not None:
            s.copy_(s0)
    batch.set_step_counter(step)
    batch.steps_run = steps_run


def time_config(batch, xchunk: int, blocks_per_sm: int, steps: int, schedule: str = None) -> float:
    """ms per step of one tile configuration (the batch state advances)."""
    import torch
    batch.tune(xchunk, blocks_per_sm, schedule)
    batch.run(2)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(batch.queue):
        e0.record(batch.queue)
        batch.run(steps)
        e1.record(batch.queue)
    e1.synchronize()
    return e0.elapsed_time(e1) / steps


def tune_batch(batch, steps: int = 10, cache_path: str | None = None, xchunks=XCHUNKS,
               blocks=BLOCKS_PER_SM, schedules=SCHEDULES, force: bool = False) -> dict:
    """Pick and apply the fastest (xchunk, blocks_per_sm); returns the choice and the timings.
    The simulations' fields, CPML state, monitor series and step counters are restored."""
    import torch
    cache_path = cache_path or os.environ.get("OPENCL_FDTD_GB300_TUNE_CACHE")
    key = _key(batch)
    disk = _load(cache_path)
    hit = None if force else (_MEMO.get(key) or disk.get(key))
    if hit is not None:
        batch.tune(hit["xchunk"], hit["blocks_per_sm"], hit.get("schedule"))
        return dict(hit, cached=True)
    snap = _snapshot(batch)
    timings = {}
    for sched in schedules:
        for xc in xchunks:
            for b in (blocks if sched == "persistent" else (0,)):
                timings["%s,%d,%d" % (sched, xc, b)] = time_config(batch, xc, b, steps, sched)
    best = min(timings, key=timings.get)
    sched, xc, b = best.split(",")
    xc, b = int(xc), int(b)
    _restore(batch, snap)
    torch.cuda.synchronize(batch.device)
    batch.tune(xc, b, sched)
    choice = {"schedule": sched, "xchunk": xc, "blocks_per_sm": b, "ms_per_step": timings[best],
              "timings": timings}
    _MEMO[key] = choice
    if cache_path:
        disk[key] = choice
        try:
            os.makedirs(os.path.dirname(os.path.abspath(cache_path)), exist_ok=True)
            with open(cache_path, "w") as f:
                json.dump(disk, f, indent=1)
        except OSError:
            pass
    return dict(choice, cached=False)
