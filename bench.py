#!/usr/bin/env python
"""
Benchmark of the FDTD time-stepping hot path on GB300.

Workload (default c2): the reference README's 395x345x73 grid (~10M cells), float32, as a
seeded L3 photonic-crystal slab cavity with 8-cell CPML on all six faces, an Ey Gaussian
point source and the Poynting vector on. One step = update_E, the soft source add,
update_H and update_S over the whole grid (the loop of opencl_fdtd's fdtd.py:162-175).
Inputs (~1 GB of fields) are far larger than the 129 MB L2, so no flush is needed between
steps.

Printed as one JSON line:
  value       Mcell-updates/s with every buffer resident in HBM (device-timed, CUDA events)
  e2e         the same metric through the public Simulation API, with the per-step source
              sample copied host->device from pinned memory and one field sample read back
  roofline    the dominant kernel's algorithmic bytes per launch / its mean event-timed
              duration, against the measured HBM copy bandwidth
  step_roofline  the whole step's algorithmic bytes (84 B/cell for E+H, +12 B/cell S,
              +32 B per CPML face-cell) per step time
  cpu_baseline   the reference's own kernels (oracle/_ref replay; else the C restatement)
              timed on the host cores on a bounded number of full-grid steps

--impl reference times the reference's CPU implementation of the same steps instead.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mcell-updates/s & %HBM peak, plain vs batched+learned-ABC at stated field err"
UNIT = "Mcell-updates/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8000)
    ap.add_argument("--warmup", type=int, default=50)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="c2")
    ap.add_argument("--e2e-steps", type=int, default=2000)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--xchunk", type=int, default=0, help="x planes per thread (0: plan default)")
    ap.add_argument("--fused-rows", type=int, default=0)
    ap.add_argument("--fused-xchunk", type=int, default=0)
    ap.add_argument("--fused-stages", type=int, default=0)
    ap.add_argument("--fused-tma", type=int, default=-1)
    ap.add_argument("--slab", type=int, default=-1, help="x planes per L2 slab (-1: plan default)")
    ap.add_argument("--hs-xchunk", type=int, default=0)
    ap.add_argument("--hs-prefetch", type=int, default=-1)
    ap.add_argument("--c4-variants", type=int, default=64, help="c4: number of cavity variants")
    ap.add_argument("--c4-steps", type=int, default=2000, help="c4: steps of every variant")
    ap.add_argument("--c4-chunk", type=int, default=100, help="c4: steps per captured launch")
    ap.add_argument("--c5-runs", type=int, default=200, help="c5: teacher runs at 128^3")
    ap.add_argument("--c5-steps", type=int, default=2000, help="c5: timed steps of the c2 cavity forms")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the parity, batched and learned-boundary sections of the default run")
    ap.add_argument("--parity-steps", type=int, default=400, help="steps of the float64 comparison run")
    ap.add_argument("--extras-variants", type=int, default=16, help="batched section: c4 variants")
    ap.add_argument("--extras-steps", type=int, default=400, help="batched section: steps per variant")
    ap.add_argument("--learned-runs", type=int, default=40, help="learned section: teacher runs")
    ap.add_argument("--learned-steps", type=int, default=1000, help="learned section: timed steps")
    ap.add_argument("--path", choices=["fused", "slab", "hs", "dropin", "default", "all"], default="default",
                    help="default = per-call loop (per-kernel timing) + Simulation.run (hs path); "
                         "slab = run over the per-update kernels; fused = the opt-in fused step")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    return rank, world, local


def peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def committed_traffic(workload: str):
    """dram bytes per launch per kernel from the committed ncu summary, if one exists."""
    p = os.path.join(ROOT, "profiles", "traffic_%s.json" % workload)
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def algorithmic_bytes(N: int, face_cells: int, elem: int, poynting: bool):
    """Per-launch compulsory bytes (each input read once, each output written once)."""
    e = N * 12 * elem + face_cells * 4 * elem           # E r/w, H r, eps r; psi_E r/w
    h = N * 9 * elem + face_cells * 4 * elem             # H r/w, E r; psi_H r/w
    s = 0
    if poynting:
        h += N * 6 * elem                                 # oS w
        s = N * 9 * elem                                  # oS r, S w
    step = N * 21 * elem + face_cells * 8 * elem + (N * 3 * elem if poynting else 0)
    # run()'s H+S kernel: H read (one copy) and written (the other), E read, S written;
    # psi_H read / written
    hs = N * 12 * elem + face_cells * 4 * elem
    return {"k_bulk_e": e, "k_bulk_h": h, "k_bulk_s": s, "k_bulk_hs": hs}, step


# FP64 DFT monitor of the c2 ringdown (the north star's "FP64 DFT monitor at 5 interior points"):
# E_y at the cavity centre and at four points two lattice constants away in x and y, transformed at
# the source's centre frequency and 5% either side of it
MONITOR_OFFSETS = ((0, 0), (20, 0), (-20, 0), (0, 20), (0, -20))
MONITOR_DESC = "FP64 DFT of E_y at 5 interior points (centre, +-20 cells in x and y), 3 frequencies, every step"


def monitor_points(wl):
    shape = wl["shape"]
    N = int(numpy.prod(shape))
    c = numpy.unravel_index(wl["source_index"] % N, shape)
    return [(1, (int(c[0]) + dx, int(c[1]) + dy, int(c[2]))) for dx, dy in MONITOR_OFFSETS]


def monitor_omegas():
    w0 = 2 * math.pi * 40.0 / 1550.0
    return [0.95 * w0, w0, 1.05 * w0]


def workload_config(wl, fc: int, elem: int, poynting: bool):
    """The workload as both arms report it (the same keys and values)."""
    N = int(numpy.prod(wl["shape"]))
    cfg = {"workload": wl["describe"], "grid": list(wl["shape"]), "cells": N, "cpml_face_cells": fc,
           "l2": "inputs (~%.0f MB of fields) larger than the 129 MB L2; no flush" % (3 * N * elem * (6 if poynting else 3) / 1e6)}
    if wl["name"] == "c2":
        cfg["monitor"] = MONITOR_DESC
    return cfg


def cpu_sample(wl, seconds: float, nthreads: int):
    """Time full-grid steps of the reference's CPU kernels (replay) or the C restatement."""
    from oracle import ref_replay
    kw = wl["kwargs"]
    eps = numpy.concatenate([e.ravel() for e in kw["epsilon"]])
    if wl["name"] == "c2" and ref_replay.available("c2"):
        sim = ref_replay.ReplaySimulation("c2", eps, nthreads=nthreads)
        kind = "reference"
    else:
        from oracle import port
        import copy
        sim = port.PortSimulation(**copy.deepcopy(kw), nthreads=nthreads)
        kind = "port"
    N = int(numpy.prod(wl["shape"]))
    ind = wl["source_index"]
    mon_idx = numpy.array([c * N + int(numpy.ravel_multi_index(p, wl["shape"])) for c, p in monitor_points(wl)]) \
        if wl["name"] == "c2" else None
    om = numpy.array(monitor_omegas())
    acc = numpy.zeros((5, 3), numpy.complex128)
    dt = float(getattr(sim, "dt", 0.0) or 0.0)

    def step(t):
        sim.update_E([])
        sim.E[ind] += numpy.float32(wl["wave"](t))
        if mon_idx is not None:
            x = numpy.asarray(sim.E).reshape(-1)[mon_idx].astype(numpy.float64)
            acc[:] += x[:, None] * numpy.exp(-1j * om[None, :] * (t + 1) * dt)
        sim.update_H([])
        if kw.get("do_poynting", True):
            sim.update_S([])

    step(0)
    t0 = time.perf_counter()
    n = 0
    while True:
        step(n + 1)
        n += 1
        el = time.perf_counter() - t0
        if el >= seconds or n >= 1000:
            break
    return {"value": N * n / el / 1e6, "unit": UNIT, "cores": nthreads, "kind": kind,
            "sample": "%d full-grid steps of %s (%d cells) after 1 warm-up step, %.1f s"
                      % (n, wl["name"], N, el)}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from opencl_fdtd_gb300 import workloads
    wl = workloads.get(args.workload)
    nthreads = os.cpu_count() or 1
    # one step = one full-grid canonical step; the number of steps run is capped so the
    # whole run stays within about a minute
    base = cpu_sample(wl, seconds=2.0, nthreads=nthreads)
    per_step = wl["shape"][0] * wl["shape"][1] * wl["shape"][2] / (base["value"] * 1e6)
    k = max(1, min(args.steps, int(60.0 / max(per_step, 1e-6))))
    res = cpu_sample(wl, seconds=k * per_step, nthreads=nthreads)
    out = {
        "impl": "reference", "metric": METRIC, "value": round(res["value"], 3), "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * numpy.prod(wl["shape"]) / (res["value"] * 1e6), 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)",
        "config": workload_config(wl, workloads.face_cells(wl["shape"], wl["kwargs"]["pmls"]), 4,
                                  wl["kwargs"].get("do_poynting", True)),
        "path": "the reference's own kernels (rendered OpenCL C) stepping the grid on the host cores"
                + ("; E at the monitor points transformed in float64 every step" if wl["name"] == "c2" else ""),
        "cpu_baseline": {"value": round(res["value"], 3), "unit": UNIT, "cores": nthreads,
                         "kind": res["kind"], "sample": res["sample"]},
        "e2e": {"value": round(res["value"], 3), "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def time_dropin(sim, lib, wave_dev, ind, K, W, poynting, world):
    """K per-call steps (update_E, source add, update_H, update_S) with CUDA events around
    every launch; returns total and per-kernel milliseconds."""
    import torch
    from opencl_fdtd_gb300 import _lib
    stream = sim.queue
    plan = sim._plan
    bufp = ctypes.byref(sim._buffers())
    st = ctypes.c_void_p(stream.cuda_stream)
    E1 = sim.E[ind:ind + 1]

    def step(t, ev=None):
        if ev is not None:
            ev[0].record(stream)
        _lib.check(lib.fdtd_update_e(plan, bufp, st))
        if ev is not None:
            ev[1].record(stream)
        E1.add_(wave_dev[t:t + 1])
        if ev is not None:
            ev[2].record(stream)
        _lib.check(lib.fdtd_update_h(plan, bufp, st))
        if ev is not None:
            ev[3].record(stream)
        if poynting:
            _lib.check(lib.fdtd_update_s(plan, bufp, st))
        if ev is not None:
            ev[4].record(stream)

    with torch.cuda.stream(stream):
        for t in range(W):
            step(t)
        torch.cuda.synchronize()
        if world > 1:
            from opencl_fdtd_gb300 import replicas
            replicas.barrier()
        evs = [[torch.cuda.Event(enable_timing=True) for _ in range(5)] for _ in range(K)]
        torch.cuda.synchronize()
        for t in range(K):
            step(W + t, evs[t])
        torch.cuda.synchronize()
        if world > 1:
            from opencl_fdtd_gb300 import replicas
            replicas.barrier()
    total = evs[0][0].elapsed_time(evs[-1][4])
    per = {"k_bulk_e": statistics.mean(evs[t][0].elapsed_time(evs[t][1]) for t in range(K)),
           "k_bulk_h": statistics.mean(evs[t][2].elapsed_time(evs[t][3]) for t in range(K))}
    if poynting:
        per["k_bulk_s"] = statistics.mean(evs[t][3].elapsed_time(evs[t][4]) for t in range(K))
    return total, per


def time_run(sim, lib, wave_dev, ind, K, W, world, mode, monitor=None):
    """K steps in one fdtd_run call bracketed by CUDA events. mode: 'hs' (E in place, H and S
    in one launch), 'fused' (one kernel per step) or None (the per-update kernels); monitor: a
    DftMonitor sampled after every timed step (inside the timed region)."""
    import torch
    from opencl_fdtd_gb300 import _lib
    stream = sim.queue
    if mode:
        sim._ensure_scratch(mode)
    bufs = sim._buffers()
    sim._attach_scratch(mode)
    st = ctypes.c_void_p(stream.cuda_stream)
    idx = (ctypes.c_int64 * 1)(ind)
    esz = wave_dev.element_size()
    warm = _lib.FdtdPointSources(1, 0, ctypes.addressof(idx), wave_dev.data_ptr())
    timed = _lib.FdtdPointSources(1, 0, ctypes.addressof(idx), wave_dev.data_ptr() + W * esz)
    with torch.cuda.stream(stream):
        _lib.check(lib.fdtd_run(sim._plan, ctypes.byref(bufs), st, W, ctypes.byref(warm), None))
        torch.cuda.synchronize()
        if world > 1:
            from opencl_fdtd_gb300 import replicas
            replicas.barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        mon = ctypes.byref(monitor.struct(K)) if monitor is not None else None
        e0.record(stream)
        _lib.check(lib.fdtd_run(sim._plan, ctypes.byref(bufs), st, K, ctypes.byref(timed), mon))
        e1.record(stream)
        if monitor is not None:
            monitor.samples += K
        torch.cuda.synchronize()
        if world > 1:
            from opencl_fdtd_gb300 import replicas
            replicas.barrier()
    return e0.elapsed_time(e1)


def run_kernel_ms(sim, lib, wave_dev, ind, steps):
    """Mean launch times of the H+S path's two kernels: one more fdtd_run with the plan's
    timing events on (CUDA events on the launching stream around update_E and the H+S kernel
    of up to 64 sampled steps)."""
    import torch
    from opencl_fdtd_gb300 import _lib
    stream = sim.queue
    sim._ensure_scratch("hs")
    bufs = sim._buffers()
    sim._attach_scratch("hs")
    idx = (ctypes.c_int64 * 1)(ind)
    src = _lib.FdtdPointSources(1, 0, ctypes.addressof(idx), wave_dev.data_ptr())
    _lib.check(lib.fdtd_plan_tune(sim._plan, _lib.FDTD_TUNE_TIMING, 1))
    with torch.cuda.stream(stream):
        _lib.check(lib.fdtd_run(sim._plan, ctypes.byref(bufs), ctypes.c_void_p(stream.cuda_stream),
                                steps, ctypes.byref(src), None))
    torch.cuda.synchronize()
    _lib.check(lib.fdtd_plan_tune(sim._plan, _lib.FDTD_TUNE_TIMING, 0))
    ms = (ctypes.c_double * 2)()
    n = ctypes.c_int32()
    _lib.check(lib.fdtd_run_kernel_ms(sim._plan, ms, ctypes.byref(n)))
    return {"k_bulk_e": ms[0], "k_bulk_hs": ms[1]}, n.value


def c2_parity(wl, steps: int):
    """Relative L2 of the float32 run (the default Simulation.run path) against the same steps in
    float64 on the GPU, for E, H and S."""
    import copy
    import torch
    from opencl_fdtd_gb300 import Simulation
    vals = [wl["wave"](t) for t in range(steps)]
    g = Simulation(**copy.deepcopy(wl["kwargs"]))
    g.run(steps, point_sources=[(wl["source_index"], vals)])
    path = {1: "per-update", 2: "H+S", 3: "one-pass"}.get(g.tuning("last_run_path"), "?")
    got = {k: g.get(k).astype(numpy.float64) for k in ("E", "H", "S")}
    del g
    kw = copy.deepcopy(wl["kwargs"])
    kw["epsilon"] = [e.astype(numpy.float64) for e in kw["epsilon"]]
    kw["float_type"] = numpy.float64
    d = Simulation(**kw)
    d.run(steps, point_sources=[(wl["source_index"], vals)])
    err = {}
    for k in ("E", "H", "S"):
        ref = d.get(k)
        err[k] = float("%.4g" % (numpy.linalg.norm(got[k] - ref) / numpy.linalg.norm(ref)))
    del d
    torch.cuda.empty_cache()
    return {"steps": steps, "path": path, "rel_l2_vs_fp64": err,
            "reference": "the same steps in float64 on the GPU (bit-identical to the float64 oracle in the "
                         "GPU tests); float32 bit-identical to the oracle (tests/test_gpu_config2.py)"}


def run_extras(args, wl):
    """Bounded versions of the other halves of the metric, for the default run: the float64
    error of the benchmarked workload, the batched sweep (a subset of c4's variants and steps)
    and the learned thin boundary (fewer teacher runs than c5 states)."""
    import torch
    out = {}
    t0 = time.perf_counter()
    out["parity"] = c2_parity(wl, args.parity_steps) if wl["name"] == "c2" else None
    t1 = time.perf_counter()
    b = c4_measure(args.extras_variants, args.extras_steps, 100 if args.extras_steps % 100 == 0 else args.extras_steps,
                   storages=("f32", "bf16u"))
    torch.cuda.empty_cache()
    cfg = b["config"]
    out["batched"] = {
        "workload": "c4 subset: the first %d of c4's seeded L3 variants, %d steps each, f32 arithmetic"
                    % (cfg["variants"], cfg["steps"]),
        "cells": cfg["cells"], "interior_cells": cfg["interior_cells"],
        "plain": {"value": b["plain"]["value"], "interior_value": b["plain"]["interior_value"],
                  "ms": b["plain"]["ms"], "error_vs_f64": b["plain"]["error_vs_f64"],
                  "path": "per-variant Simulation.run (per-update kernels)"},
        "f32": {k: b["batched"]["f32"][k] for k in ("value", "interior_value", "ms", "error_vs_f64",
                                                    "rel_l2_E_vs_plain_f32", "bit_identical_to_plain")},
        "bf16u": {k: b["batched"]["bf16u"][k] for k in ("value", "interior_value", "ms", "error_vs_f64",
                                                        "rel_l2_E_vs_plain_f32")},
        "schedule": b["batched"]["f32"]["tiles"]["schedule"],
        "speedup_f32_vs_plain": round(b["plain"]["ms"] / b["batched"]["f32"]["ms"], 3),
        "speedup_bf16u_vs_plain": round(b["plain"]["ms"] / b["batched"]["bf16u"]["ms"], 3),
        "unit": UNIT}
    for k in ("f32", "bf16u"):
        e = out["batched"][k]["error_vs_f64"]
        out["batched"][k]["error_vs_f64"] = {"rel_l2_E": e["rel_l2_E"], "dft_peak_rel": e["dft_peak_rel"]}
    t2 = time.perf_counter()
    c = c5_measure(args.learned_runs, args.learned_steps)
    torch.cuda.empty_cache()
    pick = c["verdicts"][c["candidate_timed"]]
    out["learned"] = {
        "workload": "c5 at %d teacher runs (c5 states 200): the c2 cavity with a 2-cell learned layer on "
                    "every face or on the z faces, against its 8-cell CPML, %d steps" % (args.learned_runs,
                                                                                     args.learned_steps),
        "deployed": c["deployed"], "candidate": c["candidate_timed"],
        "useful_interior_value": c["value"], "unit": UNIT,
        "plain_cpml8_useful_value": c["plain_cpml8"]["useful_mcells_per_s"],
        "thin_all_faces": {"useful_value": c["thin_learned"]["useful_mcells_per_s"],
                           "interior_rel_l2_vs_plain_cpml8": c["thin_learned"]["interior_rel_l2_vs_plain_cpml8"],
                           "reflection_db": pick.get("reflection_db"), "accepted": pick.get("accepted")},
        "thin_z_faces": {"useful_value": c["thin_z_learned"]["useful_mcells_per_s"],
                         "interior_rel_l2_vs_plain_cpml8": c["thin_z_learned"]["interior_rel_l2_vs_plain_cpml8"],
                         "reflection_db": c["thin_z_learned"]["verdict"].get("reflection_db"),
                         "accepted": c["thin_z_learned"]["verdict"].get("accepted")},
        "target": "reflection <= -40 dB and interior relative L2 <= 1e-3 against the plain 8-cell CPML run; "
                  "CPML is deployed otherwise",
        "predict_roofline": c["roofline"]}
    t3 = time.perf_counter()
    out["extras_seconds"] = {"parity": round(t1 - t0, 1), "batched": round(t2 - t1, 1), "learned": round(t3 - t2, 1)}
    return out


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from opencl_fdtd_gb300 import Simulation, workloads

    wl = workloads.get(args.workload)
    kw = wl["kwargs"]
    sim = Simulation(**kw)
    if args.xchunk:
        sim.tune(xchunk=args.xchunk)
    if args.fused_rows:
        sim.tune(fused_rows=args.fused_rows)
    if args.fused_xchunk:
        sim.tune(fused_xchunk=args.fused_xchunk)
    if args.fused_stages:
        sim.tune(fused_stages=args.fused_stages)
    if args.fused_tma >= 0:
        sim.tune(fused_tma=bool(args.fused_tma))
    if args.slab >= 0:
        sim.tune(slab=args.slab)
    if args.hs_xchunk:
        sim.tune(hs_xchunk=args.hs_xchunk)
    if args.hs_prefetch >= 0:
        sim.tune(hs_prefetch=bool(args.hs_prefetch))
    N = int(numpy.prod(wl["shape"]))
    fc = workloads.face_cells(wl["shape"], kw["pmls"])
    poynting = kw.get("do_poynting", True)
    elem = 4 if kw.get("float_type", numpy.float32) == numpy.float32 else 8
    K, W = args.steps, args.warmup
    ind = wl["source_index"]
    waves = numpy.array([wl["wave"](t) for t in range(W + K)], dtype=numpy.float32)
    wave_dev = torch.from_numpy(waves).cuda()
    lib = sim._lib

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    res = {}
    if args.path in ("dropin", "default", "all"):
        res["dropin"] = time_dropin(sim, lib, wave_dev, ind, K, W, poynting, world)
    mon = sim.dft_monitor(monitor_points(wl), monitor_omegas(), record=False) if wl["name"] == "c2" else None
    if args.path in ("hs", "default", "all") and poynting:
        res["hs"] = time_run(sim, lib, wave_dev, ind, K, W, world, "hs", monitor=mon)
        hs_per = run_kernel_ms(sim, lib, wave_dev, ind, min(W + K, 640))
    if args.path in ("slab", "all"):
        res["slab"] = time_run(sim, lib, wave_dev, ind, K, W, world, None)
        sim.tune(slab=0)
    if args.path in ("fused", "all"):
        res["fused"] = time_run(sim, lib, wave_dev, ind, K, W, world, "fused",
                                monitor=mon if args.path == "fused" else None)
    clock = clocks.stop()

    from opencl_fdtd_gb300 import replicas

    def allmax(v):
        return replicas.max_over_ranks(v, device="cuda")

    peak, peak_kind = peak_hbm()
    per_launch, step_bytes = algorithmic_bytes(N, fc, elem, poynting)
    traffic = committed_traffic(args.workload)
    out_paths = {}
    if "dropin" in res:
        total, per = res["dropin"]
        total = allmax(total)
        dom = max(per, key=lambda k: per[k])
        ach = per_launch[dom] / (per[dom] * 1e-3) / 1e9
        out_paths["dropin"] = {
            "ms_per_step": total / K, "value": world * N * K / (total * 1e-3) / 1e6,
            "gpu_launches": (3 if poynting else 2) * K,
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(ach, 1), "peak": peak,
                         "unit": "GB/s", "frac": round(ach / peak, 4), "peak_source": peak_kind,
                         "traffic": traffic.get(dom), "algorithmic_bytes_per_launch": per_launch[dom],
                         "mean_launch_ms": round(per[dom], 5),
                         "per_kernel_ms": {k: round(v, 5) for k, v in per.items()}}}
    compulsory = N * (18 if poynting else 15) * elem + fc * 8 * elem
    for name in ("fused", "slab", "hs"):
        if name not in res:
            continue
        total = allmax(res[name])
        ms = total / K
        ach = step_bytes / (ms * 1e-3) / 1e9
        nslab = (wl["shape"][0] + sim.slab_planes() - 1) // sim.slab_planes()
        # per step: the path's kernels (the workload's one point source is added inside k_step
        # on the fused path and inside the E kernel on the hs path) and the DFT monitor sample
        # when the monitor is timed (on the hs path by one block of the H+S launch unless the
        # plan's hs_dft is off)
        launches = {"fused": K, "hs": 2 * K,
                    "slab": K * ((3 if poynting else 2) * nslab + (3 if poynting else 1) + 1)}[name]
        if mon is not None and ((name == "hs" and not sim.tuning("hs_dft"))
                                or (name == "fused" and args.path == "fused")):
            launches += K
        kname = {"fused": "k_step", "hs": "step (k_bulk_e + k_bulk_hs)",
                 "slab": "step (k_bulk_e/h/s over L2 slabs)"}[name]
        out_paths[name] = {
            "ms_per_step": ms, "value": world * N * K / (total * 1e-3) / 1e6, "gpu_launches": launches,
            "roofline": {"bound": "hbm", "kernel": kname,
                         "achieved": round(ach, 1),
                         "peak": peak, "unit": "GB/s", "frac": round(ach / peak, 4),
                         "peak_source": peak_kind, "traffic": traffic.get(name),
                         "algorithmic_bytes_per_launch" if name == "fused" else "algorithmic_bytes_per_step": step_bytes,
                         "accounting": "84 B/cell E+H, +12 B/cell S, +32 B per CPML face-cell (f32)",
                         "compulsory_bytes_per_step": compulsory,
                         "compulsory_frac": round(compulsory / (ms * 1e-3) / 1e9 / peak, 4),
                         "mean_step_ms": round(ms, 5)}}
    if "hs" in out_paths:
        per, nsamp = hs_per
        dom = max(per, key=lambda k: per[k])
        ach = per_launch[dom] / (per[dom] * 1e-3) / 1e9
        out_paths["hs"]["kernel_roofline"] = {
            "bound": "hbm", "kernel": dom, "achieved": round(ach, 1), "peak": peak, "unit": "GB/s",
            "frac": round(ach / peak, 4), "peak_source": peak_kind, "traffic": traffic.get(dom),
            "algorithmic_bytes_per_launch": per_launch[dom], "mean_launch_ms": round(per[dom], 5),
            "per_kernel_ms": {k: round(v, 5) for k, v in per.items()}, "sampled_launches": nsamp,
            "per_kernel_frac": {k: round(per_launch[k] / (v * 1e-3) / 1e9 / peak, 4)
                                for k, v in per.items()}}
    cands = [n for n in ("fused", "slab", "hs") if n in out_paths]
    head = min(cands, key=lambda n: out_paths[n]["ms_per_step"]) if cands else "dropin"
    hp = out_paths[head]
    step_gbs = step_bytes / (hp["ms_per_step"] * 1e-3) / 1e9
    # launch options of the H+S path as the timed run used them
    launch = ({"hs_xchunk": sim.tuning("hs_xchunk_used"), "pdl": sim.tuning("pdl"),
               "dft_in_hs_launch": sim.tuning("hs_dft"), "e_xchunk": sim.tuning("xchunk"),
               "e_form": sim.tuning("e_form")}
              if head == "hs" else None)

    e2e = None
    if not args.no_e2e:
        # the same FP64 DFT monitor as the timed run (a separate accumulator)
        e2e_mon = (sim.dft_monitor(monitor_points(wl), monitor_omegas(), record=False)
                   if wl["name"] == "c2" else None)
        e2e = run_e2e(sim, wl, args.e2e_steps, world, run_api=(head != "dropin"),
                      path={"fused": "fused", "hs": "hs", "slab": "plain"}.get(head, "auto"), monitor=e2e_mon)

    mon_out = None
    if mon is not None and mon.samples:
        acc = mon.accum.cpu().numpy()
        mag = numpy.hypot(acc[..., 0], acc[..., 1])
        mon_out = {"points": len(MONITOR_OFFSETS), "frequencies": len(monitor_omegas()), "samples": mon.samples,
                   "in_timed_region": True, "centre_abs_dft": [float("%.6g" % v) for v in mag[0]]}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_sample(wl, args.cpu_seconds, os.cpu_count() or 1)

    extras = {}
    if rank == 0 and world == 1 and not args.no_extras:
        del sim
        torch.cuda.empty_cache()
        extras = run_extras(args, wl)

    if rank == 0:
        out = {
            "metric": METRIC, "value": round(hp["value"], 2), "unit": UNIT, "n_gpus": world,
            "steps": K, "warmup": W, "ms_per_step": round(hp["ms_per_step"], 5),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded L3 cavity geometry and source)",
            "config": workload_config(wl, fc, elem, poynting),
            "path": {"fused": "Simulation.run(path='fused'): one fused E+source+H+S kernel per step",
                                "hs": "Simulation.run: E in place, point source, H+S in one launch (H ping-pong)",
                                "slab": "Simulation.run(path='plain'): E, point source, H, S update kernels",
                                "dropin": "per-call update_E / source add / update_H / update_S"}[head],
            "parallelism": "replicas" if world > 1 else "single GPU",
            "launch": launch,
            "monitor": mon_out,
            # the dominant kernel's roofline: per-call timing of the same kernels the run
            # path launches (the fused path reports its own kernel)
            # the dominant kernel of the headline path, timed per launch with CUDA events
            "roofline": (hp["kernel_roofline"] if "kernel_roofline" in hp else
                         out_paths["dropin"]["roofline"] if head != "fused" and "dropin" in out_paths
                         else hp["roofline"]),
            "step_roofline": {"achieved": round(step_gbs, 1), "peak": peak, "unit": "GB/s",
                              "frac": round(step_gbs / peak, 4), "bytes_per_step": step_bytes},
            "clocks": clock, "e2e": e2e, "gpu_launches": hp["gpu_launches"],
            "cpu_baseline": cpu,
            "dropin_roofline": out_paths["dropin"]["roofline"] if "dropin" in out_paths else None,
            # roofline_frac: the path's own kernel (dropin: its dominant kernel per launch);
            # step_roofline_frac: the whole step against the step's algorithmic bytes, the same
            # basis for every path (the per-call loop moves more than those bytes: it writes
            # and re-reads the six Poynting products)
            "paths": {k: {"value": round(v["value"], 2), "ms_per_step": round(v["ms_per_step"], 5),
                          "roofline_frac": v["roofline"]["frac"], "kernel": v["roofline"]["kernel"],
                          "step_roofline_frac": round(step_bytes / (v["ms_per_step"] * 1e-3) / 1e9 / peak, 4)}
                      for k, v in out_paths.items()},
        }
        out.update(extras)
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_e2e(sim, wl, steps: int, world: int, run_api: bool = False, path: str = "auto", monitor=None):
    """End to end through the public API with host buffers.

    API: Simulation.run() in calls of 10 steps, each given its 10 source samples from host
    memory (copied to the device inside the call, from pinned staging, without blocking the
    host) and followed by a device-to-host copy of the driven field sample into pinned host
    memory on the simulation's stream; the host synchronizes once at the end and the samples
    are checked; `monitor` (the workload's DFT monitor) is sampled every step as in the
    device-timed run. Otherwise the per-call loop of fdtd.py:162-175 with the source sample copied
    from pinned host memory each step and the field sample read back the same way."""
    import torch
    if run_api:
        ind = wl["source_index"]
        chunk = 10
        host = numpy.array([wl["wave"](t) for t in range(steps + 2 * chunk)], dtype=numpy.float64)
        probe = torch.empty(steps // chunk + 2, dtype=torch.float32, pin_memory=True)
        sim.run(chunk, point_sources=[(ind, host[:chunk])], path=path, monitor=monitor).wait()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        n = 0
        for c in range(steps // chunk):
            sim.run(chunk, point_sources=[(ind, host[c * chunk:(c + 1) * chunk])], path=path, monitor=monitor)
            with torch.cuda.stream(sim.queue):
                probe[c:c + 1].copy_(sim.E[ind:ind + 1], non_blocking=True)
            n += chunk
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        if not bool(torch.isfinite(probe[:steps // chunk]).all()):
            raise SystemExit("e2e: non-finite field sample")
        N = int(numpy.prod(wl["shape"]))
        return {"value": round(world * N * n / el / 1e6, 2), "unit": UNIT,
                "h2d_bytes_per_step": 4, "d2h_bytes_per_step": round(4 / chunk, 2), "steps": n,
                "api": "Simulation.run(10 steps, point_sources from host, DFT monitor) + field sample read back",
                "monitor": monitor is not None}
    ind = wl["source_index"]
    poynting = wl["kwargs"].get("do_poynting", True)
    host_src = torch.from_numpy(numpy.array([wl["wave"](t) for t in range(steps)],
                                            dtype=numpy.float32)).pin_memory()
    host_probe = torch.empty(steps, dtype=torch.float32).pin_memory()
    dev_src = torch.empty(1, dtype=torch.float32, device=sim.device)
    E1 = sim.E[ind:ind + 1]
    stream = sim.queue

    def one(t):
        sim.update_E([])
        dev_src.copy_(host_src[t:t + 1], non_blocking=True)
        E1.add_(dev_src)
        e = sim.update_H([])
        if poynting:
            sim.update_S([e])
        host_probe[t:t + 1].copy_(E1, non_blocking=True)

    with torch.cuda.stream(stream):
        for t in range(min(20, steps)):
            one(t)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for t in range(steps):
            one(t)
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
    N = int(numpy.prod(wl["shape"]))
    return {"value": round(world * N * steps / el / 1e6, 2), "unit": UNIT,
            "h2d_bytes_per_step": 4, "d2h_bytes_per_step": 4, "steps": steps,
            "api": "Simulation.update_E/H/S + tensor source add, stream-ordered"}


def _peak_frequency(series, dt, w0):
    """Angular frequency of the largest spectral peak within [0.5 w0, 1.5 w0] of a sampled
    series (zero-padded FFT, parabolic interpolation of the log magnitude)."""
    x = numpy.asarray(series, dtype=numpy.float64)
    n = 1 << 18
    spec = numpy.abs(numpy.fft.rfft(x, n))
    w = 2 * numpy.pi * numpy.fft.rfftfreq(n, dt)
    band = numpy.flatnonzero((w > 0.5 * w0) & (w < 1.5 * w0))
    k = band[numpy.argmax(spec[band])]
    if 0 < k < len(spec) - 1 and spec[k - 1] > 0 and spec[k + 1] > 0:
        a, b, c = numpy.log(spec[k - 1]), numpy.log(spec[k]), numpy.log(spec[k + 1])
        den = a - 2 * b + c
        off = 0.5 * (a - c) / den if den != 0 else 0.0
        return float(w[k] + off * (w[1] - w[0]))
    return float(w[k])


def c4_measure(n_variants: int, steps: int, chunk: int, storages=("f32", "bf16", "fp16", "bf16u")):
    """Batched sweep: per-variant Simulation.run against one persistent launch per chunk of
    steps (CUDA graph replays, autotuned tiles) in float32 and 16-bit storage; every storage's
    errors against a float64 run of every variant (relative L2 of E, DFT-peak frequency of the
    centre E_y series). Returns the plain and batched timings, the errors and the setup."""
    import torch
    from opencl_fdtd_gb300 import Simulation, workloads
    from opencl_fdtd_gb300.batch import BatchSimulation
    if steps % chunk:
        raise SystemExit("the c4 step count must be a multiple of the chunk")
    t_setup = time.perf_counter()
    variants = workloads.c4(n=n_variants, steps=steps)
    kws, idx = [], []
    for var in variants:
        kw, ind = workloads.c4_kwargs(var)
        kws.append(kw)
        idx.append(ind)
    sims = [Simulation(**kw) for kw in kws]
    wave = numpy.array([variants[0]["wave"](t) for t in range(steps)], dtype=numpy.float64)
    cells = sum(s.N for s in sims)
    interior = sum(max(s.shape[0] - 16, 0) * max(s.shape[1] - 16, 0) * max(s.shape[2] - 16, 0) for s in sims)
    sources = [[(ind, wave)] for ind in idx]
    monitors = [[ind] for ind in idx]
    setup_s = time.perf_counter() - t_setup
    stream = sims[0].queue

    def reset():
        for s in sims:
            s.E.zero_()
            s.H.zero_()
            for f in ("E", "H"):
                for u, v in s.psi[f]:
                    u.zero_()
                    v.zero_()
            s.steps_run = 0
        torch.cuda.synchronize()

    def timed(fn):
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            fn()
            e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    out = {"plain": {}, "batched": {}}
    # per-variant Simulation.run, one after the other on one stream
    mons = [s.dft_monitor([(1, tuple(c // 2 for c in s.shape))], ()) for s in sims]

    def plain():
        for s, src, m in zip(sims, sources, mons):
            s.run(steps, point_sources=src, monitor=m, path="plain")
    ms = timed(plain)
    out["plain"] = {"ms": round(ms, 3), "value": round(cells * steps / (ms * 1e-3) / 1e6, 2),
                    "interior_value": round(interior * steps / (ms * 1e-3) / 1e6, 2),
                    "launches": len(sims) * steps * 3}
    plain_E = [s.E.clone() for s in sims]
    plain_series = [m.series()[:, 0] for m in mons]
    results = {}
    for storage in storages:
        reset()
        b = BatchSimulation(sims, storage=storage, sources=sources, monitors=monitors, steps=steps)
        tune = b.autotune(steps=10)
        b.capture(chunk)
        ms = timed(lambda: [b.replay() for _ in range(steps // chunk)])
        b.sync()
        torch.cuda.synchronize()
        results[storage] = {"E": [s.E.clone() for s in sims], "series": [x.cpu().numpy()[:, 0] for x in b.series]}
        out["batched"][storage] = {
            "ms": round(ms, 3), "value": round(cells * steps / (ms * 1e-3) / 1e6, 2),
            "interior_value": round(interior * steps / (ms * 1e-3) / 1e6, 2),
            "tiles": {"schedule": tune["schedule"], "xchunk": tune["xchunk"],
                      "blocks_per_sm": tune["blocks_per_sm"], "autotune_ms_per_step": tune.get("timings")},
            "launches": steps // chunk if tune["schedule"] == "persistent" else 2 * steps,
            "steps_per_graph": chunk, "graph_replays": steps // chunk}
        b.close()
        del b
    out["batched"]["f32"]["bit_identical_to_plain"] = all(
        torch.equal(a, c) for a, c in zip(plain_E, results["f32"]["E"])) and all(
        numpy.array_equal(a, c) for a, c in zip(plain_series, results["f32"]["series"]))
    # float64 reference of every variant: errors of the float32 and 16-bit runs
    w0 = 2 * math.pi * 40.0 / 1550.0
    err = {k: {"rel_l2": [], "peak_rel": []} for k in storages}
    for v, var in enumerate(variants):
        kw64, ind = workloads.c4_kwargs(var, float_type=numpy.float64)
        s64 = Simulation(**kw64)
        m64 = s64.dft_monitor([(1, tuple(c // 2 for c in s64.shape))], ())
        s64.run(steps, point_sources=[(ind, wave)], monitor=m64, path="plain")
        ref = s64.E
        fin = torch.isfinite(ref)
        nref = torch.linalg.norm(ref[fin])
        w_ref = _peak_frequency(m64.series()[:, 0], s64.dt, w0)
        for k in err:
            e = results[k]["E"][v].double()
            err[k]["rel_l2"].append(float(torch.linalg.norm((e - ref)[fin]) / nref))
            err[k]["peak_rel"].append(abs(_peak_frequency(results[k]["series"][v], s64.dt, w0) - w_ref) / w_ref)
        del s64, m64, ref
    # plain (per-variant) float32 against float64: the error every batched storage adds to
    plain_err = []
    for v, var in enumerate(variants):
        kw64, ind = workloads.c4_kwargs(var, float_type=numpy.float64)
        s64 = Simulation(**kw64)
        s64.run(steps, point_sources=[(ind, wave)], path="plain")
        ref = s64.E
        fin = torch.isfinite(ref)
        plain_err.append(float(torch.linalg.norm((plain_E[v].double() - ref)[fin]) / torch.linalg.norm(ref[fin])))
        del s64, ref
    out["plain"]["error_vs_f64"] = {"rel_l2_E": {"median": float(numpy.median(plain_err)),
                                                  "max": float(numpy.max(plain_err))}}
    for k in err:
        a = numpy.array(err[k]["rel_l2"])
        p = numpy.array(err[k]["peak_rel"])
        out["batched"][k]["error_vs_f64"] = {
            "rel_l2_E": {"median": float(numpy.median(a)), "max": float(a.max())},
            "dft_peak_rel": {"median": float(numpy.median(p)), "max": float(p.max())},
            "per_variant_rel_l2_E": [float("%.3g" % x) for x in a],
            "per_variant_dft_peak_rel": [float("%.3g" % x) for x in p]}
        # against the plain per-variant float32 run
        d = [float(torch.linalg.norm((results[k]["E"][v] - plain_E[v]).double()) /
                   torch.linalg.norm(plain_E[v].double())) for v in range(len(variants))]
        out["batched"][k]["rel_l2_E_vs_plain_f32"] = {"median": float(numpy.median(d)), "max": float(max(d))}
    out["config"] = {"variants": len(variants), "steps": steps, "cells": cells, "interior_cells": interior,
                     "setup_s": round(setup_s, 1), "steps_per_graph": chunk}
    return out


def run_c4(args):
    """The batched sweep of c4 at its stated size, as one JSON line."""
    import torch
    torch.cuda.set_device(0)
    steps, chunk = args.c4_steps, args.c4_chunk
    out = c4_measure(args.c4_variants, steps, chunk)
    cells, interior = out["config"]["cells"], out["config"]["interior_cells"]
    best = out["batched"]["f32"]
    line = {
        "metric": METRIC, "value": best["value"], "unit": UNIT, "n_gpus": 1, "steps": steps, "warmup": 10,
        "ms_per_step": round(best["ms"] / steps, 5), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 arithmetic; f32 / bf16 / fp16 / bf16 (no tile exponents) storage", "data": "synthetic (seeded L3 variants)",
        "config": {"workload": "c4: %d seeded L3-cavity variants, grids U{96..256}xU{96..224}xU{48..73}, "
                               "a ~ U[8,12], r ~ U[0.25a,0.35a], 8-cell CPML x6, Poynting off, %d steps"
                               % (out["config"]["variants"], steps),
                   "cells": cells, "interior_cells": interior, "setup_s": out["config"]["setup_s"],
                   "l2": "inputs (%.1f GB of fields) larger than the 129 MB L2; no flush" % (cells * 36 / 1e9)},
        "plain": out["plain"], "batched": out["batched"],
        "speedup_batched_f32_vs_plain": round(out["plain"]["ms"] / best["ms"], 3),
    }
    print(json.dumps(line), flush=True)


def run_c3(args):
    """Anisotropic + Bloch cell (128x128x256, split complex float32, Bloch phases on x and y,
    8-cell CPML on z, diagonal eps / mu spheres with one PEC sphere): Simulation.run over the
    per-update kernels (E, F, H, G per step), timed with CUDA events; fields start from seeded
    random values (the plane-wave source does not change the work). Algorithmic bytes per
    cell-step: the real and imaginary passes each read and write their field once and read the
    coupled partners and eps / mu; the count is spelled out below."""
    import torch
    from opencl_fdtd_gb300 import Simulation, workloads
    torch.cuda.set_device(0)
    wl = workloads.get("c3")
    kw = dict(wl["kwargs"])
    shape = wl["shape"]
    N = int(numpy.prod(shape))
    rng = numpy.random.default_rng(33)
    kw["initial_fields"] = {k: [(1e-3 * rng.standard_normal(shape)).astype(numpy.float32) for _ in range(3)]
                            for k in ("E", "H", "F", "G")}
    sim = Simulation(**kw)
    K = args.steps if args.steps != 8000 else 2000
    W = max(args.warmup if args.warmup != 50 else 20, 3)
    sim.run(W)
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    time.sleep(0.3)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(sim.queue)
    sim.run(K)
    e1.record(sim.queue)
    e1.synchronize()
    clock = clocks.stop()
    ms = e0.elapsed_time(e1)
    finite = bool(torch.isfinite(sim.E).all())
    # bytes per cell-step, one access per array per pass (float32): the E pass reads and writes
    # E and reads H and eps, the F pass likewise F, G and eps, the H and G passes their field,
    # the E-type field and mu (the Bloch partner is read only on the wrapped planes): 4 passes x
    # 4 arrays x 3 components x 4 B = 192 B per cell; CPML psi on the z faces: 4 passes x
    # 2 arrays read and written x 4 B = 64 B per face-cell
    fc = workloads.face_cells(shape, kw["pmls"])
    step_bytes = 192.0 * N + 64.0 * fc
    peak, peak_kind = peak_hbm()
    gbs = step_bytes * K / (ms * 1e-3) / 1e9
    line = {
        "metric": METRIC, "value": round(N * K / (ms * 1e-3) / 1e6, 2), "unit": UNIT, "n_gpus": 1,
        "steps": K, "warmup": W, "ms_per_step": round(ms / K, 5), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (split complex)", "data": "synthetic (seeded spheres, random fields)",
        "config": {"workload": "c3: " + wl["describe"], "cells": N, "cpml_face_cells": fc,
                   "path": "Simulation.run, per-update kernels (E, F, H, G)",
                   "l2": "fields (%.0f MB) larger than the 129 MB L2; no flush" % (N * 4 * 3 * 6 / 1e6)},
        "step_roofline": {"bound": "hbm", "achieved": round(gbs, 1), "peak": peak, "unit": "GB/s",
                          "frac": round(gbs / peak, 4), "bytes_per_step": step_bytes, "peak_kind": peak_kind},
        "finite_after_steps": finite, "clocks": clock,
    }
    print(json.dumps(line), flush=True)


def c5_measure(runs: int, K: int):
    """Learned thin boundary on the c2 cavity: teacher data (Mur-memory targets), candidate
    networks (least squares on Mur's stencil, least squares shrunk towards Mur's map at two
    strengths, and Mur's map itself),
    the evaluation of each (reflection against a doubled grid, long-run stability), then the c2
    cavity timed (a) plain with its 8-cell CPML (395x345x73) and (b) cut to its useful
    interior plus a 2-cell learned layer per face (383x333x61) with the picked candidate; the
    line reports the form the evaluation deploys. Throughput counts useful-interior cells
    (379x329x57 in both forms)."""
    import torch
    from opencl_fdtd_gb300 import Simulation, workloads
    from opencl_fdtd_gb300 import learned_boundary as L
    torch.cuda.set_device(0)
    t0 = time.perf_counter()
    data = L.make_teacher_data(runs=runs, seed=5, memory=L.MUR_MEMORY)
    torch.cuda.synchronize()
    data_s = time.perf_counter() - t0
    probe = L.BoundaryNet(seed=6, memory=L.MUR_MEMORY)
    tvar = {f: float(((data.T[f] ** 2) * probe.output_weights(f)).mean()) for f in range(6)}
    samples = data.sizes()
    # candidates: least squares shrunk towards Mur's map (two strengths), and Mur's map itself;
    # the evaluation (bf16x2 inference, the deployed precision) picks the best accepted one
    cands = {}
    t0 = time.perf_counter()
    for name, rho, support in (("learned, Mur stencil", 0.0, "mur"), ("learned, shrink 0.3", 0.3, None),
                               ("learned, shrink 1", 1.0, None), ("Mur first order", None, None)):
        net_c = L.BoundaryNet(seed=6, memory=L.MUR_MEMORY)
        if rho is None:
            for f in range(6):
                net_c.embed_linear(f, L.mur_map(f))
        else:
            net_c.fit_linear(data, ridge=rho, prior="mur", support=support)
        rel_c = [round(net_c.loss(f, data.X[f], data.T[f]) / tvar[f], 5) for f in range(6)]
        cands[name] = (net_c, rel_c)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    del data
    torch.cuda.empty_cache()
    t0 = time.perf_counter()
    verdicts = {name: L.evaluate(L.LearnedBoundary(n_, "bf16x2")) for name, (n_, _) in cands.items()}
    evaluate_s = time.perf_counter() - t0
    # the deployed candidate: the best accepted one; for the timing of the thin form when none
    # is accepted, the best stable learned one
    accepted = [k for k, v in verdicts.items() if v["accepted"]]
    stable = [k for k, v in verdicts.items() if v["stable"] and k.startswith("learned")]
    pool = accepted or stable or ["learned, shrink 0.3"]
    pick = min(pool, key=lambda k: verdicts[k]["reflection_db"])
    net = cands[pick][0]
    verdict = verdicts[pick]
    lin_ok = all(a is not None for a in net.linear)
    lb = L.LearnedBoundary(net, "linear" if lin_ok else "bf16x2")
    zero = L.BoundaryNet(seed=3, memory=L.MUR_MEMORY)
    zero.params.zero_()
    held = L.reflection_db(L.LearnedBoundary(zero, "bf16x2"), shape=(96, 96, 96), steps=400, period=20.0)
    first_pass = L.reflection_db(lb, shape=(96, 96, 96), steps=250, period=20.0)
    held_first = L.reflection_db(L.LearnedBoundary(zero, "bf16x2"), shape=(96, 96, 96), steps=250, period=20.0)
    rel = {name: r for name, (_, r) in cands.items()}

    # the c2 cavity: plain with its CPML, and cut to the useful interior plus the 2-cell layer
    wl = workloads.c2()
    kw = dict(wl["kwargs"])
    shape = wl["shape"]
    thin_off = 8 - 2
    thin_shape = tuple(s_ - 2 * thin_off for s_ in shape)
    useful = tuple(s_ - 16 for s_ in shape)
    useful_cells = int(numpy.prod(useful))
    wave = [wl["wave"](t) for t in range(K)]

    def timed(sim, ind):
        sim.run(3, point_sources=[(ind, wave[:3])])
        for t_ in (sim.E, sim.H):
            t_.zero_()
        if sim.do_poynting:
            sim.S.zero_()
        for f_ in ("E", "H"):
            for u, v in sim.psi[f_]:
                u.zero_()
                v.zero_()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(sim.queue)
        sim.run(K, point_sources=[(ind, wave)])
        e1.record(sim.queue)
        e1.synchronize()
        return e0.elapsed_time(e1)

    plain = Simulation(**kw)
    ms_plain = timed(plain, wl["source_index"])
    Ep = plain.E.view(3, *shape)[:, 8:8 + useful[0], 8:8 + useful[1], 8:8 + useful[2]].clone()
    plain.close()
    del plain
    sl = tuple(slice(thin_off, thin_off + n) for n in thin_shape)
    kw_thin = dict(kw)
    kw_thin["epsilon"] = [numpy.ascontiguousarray(e[sl]) for e in kw["epsilon"]]
    kw_thin["pmls"] = []
    kw_thin["dt"] = L.DEFAULT_DT
    thin = Simulation(**kw_thin)
    lb.attach(thin)
    c = numpy.unravel_index(wl["source_index"] % int(numpy.prod(shape)), shape)
    comp = wl["source_index"] // int(numpy.prod(shape))
    ind_thin = comp * thin.N + int(numpy.ravel_multi_index(tuple(ci - thin_off for ci in c), thin_shape))
    ms_thin = timed(thin, ind_thin)
    Et = thin.E.view(3, *thin_shape)[:, 2:2 + useful[0], 2:2 + useful[1], 2:2 + useful[2]]
    finite = bool(torch.isfinite(Et).all())
    l2 = float(torch.linalg.norm((Et - Ep).double()) / torch.linalg.norm(Ep.double())) if finite else float("inf")
    # the network's share of a thin step: one predict launch per step, timed alone
    n_cols, _ = L.columns(thin_shape)
    W = net.weights("bf16x2")
    pred = torch.empty(n_cols * 6, dtype=torch.float32, device="cuda")
    lib = L._lib.load()

    def predict():
        L._lib.check(lib.fdtd_lbc_predict(L._shape_arg(thin_shape), 63, -1, L.PRECISIONS["bf16x2"], net.memory,
                                          W.data_ptr(),
                                          thin.E.data_ptr(), thin.H.data_ptr(), pred.data_ptr(), pred.numel(),
                                          ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
    thin.E.zero_()
    thin.H.zero_()
    for _ in range(3):
        predict()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(50):
        predict()
    e1.record()
    e1.synchronize()
    ms_pred = e0.elapsed_time(e1) / 50
    flops = 2.0 * (108 * 64 + 64 * 64 + 64 * 6) * n_cols
    peaks = {}
    try:
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")) as fh:
            peaks = json.load(fh)
    except (OSError, ValueError):
        pass
    tc_peak = float(peaks.get("bf16_tflops", 1900.0))
    lb.detach(thin)
    thin.close()
    del thin

    # the learned layer on the z faces only (air above and below the slab), CPML on x and y
    # where the slab crosses, with the linear-layer kernel when the picked network is linear
    zprec = "linear" if lin_ok else "bf16x2"
    lbz = L.LearnedBoundary(net, zprec, faces=["-z", "+z"])
    verdict_z = L.evaluate(lbz, cpml_other=8)
    zshape = (shape[0], shape[1], shape[2] - 2 * thin_off)
    kw_z = dict(kw)
    kw_z["epsilon"] = [numpy.ascontiguousarray(e[:, :, thin_off:thin_off + zshape[2]]) for e in kw["epsilon"]]
    kw_z["pmls"] = [p_ for p_ in kw["pmls"] if p_["axis"] != "z"]
    kw_z["dt"] = L.DEFAULT_DT
    thz = Simulation(**kw_z)
    lbz.attach(thz)
    ind_z = comp * thz.N + int(numpy.ravel_multi_index((c[0], c[1], c[2] - thin_off), zshape))
    ms_z = timed(thz, ind_z)
    Ez = thz.E.view(3, *zshape)[:, 8:8 + useful[0], 8:8 + useful[1], 2:2 + useful[2]]
    fin_z = bool(torch.isfinite(Ez).all())
    l2_z = float(torch.linalg.norm((Ez - Ep).double()) / torch.linalg.norm(Ep.double())) if fin_z else float("inf")
    lbz.detach(thz)
    thz.close()
    del thz
    v_z = useful_cells * K / (ms_z * 1e-3) / 1e6

    v_plain = useful_cells * K / (ms_plain * 1e-3) / 1e6
    v_thin = useful_cells * K / (ms_thin * 1e-3) / 1e6
    if verdict["accepted"]:
        deployed, value, ms_dep = "learned", v_thin, ms_thin
    elif verdict_z["accepted"]:
        deployed, value, ms_dep = "learned on z faces, CPML on x and y", v_z, ms_z
    else:
        deployed, value, ms_dep = "cpml", v_plain, ms_plain
    line = {
        "metric": METRIC + " (useful interior)", "value": round(value, 2), "unit": UNIT, "n_gpus": 1, "steps": K,
        "warmup": 3, "ms_per_step": round(ms_dep / K, 5),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 fields; boundary MLP bf16 weights, f32 accumulation (bf16x2 activations)",
        "data": "synthetic (seeded)",
        "config": {"workload": "c5: c2 cavity %s, useful interior %s; 2-cell learned layer (%s grid) or "
                               "8-cell CPML; Poynting on; %d steps" % ("x".join(map(str, shape)),
                                                                      "x".join(map(str, useful)),
                                                                      "x".join(map(str, thin_shape)), K),
                   "teacher": "%d runs at 128^3, 16-cell CPML, 1500 steps, 1-8 spheres eps U[1,12] inside "
                              "the box, dipole pulse period U[10,30] steps, random polarisation" % runs,
                   "l2": "c2 fields (%.0f MB) larger than the 129 MB L2; no flush" % (int(numpy.prod(shape)) * 36 / 1e6)},
        "deployed": deployed, "candidate_timed": pick,
        "verdicts": {name: {k: (round(v, 2) if isinstance(v, float) and math.isfinite(v) else
                                ({str(a): round(b, 2) for a, b in v.items()} if isinstance(v, dict) else v))
                            for k, v in vd.items()} for name, vd in verdicts.items()},
        "first_pass_reflection_db": {"learned": round(first_pass["reflection_db"], 2),
                                     "zero_ghost_layer": round(held_first["reflection_db"], 2)},
        "zero_ghost_layer_reflection_db": round(held["reflection_db"], 2),
        "training": {"data_seconds": round(data_s, 1), "fit_seconds": round(train_s, 1),
                     "samples_per_face": samples, "memory": round(L.MUR_MEMORY, 5),
                     "relative_loss_per_face": rel},
        "evaluate_seconds": round(evaluate_s, 1),
        "plain_cpml8": {"ms": round(ms_plain, 3), "useful_mcells_per_s": round(v_plain, 2),
                        "grid": list(shape)},
        "thin_learned": {"precision": "linear" if lin_ok else "bf16x2",
                         "ms": round(ms_thin, 3), "useful_mcells_per_s": round(v_thin, 2), "grid": list(thin_shape),
                         "finite_after_steps": finite,
                         "interior_rel_l2_vs_plain_cpml8": l2 if math.isfinite(l2) else "inf",
                         "predict_ms_per_step": round(ms_pred, 4), "boundary_columns": n_cols},
        "thin_z_learned": {"faces": "learned on z (air), 8-cell CPML on x and y", "precision": zprec,
                           "ms": round(ms_z, 3), "useful_mcells_per_s": round(v_z, 2), "grid": list(zshape),
                           "vs_plain": round(v_z / v_plain, 3), "finite_after_steps": fin_z,
                           "interior_rel_l2_vs_plain_cpml8": l2_z if math.isfinite(l2_z) else "inf",
                           "verdict": {k: (round(v, 2) if isinstance(v, float) and math.isfinite(v) else
                                           ({str(a): round(b, 2) for a, b in v.items()} if isinstance(v, dict) else v))
                                       for k, v in verdict_z.items()}},
        "roofline": {"bound": "tensor", "achieved": round(flops / (ms_pred * 1e-3) / 1e12, 2),
                     "peak": tc_peak, "unit": "TFLOP/s", "frac": round(flops / (ms_pred * 1e-3) / 1e12 / tc_peak, 4),
                     "traffic": None, "kernel": "k_lbc_predict_mma<split> (bf16 mma.sync, algorithmic FLOPs "
                                               "of one bf16 pass)"},
        "gpu_launches": "thin: 4 + the plain step's per step; plain: the plain step's",
    }
    return line


def run_c5(args):
    """The learned thin boundary of c5 at its stated teacher-run count, as one JSON line."""
    print(json.dumps(c5_measure(args.c5_runs, args.c5_steps)), flush=True)


if __name__ == "__main__":
    _a = parse()
    if _a.workload == "c4" and _a.impl == "ours":
        run_c4(_a)
    elif _a.workload == "c5" and _a.impl == "ours":
        run_c5(_a)
    elif _a.workload == "c3" and _a.impl == "ours":
        run_c3(_a)
    else:
        main()
