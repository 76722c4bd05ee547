"""The benchmarked workload itself (395 x 345 x 73 L3 photonic-crystal slab, 8-cell CPML on six
faces, Ey Gaussian pulse, Poynting on) through the default Simulation.run path against the
oracle bit for bit, and the float32 result's error against float64 at the
workload's stated 8000 steps.

The oracle (the C restatement, itself pinned bit for bit to the reference's own kernels) steps
the same inputs with the per-call loop of fdtd.py:161-179 (update_E, the soft source, update_H,
update_S). The float64 reference for the 8000-step error is the same update in float64 on the
GPU, which equals the float64 oracle bit for bit (test_gpu_parity's float64 cases)."""
import copy
import math
import os

import numpy
import pytest

torch = pytest.importorskip("torch")

from oracle import port  # noqa: E402
from opencl_fdtd_gb300 import workloads  # noqa: E402

pytestmark = pytest.mark.gpu

K = 200


def _wave(wl, n):
    return [wl["wave"](t) for t in range(n)]


def _auto_hs_xchunk(sx, nrowblk, extra, nsm):
    """The H+S kernel's automatic x chunk: among 14..24 planes the one whose grid best fills
    whole waves of two resident blocks per SM (the smallest on a tie)."""
    best, best_eff = 16, -1.0
    for xc in range(14, 25):
        waves = (nrowblk * -(-sx // xc) + extra) / (2.0 * nsm)
        eff = waves / math.ceil(waves)
        if eff > best_eff + 1e-12:
            best, best_eff = xc, eff
    return best


def test_config2_run_path_bitwise_against_oracle():
    """The default run path (E kernel adding the source, H+S kernel with its automatic x chunk,
    programmatic dependent launches) at the benchmarked workload, bit for bit."""
    from opencl_fdtd_gb300 import Simulation
    wl = workloads.c2()
    g = Simulation(**copy.deepcopy(wl["kwargs"]))
    vals = _wave(wl, K)
    g.run(K, point_sources=[(wl["source_index"], vals)])
    assert g.tuning("last_run_path") == 2 and g.tuning("pdl") == 1
    sx, sy, sz = wl["shape"]
    nsm = torch.cuda.get_device_properties(0).multi_processor_count
    assert g.tuning("hs_xchunk_used") == _auto_hs_xchunk(sx, -(-sy // (448 // sz - 1)), 0, nsm)
    if nsm == 152:
        assert g.tuning("hs_xchunk_used") == 18
    c = port.PortSimulation(nthreads=os.cpu_count(), **copy.deepcopy(wl["kwargs"]))
    ind = wl["source_index"]
    for t in range(K):
        c.update_E()
        c.E[ind] = c.E[ind] + numpy.float32(vals[t])
        c.update_H()
        c.update_S()
    for k in ("E", "H", "S"):
        got, want = g.get(k), getattr(c, k).reshape(-1)
        bad = numpy.flatnonzero(got != want)
        assert bad.size == 0, (k, bad[:5])
    assert numpy.abs(g.get("E")).max() > 0


def fp64_error(wl, steps):
    """relative L2 of the float32 run against the float64 run, per field"""
    from opencl_fdtd_gb300 import Simulation
    vals = _wave(wl, steps)
    g = Simulation(**copy.deepcopy(wl["kwargs"]))
    g.run(steps, point_sources=[(wl["source_index"], vals)])
    kw = copy.deepcopy(wl["kwargs"])
    kw["epsilon"] = [e.astype(numpy.float64) for e in kw["epsilon"]]
    kw["float_type"] = numpy.float64
    d = Simulation(**kw)
    d.run(steps, point_sources=[(wl["source_index"], vals)])
    out = {}
    for k in ("E", "H", "S"):
        ref = d.get(k)
        out[k] = float(numpy.linalg.norm(g.get(k).astype(numpy.float64) - ref) / numpy.linalg.norm(ref))
    return out


def test_config2_fp64_error_at_stated_steps():
    wl = workloads.c2()
    err = fp64_error(wl, wl["steps"])
    print("config2 float32 vs float64 relative L2 after %d steps: %s" % (wl["steps"], err))
    assert all(numpy.isfinite(v) and v < 1e-2 for v in err.values()), err
