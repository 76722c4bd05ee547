"""Config 3 at full size (128 x 128 x 256 complex, Bloch x/y, CPML z, anisotropic eps/mu
spheres with one PEC sphere, plane-wave source): the CUDA path against the oracle bit for bit
(float32), and its error against the FP64 oracle reported."""
import copy
import os

import numpy
import pytest

torch = pytest.importorskip("torch")

from oracle import port  # noqa: E402
from opencl_fdtd_gb300 import workloads  # noqa: E402

pytestmark = pytest.mark.gpu

STEPS = 120


def _drive(sim, wl, steps, np_like):
    shape = wl["shape"]
    N = int(numpy.prod(shape))
    sx, sy, sz = shape
    z0 = wl["source_plane"]
    # Ex on the whole z = z0 plane
    idx = (numpy.arange(sx)[:, None] * sy * sz + numpy.arange(sy)[None, :] * sz + z0).ravel()
    if not np_like:
        idx = torch.from_numpy(idx).to(sim.device)
    for t in range(steps):
        sim.update_E([])
        sim.update_F([])
        v = wl["wave"](t)
        if np_like:
            sim.E[idx] = sim.E[idx] + sim.E.dtype.type(v)
        else:
            sim.E[idx] += v
        sim.update_H([])
        sim.update_G([])
    return sim


def test_config3_bitwise_and_fp64_error():
    wl = workloads.c3()
    g = _drive(__import__("opencl_fdtd_gb300").Simulation(**copy.deepcopy(wl["kwargs"])), wl, STEPS, False)
    c = _drive(port.PortSimulation(nthreads=os.cpu_count(), **copy.deepcopy(wl["kwargs"])), wl, STEPS, True)
    for k in ("E", "H", "F", "G"):
        assert numpy.array_equal(g.get(k), getattr(c, k)), k
    kw64 = copy.deepcopy(wl["kwargs"])
    kw64["epsilon"] = [e.astype(numpy.float64) for e in kw64["epsilon"]]
    kw64["mu"] = [m.astype(numpy.float64) for m in kw64["mu"]]
    kw64["float_type"] = numpy.float64
    d = _drive(port.PortSimulation(nthreads=os.cpu_count(), **kw64), wl, STEPS, True)
    errs = {}
    for k in ("E", "H", "F", "G"):
        ref = getattr(d, k)
        errs[k] = float(numpy.linalg.norm(g.get(k) - ref) / numpy.linalg.norm(ref))
    print("config3 float32 vs FP64 relative L2 after %d steps:" % STEPS, errs)
    assert all(e < 1e-4 for e in errs.values()), errs


def test_config3_stated_steps_bitwise_and_fp64_error():
    """All 4000 steps of config 3: float32 bit for bit against the oracle; the float64
    reference is the same update in float64 on the GPU (bit-identical to the float64 oracle in
    the 120-step test above)."""
    from opencl_fdtd_gb300 import Simulation
    wl = workloads.c3()
    n = wl["steps"]
    g = _drive(Simulation(**copy.deepcopy(wl["kwargs"])), wl, n, False)
    c = _drive(port.PortSimulation(nthreads=os.cpu_count(), **copy.deepcopy(wl["kwargs"])), wl, n, True)
    for k in ("E", "H", "F", "G"):
        assert numpy.array_equal(g.get(k), getattr(c, k)), k
    kw64 = copy.deepcopy(wl["kwargs"])
    kw64["epsilon"] = [e.astype(numpy.float64) for e in kw64["epsilon"]]
    kw64["mu"] = [m.astype(numpy.float64) for m in kw64["mu"]]
    kw64["float_type"] = numpy.float64
    d = _drive(Simulation(**kw64), wl, n, False)
    errs = {}
    for k in ("E", "H", "F", "G"):
        ref = d.get(k)
        errs[k] = float(numpy.linalg.norm(g.get(k) - ref) / numpy.linalg.norm(ref))
    print("config3 float32 vs FP64 relative L2 after %d steps:" % n, errs)
    assert all(numpy.isfinite(e) and e < 1e-2 for e in errs.values()), errs
