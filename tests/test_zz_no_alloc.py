"""fdtd_plane_sum_noalloc, the plane-sum entry point that allocates nothing.

Some callers cannot allocate device memory between time steps: a host time-stepping driver
that has handed the device memory to its own pool, or a monitoring callback between queued
steps, where cudaMalloc / cudaFree would synchronize the device. For them the FP64 plane sum
keeps its per-block partial sums in a static device array of the library instead of caller
scratch. This test calls it through the C ABI and checks it against fdtd_plane_sum (which
uses caller scratch) on two calls in a row, with the field changing in between, and that a
partial-sum count beyond the static array is rejected.

This file is collected last so that a run stopping at the first failure has already run
every other test."""
import ctypes

import numpy
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def test_noalloc_plane_sum_matches_scratch_entry_point():
    from opencl_fdtd_gb300 import Simulation, _lib
    shape = (20, 17, 13)
    rng = numpy.random.default_rng(77)
    eps = [rng.uniform(1, 4, shape).astype(numpy.float32) for _ in range(3)]
    init = {k: [rng.standard_normal(shape).astype(numpy.float32) for _ in range(3)] for k in "EH"}
    pmls = [{"axis": a, "polarity": p, "thickness": 3} for a in "xyz" for p in "np"]
    sim = Simulation(eps, pmls, initial_fields=init, do_poynting=True)
    sim.run(3)
    lib = _lib.load()
    st = ctypes.c_void_p(sim.queue.cuda_stream)
    scratch = torch.empty(256, dtype=torch.float64, device=sim.device)
    ref = torch.empty(1, dtype=torch.float64, device=sim.device)
    got = torch.empty(1, dtype=torch.float64, device=sim.device)
    for call in range(2):
        for name in ("S", "E", "H"):
            field = getattr(sim, name)
            for axis in range(3):
                for comp in range(3):
                    for plane in (0, shape[axis] // 2, shape[axis] - 1):
                        for nblk in (1, 37, 256):
                            _lib.check(lib.fdtd_plane_sum(sim._plan, field.data_ptr(), comp, axis, plane,
                                                          scratch.data_ptr(), nblk, ref.data_ptr(), st))
                            _lib.check(lib.fdtd_plane_sum_noalloc(sim._plan, field.data_ptr(), comp, axis,
                                                                  plane, nblk, got.data_ptr(), st))
                            sim.queue.synchronize()
                            r, g = float(ref.item()), float(got.item())
                            assert abs(g - r) <= 1e-12 * max(1.0, abs(r)), (call, name, axis, comp, plane, nblk)
        sim.run(2)
    rc = lib.fdtd_plane_sum_noalloc(sim._plan, sim.S.data_ptr(), 0, 0, 0, 1025, got.data_ptr(), st)
    assert rc == _lib.FDTD_ERR_INVALID
    assert b"1024" in lib.fdtd_last_error()
