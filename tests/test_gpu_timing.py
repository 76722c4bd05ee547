"""The profiling hook of fdtd_run (FDTD_TUNE_TIMING + fdtd_run_kernel_ms): per-kernel CUDA
event times are recorded on the H+S path and the fields are the same as without it."""
import copy
import ctypes

import numpy
import pytest

torch = pytest.importorskip("torch")

from tests.golden import cases  # noqa: E402

pytestmark = pytest.mark.gpu


def test_kernel_timing_hook():
    from opencl_fdtd_gb300 import Simulation, _lib
    kw, _ = cases.build("pml_mixed")
    kw["do_poynting"] = True
    a = Simulation(**copy.deepcopy(kw))
    b = Simulation(**copy.deepcopy(kw))
    lib = b._lib
    ms = (ctypes.c_double * 2)()
    n = ctypes.c_int32()
    _lib.check(lib.fdtd_run_kernel_ms(b._plan, ms, ctypes.byref(n)))
    assert n.value == 0
    _lib.check(lib.fdtd_plan_tune(b._plan, _lib.FDTD_TUNE_TIMING, 1))
    a.run(100, path="hs")
    b.run(100, path="hs")
    _lib.check(lib.fdtd_run_kernel_ms(b._plan, ms, ctypes.byref(n)))
    assert n.value == 50 and ms[0] > 0 and ms[1] > 0
    for k in ("E", "H", "S"):
        assert torch.equal(getattr(a, k), getattr(b, k)), k
    with pytest.raises(Exception):
        _lib.check(lib.fdtd_plan_tune(b._plan, _lib.FDTD_TUNE_TIMING, 2))
