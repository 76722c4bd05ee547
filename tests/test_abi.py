"""The C-ABI library: it loads without a GPU, exports every entry point include/*.h declares,
and the ctypes mirrors of its structures match the C compiler's layout of the header."""
import ctypes
import glob
import os
import re
import subprocess

import pytest

from opencl_fdtd_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = sorted(glob.glob(os.path.join(ROOT, "include", "*.h")))


def declared_functions():
    names = []
    for h in HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:int|const char\s*\*)\s*(fdtd_\w+)\s*\(", text, flags=re.M)
    return names


def test_library_loads_and_exports_every_declared_symbol():
    lib = _lib.load()
    names = declared_functions()
    assert len(names) >= 11
    for n in names:
        assert hasattr(lib, n), n
    bound = {s[0] for s in _lib.SIGNATURES}
    assert set(names) == bound
    assert lib.fdtd_abi_version() == 1


def test_header_constants_match_the_python_mirror():
    """Every integer #define of the header (status codes, dtypes, tuning and read-back keys,
    run paths, storage and precision codes) has the same value in the ctypes mirror."""
    defs = {}
    for h in HEADERS:
        defs.update(re.findall(r"^#define\s+(FDTD_\w+)\s+(-?\d+)\s*(?:/\*.*)?$", open(h).read(), flags=re.M))
    assert len(defs) >= 40
    lib = _lib.load()
    for name, value in defs.items():
        if name == "FDTD_ABI_VERSION":
            assert lib.fdtd_abi_version() == int(value)
            continue
        assert getattr(_lib, name) == int(value), name


def test_errors_without_a_gpu_call():
    lib = _lib.load()
    plan = ctypes.c_void_p()
    assert lib.fdtd_plan_create(None, ctypes.byref(plan)) == _lib.FDTD_ERR_INVALID
    assert b"desc" in lib.fdtd_last_error()
    d = _lib.FdtdDesc()
    d.shape[0], d.shape[1], d.shape[2] = 4, 4, 4
    d.dtype, d.uniform, d.dt, d.dx = 7, 1, 0.5, 1.0
    assert lib.fdtd_plan_create(ctypes.byref(d), ctypes.byref(plan)) == _lib.FDTD_ERR_UNSUPPORTED
    d.dtype = _lib.FDTD_F32
    d.n_pml = 2
    d.pml[0].axis = d.pml[1].axis = 1
    d.pml[0].polarity = d.pml[1].polarity = 0
    assert lib.fdtd_plan_create(ctypes.byref(d), ctypes.byref(plan)) == _lib.FDTD_ERR_INVALID
    assert b"duplicate" in lib.fdtd_last_error()
    d.n_pml = 0
    d.shape[0] = 70000
    assert lib.fdtd_plan_create(ctypes.byref(d), ctypes.byref(plan)) == _lib.FDTD_ERR_INVALID
    assert lib.fdtd_update_e(None, None, None) == _lib.FDTD_ERR_INVALID


STRUCTS = {
    "FdtdPmlDesc": _lib.FdtdPmlDesc,
    "FdtdBlochDesc": _lib.FdtdBlochDesc,
    "FdtdDesc": _lib.FdtdDesc,
    "FdtdBuffers": _lib.FdtdBuffers,
    "FdtdPointSources": _lib.FdtdPointSources,
    "FdtdBatchFace": _lib.FdtdBatchFace,
    "FdtdBatchVariant": _lib.FdtdBatchVariant,
}


def test_struct_layout_matches_header(tmp_path):
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "fdtd_gb300.h"', "int main(void) {"]
    for sname, cls in STRUCTS.items():
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (sname, sname))
        for fname, _ in cls._fields_:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (sname, fname, sname, fname))
    lines += ["return 0; }"]
    src = tmp_path / "probe.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "probe"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    out = dict(l.split() for l in subprocess.check_output([str(exe)], text=True).splitlines())
    for sname, cls in STRUCTS.items():
        assert int(out[sname]) == ctypes.sizeof(cls), sname
        for fname, _ in cls._fields_:
            assert int(out["%s.%s" % (sname, fname)]) == getattr(cls, fname).offset, (sname, fname)


def test_no_cpu_fallback():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import numpy
    from opencl_fdtd_gb300 import Simulation
    with pytest.raises(RuntimeError, match="CUDA"):
        Simulation([numpy.ones((4, 4, 4), numpy.float32)] * 3, [])


def test_type_to_C():
    import numpy
    from opencl_fdtd_gb300 import type_to_C
    assert type_to_C(numpy.float16) == "half"
    assert type_to_C(numpy.float32) == "float"
    assert type_to_C(numpy.float64) == "double"
    with pytest.raises(Exception):
        type_to_C(numpy.int32)
