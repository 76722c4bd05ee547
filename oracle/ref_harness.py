"""
Oracle A — the reference itself, run on the CPU (TEST INFRASTRUCTURE).

This module imports the reference's own ``opencl_fdtd.Simulation`` from its source tree and
runs it unmodified, with only the OpenCL runtime replaced:

* ``pyopencl`` is replaced by a small fake whose ``ElementwiseKernel`` wraps the rendered
  kernel body (the reference's own jinja2 output) in a C loop over the launch range, compiles
  it with ``gcc -O3 -fopenmp -ffp-contract=off`` into ``oracle/_ref/`` and calls it through
  ctypes. The launch range is the size of the first vector argument, as in pyopencl's
  ElementwiseKernel (opencl_fdtd/simulation.py:321-326), so the 3N range and the guard of
  opencl_fdtd/kernels/common.cl:23-25 run as written.
* ``pyopencl.array`` device arrays become numpy arrays with a ``get()`` method.
* ``fdfd_tools.vec`` (third-party, pinned ``fdfd_tools>=0.3`` in setup.py:25, ``@master`` in
  requirements.txt:8; called at simulation.py:347,357) is restated: it concatenates the
  C-order ravel of each component.
* The reference computes its CPML tables (simulation.py:284-307) for numpy 1.x value-based
  casting, where float32 arrays stay float32 against float64 scalars. numpy 2 promotes them to
  float64 and the float64 buffers would then be read through ``float *`` kernel arguments.
  The module-level ``numpy`` seen by simulation.py is therefore a shim whose ``sqrt`` of a
  scalar returns a Python float; ``dt`` and ``kappa_max`` then stay weak scalars and every
  table is computed in float32 arithmetic, as under numpy 1.x.

It needs the reference source tree and jinja2. The tree is ``$OPENCL_FDTD_REF`` when that is
set, else a checkout named ``reference`` beside this repository's folder (``../reference``
relative to the repository root); without either, ``available()`` is False and the tests that
need the reference skip. It pins the C restatement (fdtd_port.c) and writes the golden
fixtures under tests/golden/. ``export_replay`` also saves a rendered case (C sources,
argument manifest, coefficient tables) so that ``ref_replay`` can run the reference kernels
where the source tree is absent.
"""
from __future__ import annotations

import ctypes
import hashlib
import json
import os
import re
import subprocess
import sys
import types

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("OPENCL_FDTD_REF") or os.path.join(
    os.path.dirname(os.path.dirname(HERE)), "reference")
REF_OUT = os.path.join(HERE, "_ref")

_CTYPE = {
    "float": (ctypes.c_float, numpy.float32),
    "double": (ctypes.c_double, numpy.float64),
    "uint": (ctypes.c_uint, numpy.uint32),
    "int": (ctypes.c_int, numpy.int32),
}


def available() -> bool:
    return os.path.isfile(os.path.join(REF_ROOT, "opencl_fdtd", "simulation.py"))


# --------------------------------------------------------------------------------------------
# gcc wrapper for rendered ElementwiseKernel bodies
# --------------------------------------------------------------------------------------------
def parse_arguments(arguments: str):
    """Split a pyopencl argument string into (ctype, is_pointer, name) triples."""
    out = []
    for part in arguments.split(","):
        part = part.strip()
        m = re.match(r"^(\w+)\s*(\*?)\s*(\w+)$", part)
        if not m:
            raise ValueError("cannot parse kernel argument %r" % part)
        out.append((m.group(1), m.group(2) == "*", m.group(3)))
    return out


def wrap_c(operation: str, args) -> str:
    lines = [
        "/* generated from the reference's rendered kernel body; see oracle/ref_harness.py */",
        "#include <stddef.h>",
        "#include <stdint.h>",
        "#include <omp.h>",
        "typedef unsigned int uint;",
        "#define __global",
        "#define PYOPENCL_ELWISE_CONTINUE continue",
        "static int g_nthr = 0;",
        "void set_threads(int n) { g_nthr = n; }",
        "void run(void **argv, long n) {",
    ]
    for k, (ct, is_ptr, name) in enumerate(args):
        if is_ptr:
            lines.append("    %s *%s = (%s *)argv[%d];" % (ct, name, ct, k))
        else:
            lines.append("    const %s %s = *(const %s *)argv[%d];" % (ct, name, ct, k))
    lines.append("#pragma omp parallel for schedule(static) num_threads(g_nthr > 0 ? g_nthr : omp_get_max_threads())")
    lines.append("    for (long i_ = 0; i_ < n; ++i_) {")
    lines.append("        const size_t i = (size_t)i_;")
    lines.append(operation)
    lines.append("    }")
    lines.append("}")
    return "\n".join(lines) + "\n"


_LIB_CACHE: dict = {}


def compile_c(src: str, tag: str = "k"):
    """Compile a wrapped kernel into oracle/_ref/<tag>_<hash>.so (cached) and return the CDLL."""
    h = hashlib.sha256(src.encode()).hexdigest()[:16]
    if h in _LIB_CACHE:
        return _LIB_CACHE[h]
    os.makedirs(REF_OUT, exist_ok=True)
    base = os.path.join(REF_OUT, "%s_%s" % (tag, h))
    cpath, sopath = base + ".c", base + ".so"
    if not os.path.exists(sopath):
        with open(cpath, "w") as f:
            f.write(src)
        tmp = sopath + ".%d.tmp" % os.getpid()
        subprocess.check_call(["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
                               "-w", cpath, "-o", tmp])
        os.replace(tmp, sopath)
    lib = ctypes.CDLL(sopath)
    lib.run.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_long]
    lib.run.restype = None
    lib.set_threads.argtypes = [ctypes.c_int]
    _LIB_CACHE[h] = lib
    return lib


def call_kernel(lib, args_decl, values, nthreads: int = 0):
    """Invoke a compiled body: vector args are numpy arrays, scalars are cast to their ctype."""
    argv = (ctypes.c_void_p * len(args_decl))()
    keep = []
    n = None
    for k, ((ct, is_ptr, name), v) in enumerate(zip(args_decl, values)):
        if is_ptr:
            a = numpy.asarray(v)
            if a.dtype != _CTYPE[ct][1]:
                raise TypeError("argument %s: %s buffer passed for %s *" % (name, a.dtype, ct))
            if not a.flags.c_contiguous:
                raise ValueError("argument %s is not contiguous" % name)
            if n is None:
                n = a.size
            argv[k] = a.ctypes.data
            keep.append(a)
        else:
            cv = _CTYPE[ct][0](v)
            keep.append(cv)
            argv[k] = ctypes.cast(ctypes.pointer(cv), ctypes.c_void_p)
    lib.set_threads(int(nthreads))
    lib.run(argv, ctypes.c_long(n))
    return keep


# --------------------------------------------------------------------------------------------
# fake pyopencl / fdfd_tools
# --------------------------------------------------------------------------------------------
class FakeArray(numpy.ndarray):
    """Stand-in for pyopencl.array.Array: host memory with the ``get()`` the example script (fdtd.py) uses."""

    def get(self):
        return numpy.array(self)


class _Event:
    def wait(self):
        return None


class FakeElementwiseKernel:
    nthreads = 0
    sources: list = []

    def __init__(self, context, operation, arguments, name="elwise", **kwargs):
        self.args = parse_arguments(arguments)
        self.operation = operation
        self.csrc = wrap_c(operation, self.args)
        self.lib = compile_c(self.csrc)
        FakeElementwiseKernel.sources.append(self)

    def __call__(self, *values, wait_for=None, **kwargs):
        call_kernel(self.lib, self.args, values, FakeElementwiseKernel.nthreads)
        return _Event()


def _vec(f):
    """fdfd_tools.vec restated: C-order ravel of each component, concatenated."""
    if f is None:
        return None
    return numpy.hstack(tuple(numpy.asarray(fi).flatten(order="C") for fi in f))


def _install_fakes():
    if "pyopencl" in sys.modules and getattr(sys.modules["pyopencl"], "_is_fake", False):
        return
    cl = types.ModuleType("pyopencl")
    cl._is_fake = True
    cl.create_some_context = lambda *a, **k: object()
    cl.CommandQueue = lambda *a, **k: object()
    cl.Context = object
    cl.Event = _Event
    arr = types.ModuleType("pyopencl.array")
    arr.Array = FakeArray

    def to_device(queue, a):
        return numpy.array(a, copy=True).view(FakeArray)

    def zeros(queue, shape, dtype):
        return numpy.zeros(shape, dtype=dtype).view(FakeArray)

    def zeros_like(a):
        return numpy.zeros_like(numpy.asarray(a)).view(FakeArray)

    arr.to_device, arr.zeros, arr.zeros_like = to_device, zeros, zeros_like
    elw = types.ModuleType("pyopencl.elementwise")
    elw.ElementwiseKernel = FakeElementwiseKernel
    cl.array, cl.elementwise = arr, elw
    sys.modules["pyopencl"] = cl
    sys.modules["pyopencl.array"] = arr
    sys.modules["pyopencl.elementwise"] = elw
    ft = types.ModuleType("fdfd_tools")
    ft.vec = _vec
    ft.unvec = lambda v, shape: None if v is None else v.reshape((3, *shape), order="C")
    sys.modules.setdefault("fdfd_tools", ft)


class _NumpyShim(types.ModuleType):
    """numpy as simulation.py sees it: scalar sqrt returns a weak Python float (numpy 1.x casting)."""

    def __getattr__(self, name):
        return getattr(numpy, name)

    @staticmethod
    def sqrt(v):
        if numpy.ndim(v) == 0:
            return float(numpy.sqrt(v))
        return numpy.sqrt(v)


_REF_MOD = None


def reference_module():
    """Import opencl_fdtd.simulation from the reference tree with the fakes installed."""
    global _REF_MOD
    if _REF_MOD is not None:
        return _REF_MOD
    if not available():
        raise RuntimeError("reference source tree not found at %s" % REF_ROOT)
    _install_fakes()
    if REF_ROOT not in sys.path:
        sys.path.insert(0, REF_ROOT)
    import importlib
    mod = importlib.import_module("opencl_fdtd.simulation")
    mod.numpy = _NumpyShim("numpy")
    _REF_MOD = mod
    return mod


class _WeakIterArray(numpy.ndarray):
    """Spacing table whose elements iterate as Python floats, so that ``min(min(dxn) ...)`` at
    simulation.py:142 yields a weak scalar and dt stays weak (numpy 1.x casting)."""

    def __iter__(self):
        for v in numpy.asarray(self).tolist():
            yield v

    def __rtruediv__(self, other):
        # 1 / dxn at simulation.py:141 yields a plain array again
        return numpy.asarray(other) / numpy.asarray(self)


def RefSimulation(*args, nthreads: int = 0, **kwargs):
    """Construct the reference's own Simulation (arguments exactly as simulation.py:77-88)."""
    mod = reference_module()
    FakeElementwiseKernel.nthreads = nthreads
    dxes = kwargs.get("dxes")
    if dxes is not None and not isinstance(dxes, (float, int)):
        kwargs["dxes"] = [[numpy.asarray(d, dtype=numpy.float64).view(_WeakIterArray) for d in g]
                          for g in dxes]
    return mod.Simulation(*args, **kwargs)


def set_threads(n: int):
    FakeElementwiseKernel.nthreads = int(n)


# --------------------------------------------------------------------------------------------
# Replay export: what the CPU baseline needs where the reference tree is absent
# --------------------------------------------------------------------------------------------
def export_replay(name: str, sim, extra: dict | None = None) -> str:
    """Save the compiled kernels' C sources, their argument manifest and every non-field
    argument (coefficient tables, dt) of a constructed reference Simulation under
    oracle/_ref/replay_<name>/. Field arrays are recorded by role and shape only."""
    out = os.path.join(REF_OUT, "replay_" + name)
    os.makedirs(out, exist_ok=True)
    field_ids = {}
    for attr in ("E", "H", "F", "G", "S", "oS", "eps", "Jr", "Ji"):
        a = getattr(sim, attr, None)
        if a is not None:
            field_ids[id(a)] = attr
    manifest = {"shape": list(sim.shape), "dt": float(sim.dt), "kernels": {}, "extra": extra or {}}
    import collections  # noqa: F401
    # The closures returned by _create_operation hold (update, args); recover them.
    for kname in ("E", "H", "S"):
        fn = getattr(sim, "update_" + kname, None)
        if not fn:
            continue
        cells = {c.cell_contents.__class__.__name__: c.cell_contents for c in fn.__closure__}
        kern = cells["FakeElementwiseKernel"]
        args = cells["OrderedDict"]
        entries = []
        for (decl, value), (ct, is_ptr, nm) in zip(args.items(), kern.args):
            if is_ptr and id(value) in field_ids:
                entries.append({"name": nm, "ctype": ct, "ptr": True, "field": field_ids[id(value)]})
            elif is_ptr:
                a = numpy.asarray(value)
                if nm.startswith("Psi_"):
                    entries.append({"name": nm, "ctype": ct, "ptr": True, "zeros": list(a.shape)})
                else:
                    fn_npy = "%s_%s.npy" % (kname, nm)
                    numpy.save(os.path.join(out, fn_npy), a)
                    entries.append({"name": nm, "ctype": ct, "ptr": True, "npy": fn_npy})
            else:
                entries.append({"name": nm, "ctype": ct, "ptr": False, "value": float(value)})
        with open(os.path.join(out, "update_%s.c" % kname), "w") as f:
            f.write(kern.csrc)
        manifest["kernels"][kname] = entries
    with open(os.path.join(out, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1)
    return out
