"""
Write tests/golden/geometry_pcgen.npz from the reference's own lattice generator.

The reference's pcgen.py (triangular_lattice, pcgen.py:11-48; ln_defect, pcgen.py:93-108) is
imported from its source tree (oracle/ref_harness.py locates it) and called for the cases in
CASES; the returned hole arrays are saved so that the restatement in
opencl_fdtd_gb300/geometry.py can be checked where the reference is absent. pcgen.py was
written for numpy 1.x; the module sees a numpy whose two calls it relies on behave as they did
there: ``linspace`` accepts the integral float count pcgen.py passes (``dims[0] - k * j_odd``,
pcgen.py:41-42; numpy 2 raises TypeError) and ``in1d`` (removed in numpy 2.4) is ``isin``,
the same membership test.

Usage (needs the reference source tree):  python tests/golden/make_geometry_golden.py
"""
from __future__ import annotations

import importlib.util
import os
import sys

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import ref_harness  # noqa: E402

OUT = os.path.join(HERE, "geometry_pcgen.npz")

# (kind, dims or mirror_dims, defect_length)
CASES = [
    ("lattice", (1, 1), 0), ("lattice", (3, 3), 0), ("lattice", (4, 4), 0),
    ("lattice", (5, 7), 0), ("lattice", (8, 5), 0), ("lattice", (11, 11), 0),
    ("lattice", (17, 13), 0), ("lattice", (21, 21), 0),
    ("ln", (2, 2), 1), ("ln", (3, 3), 3), ("ln", (5, 4), 3), ("ln", (7, 7), 5),
    ("ln", (8, 8), 3), ("ln", (10, 6), 7), ("ln", (12, 12), 3),
]


class _Numpy1:
    """numpy as pcgen.py expects it under numpy 1.x (see the module docstring)."""

    def __getattr__(self, name):
        return getattr(numpy, name)

    @staticmethod
    def linspace(start, stop, num=50, **kw):
        if isinstance(num, (float, numpy.floating)) and float(num).is_integer():
            num = int(num)
        return numpy.linspace(start, stop, num, **kw)

    @staticmethod
    def in1d(a, b, invert=False):
        return numpy.isin(numpy.ravel(a), b, invert=invert)


def load_pcgen():
    path = os.path.join(ref_harness.REF_ROOT, "pcgen.py")
    spec = importlib.util.spec_from_file_location("ref_pcgen", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.numpy = _Numpy1()
    return mod


def reference_holes(pcgen, kind, dims, n):
    if kind == "lattice":
        return pcgen.triangular_lattice(list(dims))
    return pcgen.ln_defect(list(dims), n)


def main():
    if not ref_harness.available():
        raise SystemExit("reference source tree not found at %s" % ref_harness.REF_ROOT)
    pcgen = load_pcgen()
    arrays = {}
    for k, (kind, dims, n) in enumerate(CASES):
        arrays["case%02d" % k] = numpy.asarray(reference_holes(pcgen, kind, dims, n), numpy.float64)
    numpy.savez_compressed(OUT, cases=numpy.array([repr(c) for c in CASES]), **arrays)
    print("wrote", OUT, len(CASES), "cases")


if __name__ == "__main__":
    main()
