"""The lattice generator (opencl_fdtd_gb300/geometry.py) against the reference's pcgen.py.

``triangular_lattice`` and ``ln_defect`` restate pcgen.py:11-48 and 93-108. The fixture
tests/golden/geometry_pcgen.npz holds pcgen.py's own output for 15 cases (written by
tests/golden/make_geometry_golden.py); the live test repeats the comparison against the
reference tree itself when it is present.
"""
import os

import numpy
import pytest

from opencl_fdtd_gb300 import geometry
from oracle import ref_harness
from tests.golden import make_geometry_golden as mk

FIXTURE = os.path.join(os.path.dirname(__file__), "golden", "geometry_pcgen.npz")


def ours(kind, dims, n):
    return geometry.triangular_lattice(dims) if kind == "lattice" else geometry.ln_defect(dims, n)


@pytest.mark.parametrize("k", range(len(mk.CASES)))
def test_holes_equal_pcgen_fixture(k):
    kind, dims, n = mk.CASES[k]
    want = numpy.load(FIXTURE)["case%02d" % k]
    got = ours(kind, dims, n)
    assert got.shape == want.shape
    assert numpy.array_equal(got, want)


@pytest.mark.skipif(not ref_harness.available(), reason="reference tree absent")
@pytest.mark.parametrize("dims,n", [((6, 6), 3), ((9, 5), 1), ((13, 13), 5), ((4, 9), 3)])
def test_holes_equal_pcgen_live(dims, n):
    pcgen = mk.load_pcgen()
    assert numpy.array_equal(geometry.triangular_lattice(dims),
                             mk.reference_holes(pcgen, "lattice", dims, 0))
    assert numpy.array_equal(geometry.ln_defect(dims, n), mk.reference_holes(pcgen, "ln", dims, n))


def test_ln_defect_rejects_even_length():
    with pytest.raises(ValueError):
        geometry.ln_defect((3, 3), 2)
