"""CPML coefficient tables: the product generator (opencl_fdtd_gb300/pml.py), the oracle's
restatement and the tables the reference itself computes (simulation.py:284-307, captured
from its own constructor) must agree bit for bit."""
import copy

import numpy
import pytest

from opencl_fdtd_gb300 import pml as gpml
from oracle import port, ref_harness

PMLS = [
    {"axis": "x", "polarity": "n"},
    {"axis": "x", "polarity": "p", "thickness": 5},
    {"axis": "y", "polarity": "n", "thickness": 3, "m": 2, "ma": 2, "cfs_alpha": 0.1},
    {"axis": "z", "polarity": "p", "thickness": 7, "epsilon_eff": 3.0, "mu_eff": 1.7,
     "ln_R_per_layer": -2.3, "m": 4.0},
]


@pytest.mark.parametrize("dtype", [numpy.float32, numpy.float64])
@pytest.mark.parametrize("k", range(len(PMLS)))
def test_product_equals_oracle(dtype, k):
    p = gpml.apply_defaults(copy.deepcopy(PMLS[k]))
    dt = 0.99 / numpy.sqrt(3)
    a = gpml.grading(p, dt, dtype)
    b = port.pml_tables(p, dt, dtype)
    for ta, tb in zip(a[0] + a[1], b[0] + b[1]):
        assert ta.dtype == numpy.dtype(dtype)
        assert numpy.array_equal(ta, tb)


def test_defaults_mutate_caller_dict():
    p = {"axis": "y", "polarity": "p"}
    gpml.apply_defaults(p)
    assert p == {"axis": "y", "polarity": "p", "thickness": 8, "epsilon_eff": 1.0, "mu_eff": 1.0,
                 "ln_R_per_layer": -1.6, "m": 3.5, "cfs_alpha": 0, "ma": 1}


def test_psi_shape():
    assert gpml.psi_shape((10, 11, 12), 0, 8) == (8, 11, 12)
    assert gpml.psi_shape((10, 11, 12), 2, 3) == (10, 11, 3)


@pytest.mark.skipif(not ref_harness.available(), reason="reference tree absent")
def test_product_equals_reference_constructor():
    shape = (12, 11, 10)
    eps = [numpy.ones(shape, numpy.float32)] * 3
    pm = copy.deepcopy(PMLS)
    sim = ref_harness.RefSimulation(eps, pm, do_poynting=False)
    args_e = [c.cell_contents for c in sim.update_E.__closure__
              if c.cell_contents.__class__.__name__ == "OrderedDict"][0]
    args_h = [c.cell_contents for c in sim.update_H.__closure__
              if c.cell_contents.__class__.__name__ == "OrderedDict"][0]
    for p in pm:
        te, th = gpml.grading(p, sim.dt, numpy.float32)
        for i in range(3):
            ref_e = numpy.asarray(args_e["float *p%s%de%s" % (p["axis"], i, p["polarity"])])
            ref_h = numpy.asarray(args_h["float *p%s%dh%s" % (p["axis"], i, p["polarity"])])
            assert ref_e.dtype == numpy.float32 and numpy.array_equal(ref_e, te[i])
            assert ref_h.dtype == numpy.float32 and numpy.array_equal(ref_h, th[i])
