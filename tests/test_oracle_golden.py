"""The C restatement (oracle/fdtd_port.c) against golden fixtures written by the reference's
own Simulation class and kernel text (tests/golden/make_golden.py)."""
import json
import os

import numpy
import pytest

from oracle import port
from tests.golden import cases
from tests.golden.make_golden import c1_full, summary

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
GOLD = numpy.load(os.path.join(HERE, "golden_cases.npz"))


def _port(**kw):
    return port.PortSimulation(nthreads=4, **kw)


@pytest.mark.parametrize("name", cases.CASE_NAMES)
def test_port_matches_reference_golden(name):
    sim = cases.run_case(_port, name)
    for k, v in cases.outputs(sim, name).items():
        g = GOLD["%s__%s" % (name, k)]
        assert v.dtype == g.dtype
        # same platform as the fixture writer: bit for bit; elsewhere numpy's float32
        # exp/pow in the CPML tables may round differently, so fall back to 1e-6 rel L2
        if not numpy.array_equal(v, g):
            rel = numpy.linalg.norm((v - g).astype(numpy.float64)) / numpy.linalg.norm(g.astype(numpy.float64))
            assert rel < 1e-6, (name, k, rel)


def test_port_matches_reference_c1_full():
    with open(os.path.join(HERE, "golden_c1_full.json")) as f:
        gold = json.load(f)
    sim = c1_full(lambda **kw: port.PortSimulation(nthreads=os.cpu_count(), **kw))
    for k in ("E", "H"):
        s = summary(sim.E if k == "E" else sim.H)
        numpy.testing.assert_allclose(s["l2"], gold[k]["l2"], rtol=1e-6)
        numpy.testing.assert_allclose(s["sample"], gold[k]["sample"], rtol=1e-4, atol=1e-6)
