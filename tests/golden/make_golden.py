"""
Write the golden fixtures under tests/golden/ from the reference itself.

Every case of cases.py is run through the reference's own Simulation class and kernel text
(oracle/ref_harness.py: opencl_fdtd/simulation.py with a CPU stand-in for the OpenCL runtime),
and the final fields are saved. The full config-1 run (64^3, 8-cell CPML on six faces,
eps = 12.25 slab for z in [24, 40), soft Ez Gaussian-sine source at (32, 32, 32), 500 steps,
Poynting off) is saved as a summary: per-component L2 norms, a SHA-256 of the float32 bytes
and every 97th element.

Usage (needs the reference source tree and jinja2):  python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import ref_harness  # noqa: E402
from tests.golden import cases  # noqa: E402


def c1_full(sim_cls, steps=500, **extra):
    """Config 1 at full size: 64^3, 8-cell CPML on 6 faces, slab z in [24, 40) eps=12.25."""
    shape = (64, 64, 64)
    eps = [numpy.ones(shape, numpy.float32) for _ in range(3)]
    for e in eps:
        e[:, :, 24:40] = 12.25
    pmls = [{"axis": a, "polarity": p, "thickness": 8} for a in "xyz" for p in "np"]
    sim = sim_cls(epsilon=eps, pmls=pmls, do_poynting=False, **extra)
    N = 64 ** 3
    ind = int(numpy.ravel_multi_index((32, 32, 32), shape)) + 2 * N
    for t in range(steps):
        sim.update_E([])
        sim.E[ind] += cases.pulse_c1(t)
        sim.update_H([])
    return sim


def summary(a: numpy.ndarray) -> dict:
    a = numpy.ascontiguousarray(a, dtype=numpy.float32)
    n = a.size // 3
    return {"sha256": hashlib.sha256(a.tobytes()).hexdigest(),
            "l2": [float(numpy.linalg.norm(a[k * n:(k + 1) * n].astype(numpy.float64))) for k in range(3)],
            "sample": a[::97].tolist()}


def main():
    if not ref_harness.available():
        raise SystemExit("reference source tree not found")
    out = {}
    for name in cases.CASE_NAMES:
        sim = cases.run_case(lambda **kw: ref_harness.RefSimulation(nthreads=4, **kw), name)
        res = cases.outputs(sim, name)
        for k, v in res.items():
            out["%s__%s" % (name, k)] = v
        print(name, {k: float(numpy.abs(v).max()) for k, v in res.items()})
    numpy.savez_compressed(os.path.join(HERE, "golden_cases.npz"), **out)
    sim = c1_full(lambda **kw: ref_harness.RefSimulation(nthreads=os.cpu_count(), **kw))
    doc = {"case": "config1_64cube_500steps", "E": summary(sim.E), "H": summary(sim.H)}
    with open(os.path.join(HERE, "golden_c1_full.json"), "w") as f:
        json.dump(doc, f)
    print("c1 full", doc["E"]["l2"], doc["H"]["l2"])


if __name__ == "__main__":
    main()
