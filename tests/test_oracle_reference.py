"""Pin the C restatement against the reference run live (its own Simulation class and rendered
kernel text, oracle/ref_harness.py) on seeded random configurations. Needs the reference
source tree; skipped where it is absent."""
import copy

import numpy
import pytest

from oracle import port, ref_harness

pytestmark = pytest.mark.skipif(not ref_harness.available(), reason="reference tree absent")


def _pair(seed, shape, pmls, poynting, steps, **kw):
    rng = numpy.random.default_rng(seed)
    eps = [rng.uniform(1, 5, shape).astype(numpy.float32) for _ in range(3)]
    eps[rng.integers(0, 3)][rng.integers(0, shape[0]), :, :] = numpy.inf
    init = {k: [rng.standard_normal(shape).astype(numpy.float32) for _ in range(3)] for k in "EH"}
    a = ref_harness.RefSimulation(eps, copy.deepcopy(pmls), initial_fields=init, do_poynting=poynting,
                                  nthreads=2, **kw)
    b = port.PortSimulation(eps, copy.deepcopy(pmls), initial_fields=init, do_poynting=poynting,
                            nthreads=2, **kw)
    N = int(numpy.prod(shape))
    ind = int(rng.integers(0, 3 * N))
    for t in range(steps):
        for s in (a, b):
            s.update_E([])
            s.E[ind] += float(numpy.cos(0.2 * t))
            s.update_H([])
            if poynting:
                s.update_S([])
    for k in ("E", "H") + (("S",) if poynting else ()):
        assert numpy.array_equal(numpy.asarray(getattr(a, k)), getattr(b, k)), k


@pytest.mark.parametrize("seed", range(6))
def test_random_configs(seed):
    rng = numpy.random.default_rng(100 + seed)
    shape = tuple(int(v) for v in rng.integers(5, 14, 3))
    faces = [(a, p) for a in "xyz" for p in "np"]
    rng.shuffle(faces)
    nf = int(rng.integers(0, 7))
    pmls = []
    for a, p in faces[:nf]:
        d = {"axis": a, "polarity": p, "thickness": int(rng.integers(1, 5))}
        if rng.random() < 0.5:
            d.update(m=float(rng.uniform(2, 4)), ln_R_per_layer=float(rng.uniform(-3, -1)),
                     cfs_alpha=float(rng.uniform(0, 0.1)), ma=int(rng.integers(1, 3)),
                     epsilon_eff=float(rng.uniform(1, 3)), mu_eff=float(rng.uniform(1, 2)))
        pmls.append(d)
    _pair(seed, shape, pmls, bool(seed % 2), 12)


def test_dt_and_spacing_variants():
    shape = (8, 7, 6)
    pm = [{"axis": a, "polarity": p, "thickness": 2} for a in "xyz" for p in "np"]
    _pair(7, shape, pm, True, 10, dt=0.3)
    _pair(8, shape, pm, True, 10, dxes=2.5)
