"""The field watchdog (fdtd_count_nonfinite, Simulation.nonfinite_count / run(watchdog=K)):
non-finite values are planted from the host into the fields, never produced by a faulting
kernel, and the device count finds exactly them; a watched run stops at the first chunk that
leaves any and otherwise gives the same bits as an unwatched run."""
import math

import numpy
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def _sim(shape=(12, 10, 8), float_type=numpy.float32, bloch=False, seed=1):
    from opencl_fdtd_gb300 import Simulation
    rng = numpy.random.default_rng(seed)
    eps = [rng.uniform(1, 3, shape).astype(float_type) for _ in range(3)]
    init = {k: [(0.1 * rng.standard_normal(shape)).astype(float_type) for _ in range(3)] for k in "EH"}
    kw = dict(epsilon=eps, pmls=[{"axis": "z", "polarity": p, "thickness": 2} for p in "np"],
              initial_fields=init, do_poynting=False, float_type=float_type)
    if bloch:
        kw["bloch_boundaries"] = [{"axis": "x", "real": math.cos(0.3), "imag": math.sin(0.3)}]
    return Simulation(**kw)


@pytest.mark.parametrize("float_type", [numpy.float32, numpy.float64])
def test_count_finds_exactly_the_planted_values(float_type):
    sim = _sim(float_type=float_type)
    assert sim.nonfinite_count() == 0 and sim.check_finite()
    sim.E[7] = float("nan")
    sim.H[3 * sim.N - 1] = float("inf")
    sim.H[0] = -float("inf")
    assert sim.nonfinite_count() == 3
    assert not sim.check_finite()


def test_count_covers_the_bloch_fields():
    sim = _sim(bloch=True)
    assert sim.nonfinite_count() == 0
    sim.G[5] = float("nan")
    sim.F[2 * sim.N + 1] = float("nan")
    assert sim.nonfinite_count() == 2


def test_watched_run_matches_unwatched_and_stops_on_nonfinite():
    a, b = _sim(seed=4), _sim(seed=4)
    src = [(int(numpy.ravel_multi_index((6, 5, 4), a.shape)) + a.N, [0.2 * math.sin(0.3 * t) for t in range(12)])]
    a.run(12, point_sources=src)
    b.run(12, point_sources=src, watchdog=5)
    torch.cuda.synchronize()
    assert torch.equal(a.E, b.E) and torch.equal(a.H, b.H) and b.steps_run == 12
    c = _sim(seed=5)
    c.E[10] = float("inf")
    with pytest.raises(FloatingPointError):
        c.run(20, watchdog=5)
    assert c.steps_run == 5
