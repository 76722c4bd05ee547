"""Host logic of the watched run, without a GPU: the chunking of steps and source values and
where it stops (Simulation.run and nonfinite_count replaced by recorders)."""
import numpy
import pytest

from opencl_fdtd_gb300.simulation import Simulation


class _Rec:
    def __init__(self, bad_after=None):
        self.calls = []
        self.steps_run = 0
        self.bad_after = bad_after


def _make(bad_after=None):
    sim = Simulation.__new__(Simulation)
    rec = _Rec(bad_after)

    def run(nsteps, point_sources=None, wait_for=None, monitor=None, path="auto", watchdog=0):
        assert watchdog == 0
        rec.calls.append((nsteps, None if point_sources is None else [list(v) for _, v in point_sources],
                          wait_for))
        sim.steps_run += nsteps
        return "event%d" % len(rec.calls)

    def nonfinite_count():
        return 0 if rec.bad_after is None or sim.steps_run < rec.bad_after else 4

    sim.run = run
    sim.nonfinite_count = nonfinite_count
    sim.steps_run = 0
    return sim, rec


def test_chunks_and_source_slices():
    sim, rec = _make()
    vals = numpy.arange(12.0)
    ev = Simulation._run_watched(sim, 12, 5, [(7, vals)], "w", None, "auto")
    assert [c[0] for c in rec.calls] == [5, 5, 2]
    assert rec.calls[0][1] == [list(range(0, 5))]
    assert rec.calls[2][1] == [[10.0, 11.0]]
    assert [c[2] for c in rec.calls] == ["w", None, None]
    assert ev == "event3" and sim.steps_run == 12


def test_stops_at_the_first_bad_chunk():
    sim, rec = _make(bad_after=10)
    with pytest.raises(FloatingPointError, match="after step 10"):
        Simulation._run_watched(sim, 30, 5, None, None, None, "auto")
    assert sim.steps_run == 10 and len(rec.calls) == 2
