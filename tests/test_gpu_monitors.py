"""FP64 monitors on the GPU: DFT point monitors and their time series against the oracle's
fields, deterministic FP64 plane sums and energy against numpy, and a physics check of the
ringdown fit (a periodic standing wave's frequency equals the Yee dispersion relation)."""
import copy
import math
import os

import numpy
import pytest

torch = pytest.importorskip("torch")

from oracle import port  # noqa: E402
from tests.golden import cases  # noqa: E402

pytestmark = pytest.mark.gpu


def _gpu(**kw):
    from opencl_fdtd_gb300 import Simulation
    return Simulation(**kw)


def test_dft_monitor_matches_oracle_series():
    kw, loop = cases.build("pml_mixed")
    n = 30
    shape = kw["epsilon"][0].shape
    N = int(numpy.prod(shape))
    src = [(int(numpy.ravel_multi_index(p, shape)) + c * N, [cases._WAVES[w](t) for t in range(n)])
           for p, c, w in loop["sources"]]
    pts = [(0, (8, 7, 6)), (1, (3, 3, 9)), (2, (10, 2, 5))]
    om = numpy.array([0.3, 0.7, 1.1])
    g = _gpu(**copy.deepcopy(kw))
    mon = g.dft_monitor(pts, om)
    g.run(n, point_sources=src, monitor=mon)
    c = port.PortSimulation(nthreads=os.cpu_count(), **copy.deepcopy(kw))
    flat = [int(numpy.ravel_multi_index(xyz, shape)) + comp * N for comp, xyz in pts]
    ref = []
    for t in range(n):
        c.update_E()
        for ind, vals in src:
            c.E[ind] = c.E[ind] + numpy.float32(vals[t])
        c.update_H()
        c.update_S()
        ref.append(c.E[flat].astype(numpy.float64))
    ref = numpy.array(ref)
    ser = mon.series()
    assert ser.shape == (n, 3) and numpy.array_equal(ser, ref)
    tt = (numpy.arange(n) + 1) * g.dt
    want = (ref[:, :, None] * numpy.exp(-1j * om[None, None, :] * tt[:, None, None])).sum(0)
    numpy.testing.assert_allclose(mon.spectrum(), want, rtol=1e-11, atol=1e-12)


def test_plane_sums_and_energy_fp64():
    kw, _ = cases.build("periodic_pec_poynting")
    g = _gpu(**copy.deepcopy(kw))
    g.run(7)
    shape = kw["epsilon"][0].shape
    S = g.get("S").astype(numpy.float64).reshape(3, *shape)
    for axis in range(3):
        for idx in (0, shape[axis] // 2, shape[axis] - 1):
            want = numpy.take(S[axis], idx, axis=axis).sum()
            got = g.flux(axis, idx)
            assert abs(got - want) <= 1e-12 * max(1.0, numpy.abs(S[axis]).sum())
    E = g.get("E").astype(numpy.float64)
    H = g.get("H").astype(numpy.float64)
    eps = g.get("eps").astype(numpy.float64)
    fin = numpy.isfinite(eps)
    want = 0.5 * ((eps[fin] * E[fin] ** 2).sum() + (H ** 2).sum())
    assert abs(g.energy() - want) <= 1e-12 * want


def test_standing_wave_frequency_matches_yee_dispersion():
    sx, sy, sz = 48, 2, 2
    m = 3
    k = 2 * math.pi * m / sx
    x = numpy.arange(sx)[:, None, None] * numpy.ones((1, sy, sz))
    zero = numpy.zeros((sx, sy, sz))
    init = {"E": [zero, numpy.cos(k * x), zero]}
    g = _gpu(epsilon=[numpy.ones((sx, sy, sz))] * 3, pmls=[], initial_fields=init,
             float_type=numpy.float64, do_poynting=True)
    mon = g.dft_monitor([(1, (5, 0, 0))], record=True)
    g.run(600, monitor=mon)
    from opencl_fdtd_gb300.analysis import dominant_mode
    fit = dominant_mode(mon.series()[:, 0], g.dt, n_modes=2)
    w_yee = 2 / g.dt * math.asin(g.dt * math.sin(k / 2))
    assert abs(fit["omega"] - w_yee) / w_yee < 1e-9
    assert fit["Q"] > 1e8
    # a lossless periodic box keeps its energy: with E and H half a step apart the sum
    # 1/2 (E^2 + H^2) oscillates at 2*omega, so compare averages over whole periods
    period = 2 * math.pi / w_yee / g.dt
    n = int(round(10 * period))

    def mean_energy():
        vals = []
        for _ in range(n):
            g.run(1)
            vals.append(g.energy())
        return sum(vals) / len(vals)

    e0 = mean_energy()
    g.run(1000)
    assert abs(mean_energy() - e0) / e0 < 2e-3


def test_monitor_on_own_queue_grows_in_order():
    """A monitor on a simulation with its own stream, recorded past its first 1024-row
    buffer while steps are still queued: every row equals the same run on torch's default
    stream, and the series equals per-step samples of the state."""
    kw, _ = cases.build("periodic_pec_poynting")
    shape = kw["epsilon"][0].shape
    N = int(numpy.prod(shape))
    src = [(int(numpy.ravel_multi_index((3, 4, 5), shape)) + 2 * N,
            [math.sin(0.2 * t) * math.exp(-0.5 * ((t - 40) / 12) ** 2) for t in range(1400)])]
    pts = [(2, (3, 4, 5)), (0, (1, 2, 3))]
    q = torch.cuda.Stream()
    a = _gpu(queue=q, **copy.deepcopy(kw))
    mon_a = a.dft_monitor(pts, [0.4])
    b = _gpu(**copy.deepcopy(kw))
    mon_b = b.dft_monitor(pts, [0.4])
    # keep torch's current stream busy so that unordered work on it would show
    big = torch.empty(64 << 20, device="cuda")
    for t0, n in ((0, 700), (700, 700)):
        with torch.cuda.stream(torch.cuda.current_stream()):
            big.mul_(1.0)
        sub = [(i, v[t0:t0 + n]) for i, v in src]
        a.run(n, point_sources=sub, monitor=mon_a)
        b.run(n, point_sources=sub, monitor=mon_b)
    sa, sb = mon_a.series(), mon_b.series()
    assert sa.shape == (1400, 2)
    assert numpy.array_equal(sa, sb)
    assert numpy.array_equal(mon_a.spectrum(), mon_b.spectrum())
    assert numpy.abs(sa).max() > 0


@pytest.mark.parametrize("opts", [{"hs_dft": False, "pdl": False}, {"hs_dft": True, "pdl": False},
                                  {"hs_dft": True, "pdl": True}])
def test_dft_monitor_identical_on_every_run_path(opts):
    """The H+S path takes each step's DFT sample in one extra block of its H+S launch (the
    default, hs_dft), or beside that launch on a side stream (E no longer changes in the step
    by then); the
    series and the accumulators equal those of the per-update path and of the one-pass path
    bit for bit, here with the monitor grown over two runs."""
    rng = numpy.random.default_rng(21)
    shape = (14, 12, 10)
    eps = [rng.uniform(1, 4, shape).astype(numpy.float32) for _ in range(3)]
    pmls = [{"axis": a, "polarity": p, "thickness": 3} for a in "xyz" for p in "np"]
    kw = dict(epsilon=eps, pmls=pmls, do_poynting=True)
    N = int(numpy.prod(shape))
    n = 24
    src = [(int(numpy.ravel_multi_index((7, 6, 5), shape)) + N, [math.sin(0.4 * t) for t in range(2 * n)])]
    pts = [(1, (7, 6, 5)), (0, (2, 3, 4)), (2, (12, 1, 8))]
    om = numpy.array([0.2, 0.5, 0.9])
    out = {}
    for path in ("plain", "hs", "fused"):
        g = _gpu(**copy.deepcopy(kw))
        g.tune(**opts)
        mon = g.dft_monitor(pts, om)
        g.run(n, point_sources=[(src[0][0], src[0][1][:n])], monitor=mon, path=path)
        g.run(n, point_sources=[(src[0][0], src[0][1][n:])], monitor=mon, path=path)
        assert g.tuning("last_run_path") == {"plain": 1, "hs": 2, "fused": 3}[path]
        out[path] = (mon.series(), mon.spectrum())
    for path in ("hs", "fused"):
        assert numpy.array_equal(out[path][0], out["plain"][0]), path
        assert numpy.array_equal(out[path][1], out["plain"][1]), path
