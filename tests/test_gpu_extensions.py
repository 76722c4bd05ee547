"""GPU parity for what the reference lacks: diagonal anisotropic mu and Bloch-phase coupling of
split complex fields (both checked against the oracle's restatement, bit for bit in float32 and
float64), a Bloch-theorem check that needs no oracle, and the dt/eps cache refresh."""
import copy
import math
import os

import numpy
import pytest

torch = pytest.importorskip("torch")

from oracle import port  # noqa: E402
from opencl_fdtd_gb300 import geometry  # noqa: E402

pytestmark = pytest.mark.gpu


def _gpu(**kw):
    from opencl_fdtd_gb300 import Simulation
    return Simulation(**kw)


def _port(**kw):
    return port.PortSimulation(nthreads=os.cpu_count(), **kw)


def _np(a):
    return a.detach().cpu().numpy().reshape(-1) if hasattr(a, "detach") else numpy.asarray(a).reshape(-1)


def _loop(sim, steps, src, bloch, poynting):
    for t in range(steps):
        sim.update_E([])
        if bloch:
            sim.update_F([])
        for ind, w in src:
            sim.E[ind] += w(t)
        sim.update_H([])
        if bloch:
            sim.update_G([])
        if poynting:
            sim.update_S([])


def _compare(kw, steps, src=(), fields=("E", "H")):
    a = _gpu(**copy.deepcopy(kw))
    b = _port(**copy.deepcopy(kw))
    bloch = bool(kw.get("bloch_boundaries"))
    poy = kw.get("do_poynting", True)
    _loop(a, steps, src, bloch, poy)
    _loop(b, steps, src, bloch, poy)
    for k in fields + (("S",) if poy else ()):
        ga, gb = _np(getattr(a, k)), _np(getattr(b, k))
        bad = numpy.flatnonzero(ga != gb)
        assert bad.size == 0, (k, bad[:5], ga[bad[:5]], gb[bad[:5]])
    return a, b


@pytest.mark.parametrize("dtype", [numpy.float32, numpy.float64])
def test_anisotropic_mu_and_pec(dtype):
    shape = (20, 18, 24)
    eps, mu = geometry.sphere_inclusions(shape, n=4, rmin=3, rmax=6, seed=11, pec_index=1, dtype=dtype)
    pmls = [{"axis": "z", "polarity": p, "thickness": 5} for p in "np"]
    N = int(numpy.prod(shape))
    src = [(int(numpy.ravel_multi_index((10, 9, 12), shape)) + 2 * N,
            lambda t: math.sin(0.5 * t) * math.exp(-0.5 * ((t - 15) / 6) ** 2))]
    kw = dict(epsilon=eps, mu=mu, pmls=pmls, do_poynting=True, float_type=dtype)
    a, _ = _compare(kw, 40, src)
    assert float(torch.abs(a.E).max()) > 0


@pytest.mark.parametrize("dtype", [numpy.float32, numpy.float64])
def test_bloch_phase_coupling(dtype):
    shape = (14, 12, 20)
    rng = numpy.random.default_rng(5)
    eps, mu = geometry.sphere_inclusions(shape, n=3, rmin=2, rmax=4, seed=3, dtype=dtype)
    init = {k: [rng.standard_normal(shape).astype(dtype) for _ in range(3)] for k in "EHFG"}
    bloch = [{"axis": "x", "real": math.cos(0.3 * math.pi), "imag": math.sin(0.3 * math.pi)},
             {"axis": "y", "real": math.cos(0.1 * math.pi), "imag": math.sin(0.1 * math.pi)}]
    pmls = [{"axis": "z", "polarity": p, "thickness": 4} for p in "np"]
    kw = dict(epsilon=eps, mu=mu, pmls=pmls, bloch_boundaries=bloch, initial_fields=init,
              do_poynting=True, float_type=dtype)
    _compare(kw, 30, fields=("E", "H", "F", "G"))


def test_bloch_plane_wave_keeps_its_phase_law():
    """Bloch's theorem: a field started as exp(i k x) with beta = exp(i k L) stays a(t) exp(i k x)
    on the E grid (and exp(i k (x + 1/2)) on the staggered H grid) at every step."""
    sx, sy, sz = 40, 3, 3
    k = 0.3 * math.pi / sx
    beta = complex(math.cos(k * sx), math.sin(k * sx))
    x = numpy.arange(sx)[:, None, None] * numpy.ones((1, sy, sz))
    zero = numpy.zeros((sx, sy, sz), numpy.float64)
    init = {"E": [zero, numpy.cos(k * x), zero], "F": [zero, numpy.sin(k * x), zero],
            "H": [zero] * 3, "G": [zero] * 3}
    eps = [numpy.ones((sx, sy, sz), numpy.float64)] * 3
    sim = _gpu(epsilon=eps, pmls=[], initial_fields=init, float_type=numpy.float64, do_poynting=False,
               bloch_boundaries=[{"axis": "x", "real": beta.real, "imag": beta.imag}])
    for _ in range(200):
        sim.update_E([]); sim.update_F([]); sim.update_H([]); sim.update_G([])
    N = sx * sy * sz
    ey = (_np(sim.E)[N:2 * N] + 1j * _np(sim.F)[N:2 * N]).reshape(sx, sy, sz)[:, 1, 1]
    hz = (_np(sim.H)[2 * N:] + 1j * _np(sim.G)[2 * N:]).reshape(sx, sy, sz)[:, 1, 1]
    a_e = ey / numpy.exp(1j * k * numpy.arange(sx))
    a_h = hz / numpy.exp(1j * k * (numpy.arange(sx) + 0.5))
    assert abs(a_e[0]) > 0.1 and abs(a_h[0]) > 1e-3
    assert numpy.abs(a_e - a_e[0]).max() < 1e-9 * max(1.0, abs(a_e[0]))
    assert numpy.abs(a_h - a_h[0]).max() < 1e-9 * max(1.0, abs(a_h[0]))


def test_eps_change_refreshes_cached_quotient():
    shape = (16, 12, 10)
    rng = numpy.random.default_rng(9)
    eps = [rng.uniform(1, 3, shape).astype(numpy.float32) for _ in range(3)]
    init = {k: [rng.standard_normal(shape).astype(numpy.float32) for _ in range(3)] for k in "EH"}
    pm = [{"axis": "x", "polarity": "n", "thickness": 3}]
    kw = dict(epsilon=eps, pmls=pm, initial_fields=init, do_poynting=False)
    a, b = _gpu(**copy.deepcopy(kw)), _port(**copy.deepcopy(kw))
    _loop(a, 5, (), False, False)
    _loop(b, 5, (), False, False)
    a.eps.mul_(2.0)
    b.eps *= numpy.float32(2.0)
    _loop(a, 5, (), False, False)
    _loop(b, 5, (), False, False)
    assert numpy.array_equal(_np(a.E), b.E) and numpy.array_equal(_np(a.H), b.H)


def test_interior_and_shell_cover_every_cell_once():
    """A grid whose interior is a single cell line, odd sizes and one-sided CPML."""
    for shape, pm in (((3, 3, 3), []), ((5, 4, 7), [{"axis": "y", "polarity": "p", "thickness": 1}]),
                      ((11, 3, 33), [{"axis": "z", "polarity": "n", "thickness": 9},
                                     {"axis": "x", "polarity": "p", "thickness": 2}])):
        rng = numpy.random.default_rng(sum(shape))
        eps = [rng.uniform(1, 3, shape).astype(numpy.float32) for _ in range(3)]
        init = {k: [rng.standard_normal(shape).astype(numpy.float32) for _ in range(3)] for k in "EH"}
        _compare(dict(epsilon=eps, pmls=pm, initial_fields=init, do_poynting=True), 6)
