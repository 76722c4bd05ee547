"""Known-answer physics on the GPU: the 8-cell CPML absorbs. A dipole pulse in a 40^3 grid
with an 8-cell CPML on every face against the same pulse in an 80^3 grid (the small grid
centred, the same CPML at its far faces): over the 4-cell shell just inside the small grid's
CPML, the difference (the wave the CPML sends back) stays below -25 dB of the wave that
reached the shell, before the large grid's own boundary echo can return."""
import math

import numpy
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def _run(shape, pad, steps, T=8, period=20.0):
    from opencl_fdtd_gb300 import Simulation
    dt = 0.99 / math.sqrt(3)
    sim = Simulation(epsilon=[numpy.ones(shape, numpy.float32)] * 3,
                     pmls=[{"axis": a, "polarity": p, "thickness": T} for a in "xyz" for p in "np"],
                     dt=dt, do_poynting=False)
    c = tuple(s // 2 for s in shape)
    ind = int(numpy.ravel_multi_index(c, shape)) + sim.N          # Ey dipole at the centre
    wave = [math.sin(2 * math.pi * t / period) * math.exp(-0.5 * ((t - 4 * period) / period) ** 2)
            for t in range(steps)]
    frames = []
    for t0 in range(0, steps, 5):
        sim.run(5, point_sources=[(ind, wave[t0:t0 + 5])])
        E = sim.E.view(3, *shape)
        frames.append(E[:, pad:pad + 40, pad:pad + 40, pad:pad + 40].double().clone())
    return frames


def test_cpml_reflection_is_small():
    small = _run((40, 40, 40), 0, 140)
    big = _run((80, 80, 80), 20, 140)
    shell = torch.zeros((40, 40, 40), dtype=torch.bool, device="cuda")
    shell[8:32, 8:32, 8:32] = True
    shell[12:28, 12:28, 12:28] = False
    err = max(float(torch.linalg.vector_norm((a - b)[:, shell])) for a, b in zip(small, big))
    ref = max(float(torch.linalg.vector_norm(b[:, shell])) for b in big)
    db = 20 * math.log10(err / ref)
    assert db < -25.0, db
