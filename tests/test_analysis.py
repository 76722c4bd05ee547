"""Matrix-pencil ringdown fit on synthetic damped sinusoids with known parameters."""
import numpy
import pytest

from opencl_fdtd_gb300.analysis import dominant_mode, matrix_pencil


@pytest.mark.parametrize("Q", [50.0, 1e3, 1e5])
def test_recovers_frequency_and_q(Q):
    dt = 0.57
    w = 2 * numpy.pi / 38.75 * 1.0          # a 1550 nm line on a 40 nm grid (c = 1)
    g = w / (2 * Q)
    t = numpy.arange(3000) * dt
    x = 1.3 * numpy.exp(-g * t) * numpy.cos(w * t + 0.4) + 0.2 * numpy.exp(-3 * g * t) * numpy.cos(1.7 * w * t)
    m = dominant_mode(x, dt, n_modes=4, band=(0.5 * w, 1.5 * w))
    assert abs(m["omega"] - w) / w < 1e-9
    assert abs(m["Q"] - Q) / Q < 1e-6


def test_undamped_mode_has_infinite_q():
    dt, w = 0.5, 0.31
    x = numpy.cos(w * dt * numpy.arange(500))
    m = matrix_pencil(x, dt, 2)[0]
    assert abs(m["omega"] - w) < 1e-10 and (m["Q"] > 1e9 or numpy.isinf(m["Q"]))
