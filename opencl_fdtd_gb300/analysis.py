"""
Ringdown analysis in float64: frequencies, decay rates and quality factors of the modes in a
sampled signal, by the matrix-pencil method (Y. Hua and T. K. Sarkar, "Matrix pencil method
for estimating parameters of exponentially damped/undamped sinusoids in noise", IEEE Trans.
ASSP 38(5), 1990). A signal x_k = sum_m a_m z_m^k with z_m = exp((-gamma_m + i omega_m) dt)
gives a Hankel matrix of rank M; the z_m are the eigenvalues of the pencil formed by the
two shifted halves of its leading right singular vectors.
"""
from __future__ import annotations

import numpy


def matrix_pencil(x, dt: float, n_modes: int, pencil: int | None = None):
    """Fit ``n_modes`` damped exponentials to samples ``x`` (real or complex) taken every dt.

    Returns a list of dicts (omega, gamma, Q, amplitude) sorted by amplitude, with omega the
    angular frequency (rad per unit time, folded to >= 0 for real signals), gamma the
    amplitude decay rate and Q = omega / (2 gamma) (inf for an undamped mode)."""
    x = numpy.asarray(x, dtype=numpy.complex128).ravel()
    n = x.size
    L = pencil if pencil is not None else n // 3
    L = max(n_modes, min(L, n - n_modes - 1))
    Y = numpy.lib.stride_tricks.sliding_window_view(x, L + 1)          # (n - L) x (L + 1)
    _, s, vh = numpy.linalg.svd(Y, full_matrices=False)
    M = min(n_modes, s.size)
    V = vh[:M].conj().T                                               # (L + 1) x M
    V1, V2 = V[:-1], V[1:]
    z = numpy.linalg.eigvals(numpy.linalg.pinv(V1) @ V2)
    # amplitudes by least squares on the Vandermonde system
    Z = z[None, :] ** numpy.arange(n)[:, None]
    amp, *_ = numpy.linalg.lstsq(Z, x, rcond=None)
    out = []
    for zi, ai in zip(z, amp):
        lz = numpy.log(zi)
        om = lz.imag / dt
        ga = -lz.real / dt
        out.append({"omega": abs(om), "gamma": ga, "Q": (abs(om) / (2 * ga)) if ga > 0 else numpy.inf,
                    "amplitude": abs(ai), "z": zi})
    out.sort(key=lambda d: -d["amplitude"])
    return out


def dominant_mode(x, dt: float, n_modes: int = 4, band=None):
    """The strongest fitted mode, optionally restricted to omega in band = (lo, hi)."""
    modes = matrix_pencil(x, dt, n_modes)
    if band is not None:
        modes = [m for m in modes if band[0] <= m["omega"] <= band[1]]
    if not modes:
        raise ValueError("no mode in the requested band")
    return modes[0]
