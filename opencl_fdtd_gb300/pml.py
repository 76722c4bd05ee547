"""
CPML face defaults and coefficient tables (host side, computed once per Simulation).

Follows opencl_fdtd/simulation.py:161-168 (defaults) and 274-307 (grading and coefficients).
The reference was written for numpy 1.x value-based casting: its depth arrays have the field
dtype and the float64 scalars it combines with them (dt, kappa_max) do not promote them, so
every table is computed in the field dtype. Under numpy 2 the same expressions would promote
to float64; here each scalar is cast to the field dtype explicitly so the tables keep the
float32 arithmetic of the reference.
"""
from __future__ import annotations

import numpy

# simulation.py:161-168, in the reference's setdefault order
PML_DEFAULTS = (("thickness", 8), ("epsilon_eff", 1.0), ("mu_eff", 1.0),
                ("ln_R_per_layer", -1.6), ("m", 3.5), ("cfs_alpha", 0), ("ma", 1))


def apply_defaults(pml: dict) -> dict:
    """Fill the defaults into the caller's dict in place, as the reference does."""
    for key, val in PML_DEFAULTS:
        pml.setdefault(key, val)
    return pml


def _py(v):
    return v.item() if isinstance(v, numpy.generic) else v


def grading(pml: dict, dt, dtype):
    """Return ((p0e, p1e, p2e), (p0h, p1h, p2h)) for one face, each of length thickness,
    indexed by the depth from the outer face (simulation.py:284-307).

    sigma(x) = (x/T)^m * sigma_max,  sigma_max = -ln_R_per_layer/2 * (m + 1)
    kappa(x) = 1 + (x/T)^m * (kappa_max - 1),  kappa_max = sqrt(mu_eff * epsilon_eff)
    alpha(x) = (1 - x/T)^ma * cfs_alpha
    p0 = exp(-(sigma/kappa + alpha) dt),  p1 = sigma/(sigma + kappa*alpha) * (p0 - 1),
    p2 = 1/kappa.
    The E tables sit half a cell further out than the H tables on the 'p' side and half a
    cell further in on the 'n' side (simulation.py:298-302).
    """
    dtype = numpy.dtype(dtype)
    cast = dtype.type
    T = int(pml["thickness"])
    m = pml["m"]
    sigma_max = cast(-pml["ln_R_per_layer"] / 2 * (m + 1))
    kappa_m1 = cast(float(numpy.sqrt(pml["mu_eff"] * pml["epsilon_eff"])) - 1)
    alpha_max = cast(pml["cfs_alpha"])
    one = cast(1)

    # exponents stay Python scalars, as in the reference, so numpy picks the same power
    # loop (including its fast paths for exponents such as 1 and 2)
    m_exp = _py(m)
    ma_exp = _py(pml["ma"])

    def coefficients(depth):
        frac = depth / cast(T)
        scaling = frac ** m_exp
        sigma = scaling * sigma_max
        kappa = one + scaling * kappa_m1
        alpha = ((one - frac) ** ma_exp) * alpha_max
        p0 = numpy.exp(-(sigma / kappa + alpha) * cast(dt))
        p1 = sigma / (sigma + kappa * alpha) * (p0 - one)
        p2 = one / kappa
        return tuple(numpy.ascontiguousarray(a, dtype=dtype) for a in (p0, p1, p2))

    depth_e = numpy.arange(1, T + 1, dtype=dtype)[::-1].copy()
    depth_h = depth_e.copy()
    if pml["polarity"] == "p":
        depth_e -= cast(0.5)
    elif pml["polarity"] == "n":
        depth_h -= cast(0.5)
    return coefficients(depth_e), coefficients(depth_h)


def psi_shape(shape, axis: int, thickness: int):
    """Shape of one CPML auxiliary array: the grid with the face axis replaced by T."""
    s = list(shape)
    s[axis] = thickness
    return tuple(s)
