"""
Seeded synthetic geometry for the benchmark and test workloads.

The reference builds its ringdown cavity with external packages (gridlock, masque; opencl_fdtd
fdtd.py:103-125) that are not available here; this module stands in for them with a direct
rasteriser onto the three Yee-staggered permittivity grids:

  * ``triangular_lattice`` / ``ln_defect`` give the same hole sets as the reference's
    pcgen.py:11-48 and 93-108 (rows of a triangular lattice centred on the origin, odd rows
    shifted by half a period and one hole shorter; an Ln defect removes the n central holes
    of the middle row), written here from that description;
  * ``l3_cavity`` draws a slab of permittivity ``slab_eps`` and air holes through it;
  * ``gaussian_pulse`` is the source of fdtd.py:135-143 (a sine at the centre wavelength under
    a Gaussian envelope whose width follows the given bandwidth), in grid units.

Yee positions (cell units, origin at the grid centre): E_x at (x+1/2, y, z), E_y at
(x, y+1/2, z), E_z at (x, y, z+1/2). Everything is float64 until the final cast.
"""
from __future__ import annotations

import math

import numpy


def triangular_lattice(dims) -> numpy.ndarray:
    """(K, 2) lattice sites in units of the period: dims[0] rows of dims[0] sites (odd rows
    one fewer and shifted by 1/2), rows sqrt(3)/2 apart, centred, sorted by x."""
    nx = int(dims[0])
    half = (int(dims[1]) - 1) / 2
    sites = []
    for row in numpy.linspace(-half, half, nx):
        odd = math.floor(row) % 2
        xmax = (nx - 1) / 2
        xs = numpy.linspace(-xmax, xmax - odd, int(nx - odd)) + 0.5 * odd
        sites.append(numpy.stack([xs, numpy.full_like(xs, row * math.sqrt(3) / 2)], axis=1))
    xy = numpy.concatenate(sites, axis=0)
    return xy[numpy.argsort(xy[:, 0], kind="quicksort")]


def ln_defect(mirror_dims, defect_length: int) -> numpy.ndarray:
    """Triangular lattice of (2n+1) x (2m+1) sites with ``defect_length`` (odd) central holes
    of the middle row removed."""
    if defect_length % 2 != 1:
        raise ValueError("defect_length must be odd")
    xy = triangular_lattice([2 * d + 1 for d in mirror_dims])
    h = defect_length // 2
    in_defect = (xy[:, 1] == 0) & numpy.isin(xy[:, 0], numpy.arange(-h, h + 1))
    return xy[~in_defect]


def _hole_mask(n0: int, n1: int, off0: float, off1: float, holes: numpy.ndarray, radius: float):
    """Boolean (n0, n1) mask of points (i + off0 - c0, j + off1 - c1) inside any hole."""
    mask = numpy.zeros((n0, n1), dtype=bool)
    c0, c1 = n0 / 2.0, n1 / 2.0
    r2 = radius * radius
    for hx, hy in holes:
        px, py = hx + c0 - off0, hy + c1 - off1
        i0, i1 = max(int(math.floor(px - radius)), 0), min(int(math.ceil(px + radius)) + 1, n0)
        j0, j1 = max(int(math.floor(py - radius)), 0), min(int(math.ceil(py + radius)) + 1, n1)
        if i0 >= i1 or j0 >= j1:
            continue
        ii = numpy.arange(i0, i1)[:, None] - px
        jj = numpy.arange(j0, j1)[None, :] - py
        mask[i0:i1, j0:j1] |= (ii * ii + jj * jj) < r2
    return mask


def l3_cavity(shape, a: float = 10.0, r_frac: float = 0.3, slab_eps: float = 12.11,
              slab_thickness: float = 6.0, jitter_frac: float = 0.01, margin: int = 8,
              defect_length: int = 3, seed: int = 0, dtype=numpy.float32):
    """[eps_xx, eps_yy, eps_zz] of a photonic-crystal Ln cavity in a slab.

    The lattice (period ``a`` cells, hole radius ``r_frac * a``) fills the x-y extent left
    after ``margin`` + one period on each side; hole centres get seeded N(0, jitter*a)
    jitter. The slab is ``slab_thickness`` cells thick, centred in z, in air (eps = 1)."""
    sx, sy, sz = (int(s) for s in shape)
    rng = numpy.random.default_rng(seed)
    nx = max(int((sx - 2 * margin - 2 * a) // (2 * a)), 1)
    ny = max(int((sy - 2 * margin - 2 * a) // (a * math.sqrt(3))), 1)
    n = min(nx, ny)
    holes = ln_defect((n, n), defect_length) * a
    holes = holes + rng.normal(0.0, jitter_frac * a, holes.shape)
    radius = r_frac * a
    zc = sz / 2.0
    out = []
    for comp, (ox, oy, oz) in enumerate(((0.5, 0.0, 0.0), (0.0, 0.5, 0.0), (0.0, 0.0, 0.5))):
        mask = _hole_mask(sx, sy, ox, oy, holes, radius)
        zpos = numpy.arange(sz) + oz
        in_slab = numpy.abs(zpos - zc) < slab_thickness / 2.0
        eps = numpy.ones((sx, sy, sz), dtype=dtype)
        plane = numpy.where(mask, 1.0, slab_eps).astype(dtype)
        eps[:, :, in_slab] = plane[:, :, None]
        out.append(eps)
    return out


def gaussian_pulse(dt: float, dx_nm: float, wavelength_nm: float, bandwidth_nm: float):
    """Source waveform in the form of fdtd.py:135-143, in grid units (c = 1, cell = 1):
    angular frequency w = 2 pi dx / wl, envelope exp(-alpha t'^2) with alpha set by the
    bandwidth, delayed by 7 / sqrt(2 alpha). Returns f(step) -> float."""
    w = 2 * math.pi * dx_nm / wavelength_nm
    fwhm = bandwidth_nm * w * w / (2 * math.pi * dx_nm)
    alpha = (fwhm ** 2) / 8 * math.log(2)
    delay = 7 / math.sqrt(2 * alpha)

    def f(step: int) -> float:
        t0 = step * dt - delay
        return math.sin(w * t0) * math.exp(-alpha * t0 * t0)

    return f


def sphere_inclusions(shape, n: int, rmin: float, rmax: float, seed: int,
                      lo=(1.0, 1.0), hi=(12.0, 2.0), pec_index: int | None = None, dtype=numpy.float32):
    """Diagonal anisotropic eps and mu: vacuum with ``n`` seeded spheres whose eps_xx/yy/zz are
    drawn from U[lo[0], hi[0]] and mu_xx/yy/zz from U[lo[1], hi[1]]; sphere ``pec_index`` (if
    given) is a perfect conductor (eps = inf)."""
    sx, sy, sz = (int(s) for s in shape)
    rng = numpy.random.default_rng(seed)
    eps = [numpy.ones(shape, dtype) for _ in range(3)]
    mu = [numpy.ones(shape, dtype) for _ in range(3)]
    X, Y, Z = numpy.meshgrid(numpy.arange(sx), numpy.arange(sy), numpy.arange(sz), indexing="ij")
    for k in range(n):
        c = rng.uniform([0, 0, 0], [sx, sy, sz])
        r = rng.uniform(rmin, rmax)
        ev = rng.uniform(lo[0], hi[0], 3)
        mv = rng.uniform(lo[1], hi[1], 3)
        inside = (X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2 < r * r
        for q in range(3):
            eps[q][inside] = numpy.inf if k == pec_index else ev[q]
            mu[q][inside] = mv[q]
    return eps, mu
