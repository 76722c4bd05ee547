"""
Named, seeded synthetic workloads (constructor arguments plus a point source) used by the
benchmark, the smoke check and the tests. No public dataset is involved: every input is
generated here from a seed.

  c1  64x64x64, float32, dx = 1, dt = 0.99/sqrt(3); vacuum with an eps = 12.25 slab for
      z in [24, 40); 8-cell CPML on all six faces with the reference's default grading; soft
      Ez source at (32, 32, 32): sin(2 pi t/16) exp(-((t-60)/20)^2/2); 500 steps; Poynting off.
  c2  395x345x73 (~10M cells, the reference README's benchmark grid), float32, 40 nm cells:
      silicon slab eps = 12.11, 6 cells thick, centred in z, in air; triangular lattice of air
      holes, a = 10 cells, r = 0.3a, centres jittered by seeded N(0, 0.01a); L3 defect (three
      central holes removed); 8-cell CPML on all faces; Ey dipole at the centre, 1550 nm
      Gaussian pulse of 20% bandwidth; 8000 steps; Poynting on.
"""
from __future__ import annotations

import math

import numpy

from . import geometry


def c1(float_type=numpy.float32):
    shape = (64, 64, 64)
    eps = [numpy.ones(shape, float_type) for _ in range(3)]
    for e in eps:
        e[:, :, 24:40] = 12.25
    pmls = [{"axis": a, "polarity": p, "thickness": 8} for a in "xyz" for p in "np"]
    N = 64 ** 3
    index = int(numpy.ravel_multi_index((32, 32, 32), shape)) + 2 * N

    def wave(t):
        return math.sin(2 * math.pi * t / 16) * math.exp(-0.5 * ((t - 60) / 20) ** 2)

    return {"name": "c1", "shape": shape, "steps": 500,
            "kwargs": dict(epsilon=eps, pmls=pmls, do_poynting=False, float_type=float_type),
            "source_index": index, "wave": wave,
            "describe": "64^3 f32, eps=12.25 slab z in [24,40), 8-cell CPML x6, soft Ez source, 500 steps, Poynting off"}


def c2_shape():
    return (395, 345, 73)


def c2_pmls():
    return [{"axis": a, "polarity": p, "thickness": 8} for a in "xyz" for p in "np"]


def c2(float_type=numpy.float32, seed: int = 2, shape=None):
    shape = tuple(shape) if shape is not None else c2_shape()
    eps = geometry.l3_cavity(shape, a=10.0, r_frac=0.3, slab_eps=12.11, slab_thickness=6.0,
                             jitter_frac=0.01, margin=8, defect_length=3, seed=seed, dtype=float_type)
    N = int(numpy.prod(shape))
    center = tuple(s // 2 for s in shape)
    index = int(numpy.ravel_multi_index(center, shape)) + 1 * N
    dt = 0.99 / math.sqrt(3)
    wave = geometry.gaussian_pulse(dt, dx_nm=40.0, wavelength_nm=1550.0, bandwidth_nm=0.2 * 1550.0)
    return {"name": "c2", "shape": shape, "steps": 8000,
            "kwargs": dict(epsilon=eps, pmls=c2_pmls(), do_poynting=True, float_type=float_type),
            "source_index": index, "wave": wave,
            "describe": "%dx%dx%d f32 L3 photonic-crystal slab (a=10, r=0.3a, eps=12.11, 6 cells), "
                        "8-cell CPML x6, Ey Gaussian pulse 1550 nm/20%%, Poynting on" % shape}


def c3(float_type=numpy.float32, seed: int = 3, shape=(128, 128, 256)):
    """Anisotropic + Bloch periodic cell: complex fields as split real/imaginary arrays, Bloch
    phases kx = 0.3 pi / Lx and ky = 0.1 pi / Ly (phase k L across each period), 8-cell CPML
    on the z faces only, diagonal eps in U[1, 12] and mu in U[1, 2] inside 12 seeded spheres
    of radius 8-20 cells (one of them a perfect conductor), vacuum elsewhere, and a soft
    plane-wave source (Ex on the whole z = 20 plane)."""
    shape = tuple(shape)
    eps, mu = geometry.sphere_inclusions(shape, n=12, rmin=8, rmax=20, seed=seed,
                                         pec_index=5, dtype=float_type)
    bloch = [{"axis": "x", "real": math.cos(0.3 * math.pi), "imag": math.sin(0.3 * math.pi)},
             {"axis": "y", "real": math.cos(0.1 * math.pi), "imag": math.sin(0.1 * math.pi)}]
    pmls = [{"axis": "z", "polarity": p, "thickness": 8} for p in "np"]
    dt = 0.99 / math.sqrt(3)

    def wave(t):
        return math.sin(2 * math.pi * t * dt / 20.0) * math.exp(-0.5 * ((t - 80) / 25) ** 2)

    return {"name": "c3", "shape": shape, "steps": 4000,
            "kwargs": dict(epsilon=eps, mu=mu, pmls=pmls, bloch_boundaries=bloch,
                           do_poynting=False, float_type=float_type),
            "source_plane": 20, "wave": wave,
            "describe": "%dx%dx%d complex (split f32), Bloch x/y, CPML z, eps/mu spheres, PEC sphere" % shape}


def c4(n: int = 64, seed: int = 4, steps: int = 2000):
    """The batched sweep: n L3-cavity variants of the c2 construction (silicon slab eps = 12.11,
    6 cells thick, triangular lattice of air holes with an L3 defect, 8-cell CPML on all six
    faces, Ey dipole with the 1550 nm / 20% Gaussian pulse in 40 nm cells, Poynting off) on
    uneven seeded grids: sx ~ U{96..256}, sy ~ U{96..224}, sz ~ U{48..73}, lattice period
    a ~ U[8, 12] cells, hole radius r ~ U[0.25a, 0.35a]. Each variant records E_y at its
    centre every step (the DFT-peak monitor)."""
    rng = numpy.random.default_rng(seed)
    dt = 0.99 / math.sqrt(3)
    wave = geometry.gaussian_pulse(dt, dx_nm=40.0, wavelength_nm=1550.0, bandwidth_nm=0.2 * 1550.0)
    out = []
    for v in range(n):
        shape = (int(rng.integers(96, 257)), int(rng.integers(96, 225)), int(rng.integers(48, 74)))
        a = float(rng.uniform(8.0, 12.0))
        r_frac = float(rng.uniform(0.25, 0.35))
        out.append({"shape": shape, "a": a, "r_frac": r_frac, "seed": int(rng.integers(0, 2 ** 31)),
                    "steps": steps, "wave": wave})
    return out


def c4_kwargs(var, float_type=numpy.float32):
    """Simulation keyword arguments and the centre Ey flat index of one c4 variant."""
    shape = var["shape"]
    eps = geometry.l3_cavity(shape, a=var["a"], r_frac=var["r_frac"], slab_eps=12.11, slab_thickness=6.0,
                             jitter_frac=0.01, margin=8, defect_length=3, seed=var["seed"], dtype=float_type)
    N = int(numpy.prod(shape))
    centre = tuple(s // 2 for s in shape)
    index = int(numpy.ravel_multi_index(centre, shape)) + 1 * N
    kw = dict(epsilon=eps, pmls=c2_pmls(), do_poynting=False, float_type=float_type)
    return kw, index


def face_cells(shape, pmls) -> int:
    """Cells that carry a CPML auxiliary pair, summed over faces (corners count per face)."""
    total = 0
    for p in pmls:
        a = "xyz".index(p["axis"])
        T = int(p.get("thickness", 8))
        other = [shape[r] for r in range(3) if r != a]
        if T <= shape[a]:
            total += T * other[0] * other[1]
        elif p["polarity"] == "n":
            total += shape[a] * other[0] * other[1]
    return total


def get(name: str, **kw):
    return {"c1": c1, "c2": c2, "c3": c3, "c4": c4}[name](**kw)
