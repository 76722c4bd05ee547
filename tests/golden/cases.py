"""
Seeded test cases shared by the golden-fixture generator and the parity tests.

Each case is a constructor-argument set for a Simulation-like class (the reference's own
Simulation run on the CPU, the C restatement in oracle/, or the CUDA drop-in) plus a step
loop in the shape of opencl_fdtd's fdtd.py:162-175. ``run_case`` drives any of the three
through the same public API: update_E/F/H/G/S/J and ``sim.E[ind] += value``.
"""
from __future__ import annotations

import copy

import numpy

F32 = numpy.float32


def pulse_c1(t: int) -> float:
    """Gaussian-modulated sine: period 16 steps, envelope sigma 20 steps, peak at step 60."""
    return float(numpy.sin(2 * numpy.pi * t / 16) * numpy.exp(-0.5 * ((t - 60) / 20) ** 2))


def pulse_short(t: int) -> float:
    return float(numpy.sin(0.7 * t) * numpy.exp(-0.5 * ((t - 12) / 5) ** 2))


ALL6 = ("xn", "xp", "yn", "yp", "zn", "zp")


def build(name: str):
    """Return (ctor_kwargs, loop) for a named case. Arrays are numpy, seeded."""
    rng = numpy.random.default_rng(sum(map(ord, name)) * 7919)
    dtype = F32
    loop = {"steps": 20, "sources": [], "fieldsrc": None}
    kw = {}
    if name == "c1_small":
        shape = (24, 24, 24)
        eps = [numpy.ones(shape, dtype) for _ in range(3)]
        for e in eps:
            e[:, :, 9:15] = 12.25
        kw = dict(epsilon=eps, pmls=[{"axis": f[0], "polarity": f[1], "thickness": 4} for f in ALL6],
                  do_poynting=False)
        loop.update(steps=120, sources=[((12, 12, 12), 2, "c1")])
    elif name == "periodic_pec_poynting":
        shape = (14, 12, 10)
        eps = [rng.uniform(1, 4, shape).astype(dtype) for _ in range(3)]
        eps[0][3:6, 2:5, 4:7] = numpy.inf
        eps[1][3:6, 2:5, 4:7] = numpy.inf
        eps[2][3:6, 2:5, 4:7] = numpy.inf
        init = {k: [rng.standard_normal(shape).astype(dtype) for _ in range(3)] for k in "EH"}
        kw = dict(epsilon=eps, pmls=[], initial_fields=init, do_poynting=True)
        loop.update(steps=30)
    elif name == "pml_mixed":
        shape = (16, 14, 12)
        eps = [rng.uniform(1, 6, shape).astype(dtype) for _ in range(3)]
        pm = [{"axis": "z", "polarity": "p", "thickness": 4, "m": 3, "ln_R_per_layer": -2.0,
               "cfs_alpha": 0.05, "ma": 2, "epsilon_eff": 2.0, "mu_eff": 1.5},
              {"axis": "x", "polarity": "n", "thickness": 3},
              {"axis": "y", "polarity": "p", "thickness": 2, "m": 2}]
        init = {"H": [rng.standard_normal(shape).astype(dtype) for _ in range(3)]}
        kw = dict(epsilon=eps, pmls=pm, initial_fields=init, do_poynting=True)
        loop.update(steps=40, sources=[((8, 7, 6), 0, "short"), ((3, 3, 9), 1, "short")])
    elif name == "nonuniform":
        shape = (12, 10, 9)
        eps = [rng.uniform(1, 3, shape).astype(dtype) for _ in range(3)]
        dxes = [[rng.uniform(0.8, 1.25, n) for n in shape], [rng.uniform(0.8, 1.25, n) for n in shape]]
        kw = dict(epsilon=eps, pmls=[{"axis": f[0], "polarity": f[1], "thickness": 3} for f in ALL6],
                  dxes=dxes, do_poynting=True)
        loop.update(steps=25, sources=[((6, 5, 4), 2, "short")])
    elif name == "dx_half":
        shape = (12, 11, 10)
        eps = [rng.uniform(1, 3, shape).astype(dtype) for _ in range(3)]
        kw = dict(epsilon=eps, pmls=[{"axis": f[0], "polarity": f[1], "thickness": 3} for f in ALL6],
                  dxes=0.5, dt=0.2, do_poynting=True)
        loop.update(steps=25, sources=[((6, 5, 4), 1, "short")])
    elif name == "fieldsrc":
        shape = (12, 10, 9)
        eps = [rng.uniform(1, 3, shape).astype(dtype) for _ in range(3)]
        kw = dict(epsilon=eps, pmls=[{"axis": f[0], "polarity": f[1], "thickness": 3} for f in ALL6],
                  do_poynting=False, do_fieldsrc=True)
        loop.update(steps=20, fieldsrc=((2, 9, 1, 6, 3, 8), rng.standard_normal((2, 3 * numpy.prod(shape))).astype(dtype)))
    elif name == "bloch_trivial":
        shape = (10, 9, 8)
        eps = [rng.uniform(1, 3, shape).astype(dtype) for _ in range(3)]
        init = {k: [rng.standard_normal(shape).astype(dtype) for _ in range(3)] for k in "EHFG"}
        kw = dict(epsilon=eps, pmls=[{"axis": "z", "polarity": p, "thickness": 2} for p in "np"],
                  bloch_boundaries=[{"axis": "x", "real": 1.0, "imag": 0.0},
                                    {"axis": "y", "real": 1.0, "imag": 0.0}],
                  initial_fields=init, do_poynting=False)
        loop.update(steps=20)
    elif name == "thin_overlap":
        shape = (9, 5, 4)
        eps = [rng.uniform(1, 3, shape).astype(dtype) for _ in range(3)]
        init = {k: [rng.standard_normal(shape).astype(dtype) for _ in range(3)] for k in "EH"}
        pm = [{"axis": "y", "polarity": "n", "thickness": 3}, {"axis": "z", "polarity": "n", "thickness": 2},
              {"axis": "y", "polarity": "p", "thickness": 3}, {"axis": "z", "polarity": "p", "thickness": 6},
              {"axis": "x", "polarity": "p", "thickness": 2}]
        kw = dict(epsilon=eps, pmls=pm, initial_fields=init, do_poynting=True)
        loop.update(steps=15)
    elif name == "f64_mixed":
        kw, loop = build("pml_mixed")
        kw["epsilon"] = [e.astype(numpy.float64) for e in kw["epsilon"]]
        kw["initial_fields"] = {k: [a.astype(numpy.float64) for a in v] for k, v in kw["initial_fields"].items()}
        kw["float_type"] = numpy.float64
        return kw, loop
    else:
        raise KeyError(name)
    return kw, loop


CASE_NAMES = ("c1_small", "periodic_pec_poynting", "pml_mixed", "nonuniform", "dx_half",
              "fieldsrc", "bloch_trivial", "thin_overlap", "f64_mixed")

_WAVES = {"c1": pulse_c1, "short": pulse_short}


def to_numpy(a):
    if hasattr(a, "detach"):
        return a.detach().cpu().numpy().reshape(-1)
    return numpy.array(a).reshape(-1)


def run_case(sim_cls, name: str, steps: int | None = None, **extra):
    """Construct ``sim_cls`` with the case's arguments and run its loop; returns the sim."""
    kw, loop = build(name)
    kw = copy.deepcopy(kw)
    kw.update(extra)
    sim = sim_cls(**kw)
    shape = tuple(kw["epsilon"][0].shape)
    N = int(numpy.prod(shape))
    src = [(int(numpy.ravel_multi_index(p, shape)) + c * N, _WAVES[w]) for p, c, w in loop["sources"]]
    n = loop["steps"] if steps is None else steps
    bloch = bool(kw.get("bloch_boundaries"))
    for t in range(n):
        sim.update_E([])
        if bloch:
            sim.update_F([])
        for ind, wave in src:
            sim.E[ind] += wave(t)
        if loop["fieldsrc"] is not None:
            box, J = loop["fieldsrc"]
            if t == 0:
                _set(sim.Jr, J[0])
                _set(sim.Ji, J[1])
            sim.update_J([], float(numpy.cos(0.3 * t)), float(numpy.sin(0.3 * t)), *box)
        sim.update_H([])
        if bloch:
            sim.update_G([])
        if kw.get("do_poynting", True):
            sim.update_S([])
    return sim


def _set(dst, src):
    if hasattr(dst, "copy_"):
        import torch
        dst.copy_(torch.from_numpy(numpy.ascontiguousarray(src)).to(dst.device))
    else:
        dst[:] = src


def outputs(sim, name: str) -> dict:
    kw, _ = build(name)
    out = {"E": to_numpy(sim.E), "H": to_numpy(sim.H)}
    if kw.get("do_poynting", True):
        out["S"] = to_numpy(sim.S)
    if kw.get("bloch_boundaries"):
        out["F"] = to_numpy(sim.F)
        out["G"] = to_numpy(sim.G)
    return out
