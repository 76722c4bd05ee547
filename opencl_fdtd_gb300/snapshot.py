"""
Field snapshots and checkpoints.

save_snapshot writes what opencl_fdtd's example driver saves at the end of a run
(fdtd.py:181-191): a dict {'grid', 'E', 'H'[, 'S']} whose fields are unvec'd to
[f_x, f_y, f_z] arrays of the grid shape, pickled and lzma-compressed. The example script
pickles with dill, which reads plain pickles; 'grid' is whatever the caller passes (the
script's gridlock.Grid) or a dict describing the grid.

save_checkpoint / load_checkpoint keep everything needed to resume a run bit for bit
(fields, CPML auxiliary arrays, step counter; Simulation.state_dict).
"""
from __future__ import annotations

import lzma
import pickle

import numpy
import torch


def unvec(v, shape):
    """Flat [X | Y | Z] array -> array of shape (3, *shape) (fdfd_tools.unvec's layout)."""
    v = numpy.asarray(v)
    return v.reshape((3, *shape), order="C")


def vec(f):
    """[f_x, f_y, f_z] -> flat [X | Y | Z] array."""
    return numpy.concatenate([numpy.asarray(c).ravel(order="C") for c in f])


def snapshot_dict(sim, grid=None) -> dict:
    d = {"grid": grid if grid is not None else {"shape": sim.shape, "dt": sim.dt},
         "E": unvec(sim.get("E"), sim.shape), "H": unvec(sim.get("H"), sim.shape)}
    if sim.S is not None:
        d["S"] = unvec(sim.get("S"), sim.shape)
    if sim.F is not None:
        d["F"] = unvec(sim.get("F"), sim.shape)
        d["G"] = unvec(sim.get("G"), sim.shape)
    return d


def save_snapshot(sim, path, grid=None):
    with lzma.open(path, "wb") as f:
        pickle.dump(snapshot_dict(sim, grid), f)


def load_snapshot(path) -> dict:
    with lzma.open(path, "rb") as f:
        return pickle.load(f)


def save_checkpoint(sim, path):
    st = sim.state_dict()
    cpu = {k: (v.cpu() if isinstance(v, torch.Tensor) else v) for k, v in st.items() if k != "psi"}
    cpu["psi"] = {k: [(u.cpu(), w.cpu()) for u, w in lst] for k, lst in st["psi"].items()}
    cpu["shape"] = sim.shape
    torch.save(cpu, path)


def load_checkpoint(sim, path):
    st = torch.load(path, map_location="cpu", weights_only=False)
    if tuple(st.pop("shape")) != tuple(sim.shape):
        raise ValueError("checkpoint shape does not match the simulation")
    sim.load_state_dict(st)
