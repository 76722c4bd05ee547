"""
Run the reference's own rendered kernels where the reference tree is absent (TEST
INFRASTRUCTURE / CPU baseline).

oracle/ref_harness.export_replay() saves, for one constructed reference Simulation, the C
wrapping of each rendered kernel body (update_E/H/S), the argument manifest in the
reference's argument order (opencl_fdtd/simulation.py:175-245, 304-318) and every non-field
argument (CPML tables, dt) under oracle/_ref/replay_<name>/. This module compiles those
sources with gcc and steps them on host arrays, so a machine without the reference tree can
still time the reference's kernels on its CPU cores. oracle/_ref/ is generated, never
committed.
"""
from __future__ import annotations

import ctypes
import json
import os
import subprocess

import numpy

from .ref_harness import REF_OUT, call_kernel


def replay_dir(name: str) -> str:
    return os.path.join(REF_OUT, "replay_" + name)


def available(name: str) -> bool:
    return os.path.isfile(os.path.join(replay_dir(name), "manifest.json"))


def compile_replay(name: str) -> list:
    """Compile every kernel of a replay into a .so beside its source; returns the .so paths."""
    d = replay_dir(name)
    out = []
    with open(os.path.join(d, "manifest.json")) as f:
        manifest = json.load(f)
    for k in manifest["kernels"]:
        c = os.path.join(d, "update_%s.c" % k)
        so = os.path.join(d, "update_%s.so" % k)
        if not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(c):
            tmp = so + ".%d.tmp" % os.getpid()
            subprocess.check_call(["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
                                   "-w", c, "-o", tmp])
            os.replace(tmp, so)
        out.append(so)
    return out


class ReplaySimulation:
    """Fields plus the reference's compiled E/H/S kernels for one exported configuration."""

    def __init__(self, name: str, eps: numpy.ndarray, nthreads: int = 0):
        d = replay_dir(name)
        compile_replay(name)
        with open(os.path.join(d, "manifest.json")) as f:
            self.manifest = json.load(f)
        self.shape = tuple(self.manifest["shape"])
        self.dt = self.manifest["dt"]
        self.N = int(numpy.prod(self.shape))
        self.nthreads = nthreads
        self.fields = {
            "E": numpy.zeros(3 * self.N, numpy.float32),
            "H": numpy.zeros(3 * self.N, numpy.float32),
            "S": numpy.zeros(3 * self.N, numpy.float32),
            "oS": numpy.zeros((3 * self.N, 2), numpy.float32),
            "eps": numpy.ascontiguousarray(eps, dtype=numpy.float32).reshape(-1),
        }
        assert self.fields["eps"].size == 3 * self.N
        self.kernels = {}
        for kname, entries in self.manifest["kernels"].items():
            lib = ctypes.CDLL(os.path.join(d, "update_%s.so" % kname))
            lib.run.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_long]
            lib.run.restype = None
            lib.set_threads.argtypes = [ctypes.c_int]
            decl, vals = [], []
            for e in entries:
                decl.append((e["ctype"], e["ptr"], e["name"]))
                if not e["ptr"]:
                    vals.append(e["value"])
                elif "field" in e:
                    vals.append(self.fields[e["field"]])
                elif "zeros" in e:
                    vals.append(numpy.zeros(e["zeros"], numpy.float32))
                else:
                    vals.append(numpy.load(os.path.join(d, e["npy"])))
            self.kernels[kname] = (lib, decl, vals)
        self.E, self.H, self.S = self.fields["E"], self.fields["H"], self.fields["S"]

    def _run(self, k):
        lib, decl, vals = self.kernels[k]
        call_kernel(lib, decl, vals, self.nthreads)

    def update_E(self, wait_for=None):
        self._run("E")

    def update_H(self, wait_for=None):
        self._run("H")

    def update_S(self, wait_for=None):
        self._run("S")
