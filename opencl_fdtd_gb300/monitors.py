"""
FP64 monitors on a running Simulation.

DftMonitor accumulates, on the GPU and in double precision, the discrete Fourier transform
of E at a few points (the ringdown monitors of opencl_fdtd's fdtd.py driver, which itself
only saved the final fields) and can record their time series for a frequency / Q fit.
"""
from __future__ import annotations

import ctypes

import numpy
import torch

from . import _lib


class DftMonitor:
    """E at ``points`` sampled after every step, transformed at angular frequencies ``omegas``.

    points: flat indices into the 3N E array, or (component, (x, y, z)) tuples.
    omegas: angular frequencies in radians per unit time (the grid's units, c = 1).
    record: also keep the time series (grown as needed).
    t0: step index of the first sample; sample k is taken at time (t0 + k + 1) * dt.
    """

    def __init__(self, sim, points, omegas=(), record: bool = True, t0: int = 0):
        self.sim = sim
        idx = []
        for p in points:
            if isinstance(p, (tuple, list)):
                comp, xyz = p
                idx.append(int(numpy.ravel_multi_index(tuple(xyz), sim.shape)) + int(comp) * sim.N)
            else:
                idx.append(int(p))
        idx = numpy.asarray(idx, dtype=numpy.int64)
        if idx.size == 0 or (idx < 0).any() or (idx >= 3 * sim.N).any():
            raise IndexError("monitor points must be inside the 3N E array")
        om = numpy.asarray(omegas, dtype=numpy.float64).ravel()
        if om.size == 0 and not record:
            raise ValueError("a monitor needs frequencies or a recorded series")
        dev = sim.device
        # Every buffer the kernels touch is made (and zeroed) on the simulation's queue, the
        # stream its kernels run on, so the first run is ordered after the zeroing whatever
        # torch's current stream is.
        with torch.cuda.stream(sim.queue):
            self.index = torch.from_numpy(idx).to(dev)
            self.omega = torch.from_numpy(om).to(dev) if om.size else torch.zeros(1, dtype=torch.float64, device=dev)
            self.accum = torch.zeros((idx.size, max(om.size, 1), 2), dtype=torch.float64, device=dev)
            self._series = torch.zeros((0, idx.size), dtype=torch.float64, device=dev)
        self.record = record
        self.n_freq = int(om.size)
        self.samples = 0
        self.t0 = int(t0)
        self._c = _lib.FdtdDftMonitor()

    def _ensure(self, more: int):
        if not self.record:
            return
        need = self.samples + more
        if need > self._series.shape[0]:
            # Grow on the queue: the copy then follows the queued kernels that write the old
            # rows, and the caching allocator does not hand the old buffer to another stream
            # while those kernels may still write it.
            cap = max(need, 2 * self._series.shape[0], 1024)
            with torch.cuda.stream(self.sim.queue):
                grown = torch.zeros((cap, self._series.shape[1]), dtype=torch.float64, device=self.sim.device)
                if self.samples:
                    grown[:self.samples] = self._series[:self.samples]
            self._series = grown

    def struct(self, more: int) -> _lib.FdtdDftMonitor:
        """C description for the next ``more`` samples (the series grows first)."""
        self._ensure(more)
        c = self._c
        c.n_points = int(self.index.numel())
        c.n_freq = self.n_freq
        c.index = self.index.data_ptr()
        c.omega = self.omega.data_ptr()
        c.accum = self.accum.data_ptr()
        c.series = self._series.data_ptr() if self.record else None
        c.step = self.t0 + self.samples
        c.series_row = self.samples
        return c

    def sample(self):
        """Take one sample now (for per-call update loops)."""
        sim = self.sim
        c = self.struct(1)
        _lib.check(sim._lib.fdtd_monitor_sample(sim._plan, ctypes.byref(sim._buffers()),
                                                ctypes.c_void_p(sim.queue.cuda_stream), ctypes.byref(c)))
        self.samples += 1

    def spectrum(self) -> numpy.ndarray:
        """(n_points, n_freq) complex128: sum_k x_k exp(-i w (t0 + k + 1) dt)."""
        self.sim.queue.synchronize()
        a = self.accum.cpu().numpy()[:, :self.n_freq]
        return a[..., 0] + 1j * a[..., 1]

    def series(self) -> numpy.ndarray:
        """(samples, n_points) float64 time series."""
        self.sim.queue.synchronize()
        return self._series[:self.samples].cpu().numpy()
