"""Many independent cavity variants stepped together in one persistent launch.

``BatchSimulation`` takes ordinary ``Simulation`` objects (float32, diagonal eps, no mu, no
Bloch boundaries, Poynting off, uniform dx) and advances all of them with one cooperative
kernel launch per call of ``run`` (``fdtd_batch_run``): the grid of a few blocks per SM works
through the tiles of every variant for the E half-step, synchronises, does the H half-step,
and repeats. There is no per-variant launch, no per-variant tail and no host round trip; a
call can also be captured once in a CUDA graph and replayed (``capture``), since the step
counter lives on the device.

Storage: ``'f32'`` updates the simulations' own tensors in place (results are bit-identical
to ``Simulation.run`` of each variant). ``'bf16'`` / ``'fp16'`` keep E, H and dt/eps in 16-bit
copies owned here, with a power-of-two exponent per run of 32 cells of one component in one
x plane (arithmetic stays float32, CPML psi float32); ``'bf16u'`` keeps bfloat16 copies
without the exponents (bfloat16 has float32's exponent range, so the exponents change no
rounding there short of subnormals, and the codec's warp reductions go); ``sync()`` decodes
the copies back into the simulations' E and H. Point sources and monitor points are given per variant when the batch
is built: sources as the flat index into E and one value per step, monitors as flat indices
whose E values are recorded after every step's sources (float64 series).
"""
from __future__ import annotations

import ctypes

import numpy

from . import _lib

_STORE = {"f32": _lib.FDTD_STORE_F32, "bf16": _lib.FDTD_STORE_BF16, "fp16": _lib.FDTD_STORE_F16,
          "bf16u": _lib.FDTD_STORE_BF16U}


class BatchSimulation:
    def __init__(self, sims, storage: str = "f32", sources=None, monitors=None, steps: int = 0):
        """sims: list of Simulation; sources[v]: list of (flat_index, values) with at least
        ``steps`` values each; monitors[v]: list of flat indices into E; steps: rows of the
        source and monitor arrays (steps past it add no source and record nothing)."""
        import torch
        if storage not in _STORE:
            raise ValueError("storage must be 'f32', 'bf16', 'fp16' or 'bf16u'")
        if not sims:
            raise ValueError("no simulations")
        self.sims = list(sims)
        self.storage = storage
        self.steps = int(steps)
        self.steps_run = 0
        dev = self.sims[0].device
        self.device = dev
        self.queue = self.sims[0].queue
        self._lib = _lib.load()
        self._keep = []
        n = len(self.sims)
        sources = sources if sources is not None else [[] for _ in range(n)]
        monitors = monitors if monitors is not None else [[] for _ in range(n)]
        if len(sources) != n or len(monitors) != n:
            raise ValueError("sources and monitors need one entry per simulation")
        self.series = []
        self._e16, self._h16, self._eexp, self._hexp = [], [], [], []
        arr = (_lib.FdtdBatchVariant * n)()
        half = {"bf16": torch.bfloat16, "fp16": torch.float16, "bf16u": torch.bfloat16}.get(storage)
        scaled = storage in ("bf16", "fp16")
        for v, sim in enumerate(self.sims):
            if sim._np_dtype != numpy.float32:
                raise ValueError("batched stepping needs float32 simulations")
            if sim.bloch_boundaries or sim.mu is not None or sim.do_poynting or sim.inv_dxes is not None:
                raise ValueError("batched stepping supports diagonal eps, CPML, uniform dx, Poynting off")
            if sim.device != dev:
                raise ValueError("all simulations must be on one device")
            b = sim._buffers()            # refreshes dt/eps
            d = arr[v]
            d.shape[0], d.shape[1], d.shape[2] = sim.shape
            d.dt = float(sim.dt)
            d.dx = float(sim._uniform_dx)
            d.n_pml = len(sim._pml_tables)
            for f, (a, pol, T, te, th) in enumerate(sim._pml_tables):
                pf = d.pml[f]
                pf.axis, pf.polarity, pf.thickness = a, pol, T
                tabs = [torch.from_numpy(numpy.ascontiguousarray(t, dtype=numpy.float32)).to(dev) for t in (*te, *th)]
                self._keep += tabs
                for c in range(3):
                    pf.tab_e[c] = tabs[c].data_ptr()
                    pf.tab_h[c] = tabs[3 + c].data_ptr()
                (eu, ev), (hu, hv) = sim.psi["E"][f], sim.psi["H"][f]
                pf.psi_e[0], pf.psi_e[1] = eu.data_ptr(), ev.data_ptr()
                pf.psi_h[0], pf.psi_h[1] = hu.data_ptr(), hv.data_ptr()
            if half is None:
                d.E, d.H, d.ce = sim.E.data_ptr(), sim.H.data_ptr(), sim._ce.data_ptr()
            else:
                ntl = (sim.shape[1] * sim.shape[2] + 31) // 32
                e16 = torch.empty(3 * sim.N, dtype=half, device=dev)
                h16 = torch.empty(3 * sim.N, dtype=half, device=dev)
                ce16 = sim._ce.to(half)
                self._keep.append(ce16)
                self._e16.append(e16)
                self._h16.append(h16)
                d.E, d.H, d.ce = e16.data_ptr(), h16.data_ptr(), ce16.data_ptr()
                if scaled:
                    eexp = torch.zeros(sim.shape[0] * ntl, dtype=torch.int32, device=dev)
                    hexp = torch.zeros_like(eexp)
                    self._eexp.append(eexp)
                    self._hexp.append(hexp)
                    d.e_exp, d.h_exp = eexp.data_ptr(), hexp.data_ptr()
            src = list(sources[v])
            if len(src) > _lib.FDTD_BATCH_MAX_SRC:
                raise ValueError("at most %d point sources per variant" % _lib.FDTD_BATCH_MAX_SRC)
            d.n_src = len(src)
            if src:
                vals = numpy.zeros((max(self.steps, 1), len(src)), dtype=numpy.float32)
                for k, (ind, w) in enumerate(src):
                    w = numpy.asarray(w, dtype=numpy.float64).ravel()
                    if w.size < self.steps:
                        raise ValueError("source %d of variant %d has %d values for %d steps" % (k, v, w.size, self.steps))
                    vals[:self.steps, k] = w[:self.steps]
                    d.src_index[k] = int(ind)
                t = torch.from_numpy(vals).to(dev)
                self._keep.append(t)
                d.src_values = t.data_ptr()
            mon = [int(i) for i in monitors[v]]
            if len(mon) > _lib.FDTD_BATCH_MAX_MON:
                raise ValueError("at most %d monitor points per variant" % _lib.FDTD_BATCH_MAX_MON)
            d.n_mon = len(mon)
            ser = None
            if mon:
                ser = torch.zeros((max(self.steps, 1), len(mon)), dtype=torch.float64, device=dev)
                for k, i in enumerate(mon):
                    d.mon_index[k] = i
                d.series = ser.data_ptr()
            self.series.append(ser)
        torch.cuda.synchronize(dev)
        self._batch = ctypes.c_void_p()
        _lib.check(self._lib.fdtd_batch_create(arr, n, _STORE[storage], self.steps, ctypes.byref(self._batch)))
        self._arr = arr
        self.schedule = "launches"
        if half is not None:
            self.load()
        self._graph = None

    # ---- 16-bit copies ----------------------------------------------------------------------
    def load(self):
        """Encode the simulations' current E and H into the 16-bit copies (no-op for f32)."""
        if self.storage == "f32":
            return
        st = ctypes.c_void_p(self.queue.cuda_stream)
        for v, sim in enumerate(self.sims):
            _lib.check(self._lib.fdtd_batch_encode(self._batch, v, 0, ctypes.c_void_p(sim.E.data_ptr()), st))
            _lib.check(self._lib.fdtd_batch_encode(self._batch, v, 1, ctypes.c_void_p(sim.H.data_ptr()), st))

    def sync(self):
        """Decode the 16-bit copies into the simulations' E and H (no-op for f32)."""
        if self.storage == "f32":
            return
        st = ctypes.c_void_p(self.queue.cuda_stream)
        for v, sim in enumerate(self.sims):
            _lib.check(self._lib.fdtd_batch_decode(self._batch, v, 0, ctypes.c_void_p(sim.E.data_ptr()), st))
            _lib.check(self._lib.fdtd_batch_decode(self._batch, v, 1, ctypes.c_void_p(sim.H.data_ptr()), st))

    # ---- stepping ---------------------------------------------------------------------------
    def tune(self, xchunk: int = 8, blocks_per_sm: int = 0, schedule: str = None):
        """Tile shape (x planes per tile), resident blocks per SM of the persistent schedule
        (0: as many as fit) and the schedule: 'launches' (two launches per step, each over the
        tiles of every variant; default) or 'persistent' (one cooperative launch per run)."""
        _lib.check(self._lib.fdtd_batch_tune(self._batch, int(xchunk), int(blocks_per_sm)))
        if schedule is not None:
            if schedule not in ("launches", "persistent"):
                raise ValueError("schedule must be 'launches' or 'persistent'")
            _lib.check(self._lib.fdtd_batch_schedule(
                self._batch, _lib.FDTD_BATCH_LAUNCHES if schedule == "launches" else _lib.FDTD_BATCH_PERSISTENT))
            self.schedule = schedule
        self._graph = None

    def autotune(self, steps: int = 10, cache_path: str | None = None, **kw) -> dict:
        """Time the candidate tile shapes on this batch, apply the fastest and restore the
        state (autotune.tune_batch)."""
        from .autotune import tune_batch
        return tune_batch(self, steps=steps, cache_path=cache_path, **kw)

    def run(self, nsteps: int):
        """Advance every variant by nsteps steps in one launch on the simulations' stream."""
        _lib.check(self._lib.fdtd_batch_run(self._batch, ctypes.c_void_p(self.queue.cuda_stream), int(nsteps)))
        self.steps_run += int(nsteps)
        for sim in self.sims:
            sim.steps_run += int(nsteps)

    def capture(self, nsteps: int):
        """Capture one run(nsteps) in a CUDA graph; replay() then repeats it."""
        import torch
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(device=self.device)
        s.wait_stream(self.queue)
        with torch.cuda.graph(g, stream=s):
            _lib.check(self._lib.fdtd_batch_run(self._batch, ctypes.c_void_p(s.cuda_stream), int(nsteps)))
        self.queue.wait_stream(s)
        self._graph = (g, int(nsteps))
        return g

    def replay(self):
        """Replay the captured launch (advances every variant by the captured step count)."""
        import torch
        g, n = self._graph
        with torch.cuda.stream(self.queue):
            g.replay()
        self.steps_run += n
        for sim in self.sims:
            sim.steps_run += n

    def step_counter(self) -> int:
        """The device step counter: the source / monitor row of the next step."""
        v = ctypes.c_int64()
        _lib.check(self._lib.fdtd_batch_get_step(self._batch, ctypes.byref(v)))
        return int(v.value)

    def set_step_counter(self, step: int):
        _lib.check(self._lib.fdtd_batch_set_step(self._batch, int(step)))

    def close(self):
        if getattr(self, "_batch", None) is not None and self._batch.value:
            self._lib.fdtd_batch_destroy(self._batch)
            self._batch = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
