"""
Drop-in replacement of opencl_fdtd's ``Simulation`` (opencl_fdtd/simulation.py:24-271) whose
time-stepping kernels are hand-written sm_103a CUDA reached through the C ABI of
include/fdtd_gb300.h.

What stays the same for a caller of the reference:
  * the constructor arguments and their defaults, including the in-place ``setdefault`` of
    each PML dict (simulation.py:161-168) and the exceptions raised for bad epsilon/dt;
  * the members E, H (F, G with Bloch boundaries; S, oS with Poynting; Jr, Ji with the field
    source), eps, dt, shape, arg_type, inv_dxes and sources;
  * every field is one flat array of 3N elements, components [X | Y | Z] in C order, so
    ``sim.E[numpy.ravel_multi_index(p, shape) + c*N] += v`` adds a soft source as in
    opencl_fdtd's fdtd.py:168-169;
  * update_E/H/S/F/G(wait_for) and update_J(wait_for, c, s, xmin, xmax, ymin, ymax, zmin,
    zmax) enqueue one update and return an event with ``wait()``; update_S is None with
    Poynting off, update_J is None without the field source.

What differs:
  * fields are torch CUDA tensors (``sim.get('E')`` replaces pyopencl's ``sim.E.get()``);
    ``context`` selects the CUDA device and ``queue`` may be a torch.cuda.Stream;
  * ``mu`` (diagonal permeability, 3 arrays) is accepted; the reference has none;
  * Bloch boundaries couple the split real/imaginary fields with the given phase (the
    reference's template code for this is never rendered, so its F and G updates are plain
    periodic; with real=1, imag=0 both agree bit for bit);
  * an unstable dt warns and is then used (the reference warns and leaves dt unset), and
    malformed initial fields raise (the reference builds the exceptions but never raises);
  * ``run(nsteps, point_sources)`` advances many canonical steps in one call with the
    per-step source values already on the device, and ``state_dict()`` /
    ``load_state_dict()`` checkpoint every field and CPML auxiliary array.
"""
from __future__ import annotations

import ctypes
import warnings
from typing import Dict, List

import numpy
import torch

from . import _lib
from .pml import apply_defaults, grading, psi_shape

__all__ = ["Simulation", "type_to_C", "Event"]


def type_to_C(float_type) -> str:
    """C name of a numpy float type (simulation.py:360-376)."""
    if float_type == numpy.float16:
        arg_type = "half"
    elif float_type == numpy.float32:
        arg_type = "float"
    elif float_type == numpy.float64:
        arg_type = "double"
    else:
        raise Exception("Unsupported type")
    return arg_type


class Event:
    """Completion marker of one enqueued update (pyopencl.Event's role); wait() blocks."""

    __slots__ = ("_ev",)

    def __init__(self, stream: torch.cuda.Stream):
        self._ev = torch.cuda.Event()
        self._ev.record(stream)

    def wait(self):
        self._ev.synchronize()

    def query(self) -> bool:
        return self._ev.query()


_TORCH_DTYPE = {numpy.dtype(numpy.float32): torch.float32, numpy.dtype(numpy.float64): torch.float64}


class Simulation:
    """Constructs and holds the FDTD fields and the update operations acting on them.

    Canonical loop (opencl_fdtd's fdtd.py:162-175)::

        for t in range(max_t):
            sim.update_E([]).wait()
            sim.E[ind] += field_source(t)
            e = sim.update_H([])
            if sim.update_S:
                e = sim.update_S([e])
            e.wait()
    """

    E = None
    H = None
    S = None
    oS = None
    F = None
    G = None
    Jr = None
    Ji = None
    eps = None
    mu = None
    dt = None
    inv_dxes = None
    arg_type = None
    context = None
    queue = None
    update_E = None
    update_H = None
    update_S = None
    update_F = None
    update_G = None
    update_J = None
    sources = None

    def __init__(self,
                 epsilon: List[numpy.ndarray],
                 pmls: List[Dict[str, int or float]],
                 bloch_boundaries: List[Dict[str, int or float]] = (),
                 dxes: List[List[numpy.ndarray]] or float = None,
                 dt: float = None,
                 initial_fields: Dict[str, List[numpy.ndarray]] = None,
                 context=None,
                 queue=None,
                 float_type=numpy.float32,
                 do_poynting: bool = True,
                 do_fieldsrc: bool = False,
                 mu: List[numpy.ndarray] = None):
        if initial_fields is None:
            initial_fields = {}
        self._lib = _lib.load()
        self._plan = ctypes.c_void_p()

        self.shape = tuple(int(s) for s in numpy.shape(epsilon[0]))
        self.arg_type = float_type
        ctype = type_to_C(float_type)
        if ctype == "half":
            raise Exception("Unsupported type: float16 fields are not supported "
                            "(the reference's half kernels need cl_khr_fp16)")
        self._np_dtype = numpy.dtype(float_type)
        self._dtype = _TORCH_DTYPE[self._np_dtype]
        self.sources = {}
        self.N = int(numpy.prod(self.shape))
        self._create_context(context, queue)
        self._create_eps(epsilon)
        if mu is not None:
            self.mu = self._create_material(mu, "Mu")

        if dxes is None:
            dxes = 1.0
        if isinstance(dxes, (float, int)):
            uniform_dx = dxes
            min_dx = dxes
        else:
            uniform_dx = False
            spacing = list(dxes[0]) + list(dxes[1])
            self.inv_dxes = [self._to_device(1 / numpy.asarray(dxn, dtype=numpy.float64))
                             for dxn in spacing]
            for r in range(3):
                for g in (0, 3):
                    if self.inv_dxes[g + r].numel() != self.shape[r]:
                        raise Exception("dxes[{}][{}] must have length {}".format(g // 3, r, self.shape[r]))
            min_dx = min(float(numpy.min(dxn)) for dxn in spacing)

        max_dt = min_dx * .99 / numpy.sqrt(3)
        if dt is None:
            self.dt = float(max_dt)
        elif dt > max_dt:
            warnings.warn("Warning: unstable dt: {}".format(dt))
            self.dt = float(dt)
        elif dt <= 0:
            raise Exception("Invalid dt: {}".format(dt))
        else:
            self.dt = float(dt)

        self.E = self._create_field(initial_fields.get("E", None))
        self.H = self._create_field(initial_fields.get("H", None))
        self.bloch_boundaries = [dict(b) for b in bloch_boundaries]
        if bloch_boundaries:
            self.F = self._create_field(initial_fields.get("F", None))
            self.G = self._create_field(initial_fields.get("G", None))

        for pml in pmls:
            apply_defaults(pml)
        self.pmls = pmls

        self.do_poynting = bool(do_poynting)
        self.do_fieldsrc = bool(do_fieldsrc)
        if do_poynting:
            self.oS = torch.zeros((3 * self.N, 2), dtype=self._dtype, device=self.device)
            self.S = torch.zeros_like(self.E)
        if do_fieldsrc:
            self.Ji = torch.zeros_like(self.E)
            self.Jr = torch.zeros_like(self.E)

        self._create_pmls(pmls)
        self._uniform_dx = uniform_dx
        self._create_plan(uniform_dx)
        # dt/eps and dt/mu, the per-cell quotients of the updates, cached on the device and
        # refreshed whenever eps or mu change (tracked through torch's version counter)
        self._ce = torch.empty_like(self.eps)
        self._cm = torch.empty_like(self.mu) if self.mu is not None else None
        self._mat_key = None
        self._buf_key = None
        self._buf = _lib.FdtdBuffers()
        self._scratch = None
        self.steps_run = 0

        self.update_E = self._create_operation(self._lib.fdtd_update_e)
        self.update_H = self._create_operation(self._lib.fdtd_update_h)
        if do_poynting:
            self.update_S = self._create_operation(self._lib.fdtd_update_s)
        if bloch_boundaries:
            self.update_F = self._create_operation(self._lib.fdtd_update_f)
            self.update_G = self._create_operation(self._lib.fdtd_update_g)
        if do_fieldsrc:
            self.update_J = self._create_field_source_operation()
        self._describe_sources(ctype, uniform_dx)

    # ------------------------------------------------------------------------------------
    # construction helpers
    # ------------------------------------------------------------------------------------
    def _create_context(self, context=None, queue=None):
        if not torch.cuda.is_available():
            raise RuntimeError("opencl_fdtd_gb300 needs a CUDA device (no CPU fallback)")
        if context is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        elif isinstance(context, int):
            self.device = torch.device("cuda", context)
        else:
            self.device = torch.device(context)
            if self.device.index is None:
                self.device = torch.device("cuda", torch.cuda.current_device())
        self.context = self.device
        if queue is None:
            self.queue = torch.cuda.current_stream(self.device)
        else:
            self.queue = queue

    def _to_device(self, a) -> torch.Tensor:
        arr = numpy.ascontiguousarray(numpy.asarray(a), dtype=self._np_dtype)
        return torch.from_numpy(arr).to(self.device)

    def _create_material(self, mats, name: str) -> torch.Tensor:
        if len(mats) != 3:
            raise Exception("{} must be a list with length of 3".format(name))
        if not all((numpy.shape(e) == numpy.shape(mats[0]) for e in mats[1:])):
            raise Exception("All {} grids must have the same shape. Shapes are {}".format(
                name.lower(), [numpy.shape(e) for e in mats]))
        if not tuple(numpy.shape(mats[0])) == self.shape:
            raise Exception("{} shape mismatch. Expected {}, got {}".format(
                name, self.shape, numpy.shape(mats[0])))
        return self._to_device(numpy.concatenate([numpy.asarray(m).ravel(order="C") for m in mats]))

    def _create_eps(self, epsilon):
        # simulation.py:340-347
        self.eps = self._create_material(epsilon, "Epsilon")

    def _create_field(self, initial_value=None) -> torch.Tensor:
        # simulation.py:349-357
        if initial_value is None:
            return torch.zeros(3 * self.N, dtype=self._dtype, device=self.device)
        if len(initial_value) != 3:
            raise Exception("Initial field value must be a list of length 3")
        if not all((tuple(numpy.shape(f)) == self.shape for f in initial_value)):
            raise Exception("Initial field list elements must have same shape as epsilon elements")
        return self._to_device(numpy.concatenate([numpy.asarray(f).ravel(order="C")
                                                  for f in initial_value]))

    def _create_pmls(self, pmls):
        # simulation.py:274-319: coefficient tables on the host (copied by the plan), the
        # auxiliary psi arrays as device tensors owned here
        self._pml_tables = []
        self.psi = {"E": [], "H": [], "F": [], "G": []}
        seen = set()
        for pml in pmls:
            if pml["axis"] not in ("x", "y", "z"):
                raise Exception("Invalid pml axis: {}".format(pml["axis"]))
            if pml["polarity"] not in ("n", "p"):
                raise Exception("Invalid pml polarity: {}".format(pml["polarity"]))
            key = (pml["axis"], pml["polarity"])
            if key in seen:
                raise Exception("Duplicate pml face: {}".format(key))
            seen.add(key)
            a = "xyz".index(pml["axis"])
            T = int(pml["thickness"])
            te, th = grading(pml, self.dt, self._np_dtype)
            self._pml_tables.append((a, 0 if pml["polarity"] == "n" else 1, T, te, th))
            shp = psi_shape(self.shape, a, T)
            fields = "EHFG" if self.bloch_boundaries else "EH"
            for k in fields:
                self.psi[k].append((torch.zeros(shp, dtype=self._dtype, device=self.device),
                                    torch.zeros(shp, dtype=self._dtype, device=self.device)))

    def _create_plan(self, uniform_dx):
        d = _lib.FdtdDesc()
        d.shape[0], d.shape[1], d.shape[2] = self.shape
        d.dtype = _lib.FDTD_F64 if self._np_dtype == numpy.float64 else _lib.FDTD_F32
        d.uniform = 0 if uniform_dx is False else 1
        d.dx = float(uniform_dx) if uniform_dx is not False else 1.0
        d.dt = self.dt
        d.n_pml = len(self._pml_tables)
        for f, (a, pol, T, te, th) in enumerate(self._pml_tables):
            pd = d.pml[f]
            pd.axis, pd.polarity, pd.thickness = a, pol, T
            pd.p0e, pd.p1e, pd.p2e = (t.ctypes.data for t in te)
            pd.p0h, pd.p1h, pd.p2h = (t.ctypes.data for t in th)
        d.n_bloch = len(self.bloch_boundaries)
        for k, b in enumerate(self.bloch_boundaries):
            if b["axis"] not in ("x", "y", "z"):
                raise Exception("Invalid bloch axis: {}".format(b["axis"]))
            d.bloch[k].axis = "xyz".index(b["axis"])
            d.bloch[k].real = float(b["real"])
            d.bloch[k].imag = float(b["imag"])
        d.do_poynting = int(self.do_poynting)
        d.do_fieldsrc = int(self.do_fieldsrc)
        d.has_mu = int(self.mu is not None)
        self._desc = d
        with torch.cuda.device(self.device):
            _lib.check(self._lib.fdtd_plan_create(ctypes.byref(d), ctypes.byref(self._plan)))

    def _describe_sources(self, ctype, uniform_dx):
        faces = ", ".join("{}{}(T={})".format(p["axis"], p["polarity"], p["thickness"]) for p in self.pmls)
        common = "shape={} dtype={} dt={!r} dx={} pml=[{}]".format(
            self.shape, ctype, self.dt, uniform_dx if uniform_dx is not False else "tables", faces)
        self.sources["E"] = "k_yee_e<{}> (E += dt/eps * (curl H + psi_E)) {}".format(ctype, common)
        self.sources["H"] = "k_yee_h<{},mu={},poynting={}> (H -= dt{} * (curl E - psi_H)) {}".format(
            ctype, self.mu is not None, self.do_poynting, "/mu" if self.mu is not None else "", common)
        if self.do_poynting:
            self.sources["S"] = "k_poynting<{}> (S = dt/8 * sum of oS terms) {}".format(ctype, common)
        if self.bloch_boundaries:
            ph = ", ".join("{}:{}{:+}i".format(b["axis"], b["real"], b["imag"]) for b in self.bloch_boundaries)
            self.sources["F"] = "k_yee_e<{}> imaginary part, bloch=[{}] {}".format(ctype, ph, common)
            self.sources["G"] = "k_yee_h<{}> imaginary part, bloch=[{}] {}".format(ctype, ph, common)
        if self.do_fieldsrc:
            self.sources["J"] = "k_fieldsrc<{}> (E += c*Jr + s*Ji in a box) {}".format(ctype, common)

    # ------------------------------------------------------------------------------------
    # buffers and launches
    # ------------------------------------------------------------------------------------
    def _check_field(self, t: torch.Tensor, name: str, numel: int):
        if not isinstance(t, torch.Tensor):
            raise TypeError("{} must be a torch tensor".format(name))
        if t.device != self.device or t.dtype != self._dtype or not t.is_contiguous() \
                or t.numel() != numel:
            raise ValueError("{} must be a contiguous {} tensor of {} elements on {}".format(
                name, self._dtype, numel, self.device))

    def refresh_materials(self):
        """Recompute the cached dt/eps and dt/mu; needed only after eps or mu were changed
        by something other than a torch operation (torch in-place ops are detected)."""
        self._mat_key = None
        self._buffers()

    def _buffers(self) -> _lib.FdtdBuffers:
        key = (id(self.E), id(self.H), id(self.F), id(self.G), id(self.S), id(self.oS),
               id(self.eps), id(self.mu), id(self.Jr), id(self.Ji))
        if key == self._buf_key:
            mk = (self.eps._version, None if self.mu is None else self.mu._version)
            if mk != self._mat_key:
                self._prepare(mk)
            return self._buf
        n3 = 3 * self.N
        b = _lib.FdtdBuffers()
        for name in ("E", "H", "eps"):
            self._check_field(getattr(self, name), name, n3)
        b.E, b.H, b.eps = self.E.data_ptr(), self.H.data_ptr(), self.eps.data_ptr()
        if self.mu is not None:
            self._check_field(self.mu, "mu", n3)
            b.mu = self.mu.data_ptr()
        if self.bloch_boundaries:
            self._check_field(self.F, "F", n3)
            self._check_field(self.G, "G", n3)
            b.F, b.G = self.F.data_ptr(), self.G.data_ptr()
        if self.do_poynting:
            self._check_field(self.S, "S", n3)
            self._check_field(self.oS, "oS", 2 * n3)
            b.S, b.oS = self.S.data_ptr(), self.oS.data_ptr()
        if self.do_fieldsrc:
            self._check_field(self.Jr, "Jr", n3)
            self._check_field(self.Ji, "Ji", n3)
            b.Jr, b.Ji = self.Jr.data_ptr(), self.Ji.data_ptr()
        for key_psi, arr in (("E", b.psi_e), ("H", b.psi_h), ("F", b.psi_f), ("G", b.psi_g)):
            for f, pair in enumerate(self.psi[key_psi]):
                arr[f][0], arr[f][1] = pair[0].data_ptr(), pair[1].data_ptr()
        if self.inv_dxes is not None:
            for r in range(3):
                b.inv_de[r] = self.inv_dxes[r].data_ptr()
                b.inv_dh[r] = self.inv_dxes[3 + r].data_ptr()
        b.ce = self._ce.data_ptr()
        if self._cm is not None:
            b.cm = self._cm.data_ptr()
        self._buf = b
        self._attach_scratch(None)
        self._buf_key = key
        self._prepare((self.eps._version, None if self.mu is None else self.mu._version))
        return b

    def _attach_scratch(self, mode=None):
        """Point the C buffers at the second copies a run path uses: 'fused' (E, H and both
        CPML sides), 'hs' (H and the H-side CPML arrays) or None (no second copies)."""
        b = self._buf
        b.E2 = b.H2 = None
        for f in range(6):
            for c in range(2):
                b.psi_e2[f][c] = None
                b.psi_h2[f][c] = None
        if mode is None or self._scratch is None:
            return
        E2, H2, pe2, ph2 = self._scratch
        b.H2 = H2.data_ptr()
        for f, (u, v) in enumerate(ph2):
            b.psi_h2[f][0], b.psi_h2[f][1] = u.data_ptr(), v.data_ptr()
        if mode == "fused":
            b.E2 = E2.data_ptr()
            for f, (u, v) in enumerate(pe2):
                b.psi_e2[f][0], b.psi_e2[f][1] = u.data_ptr(), v.data_ptr()

    def _ensure_scratch(self, mode):
        """Second copies of H and the H-side CPML arrays (the default run path) and, for the
        fused path, of E and the E-side arrays; allocated on first use and kept."""
        E2, H2, pe2, ph2 = self._scratch if self._scratch is not None else (None, None, None, None)
        if H2 is None:
            H2 = torch.empty_like(self.H)
            ph2 = [(torch.empty_like(u), torch.empty_like(v)) for u, v in self.psi["H"]]
        if mode == "fused" and E2 is None:
            E2 = torch.empty_like(self.E)
            pe2 = [(torch.empty_like(u), torch.empty_like(v)) for u, v in self.psi["E"]]
        self._scratch = (E2, H2, pe2, ph2)

    def _prepare(self, mat_key):
        _lib.check(self._lib.fdtd_prepare(self._plan, ctypes.byref(self._buf),
                                          ctypes.c_void_p(self.queue.cuda_stream)))
        self._mat_key = mat_key

    def _stream_handle(self, wait_for):
        stream = self.queue
        if wait_for:
            for ev in wait_for:
                if isinstance(ev, Event):
                    stream.wait_event(ev._ev)
                elif isinstance(ev, torch.cuda.Event):
                    stream.wait_event(ev)
        return stream

    def _create_operation(self, fn):
        def op(wait_for=None):
            stream = self._stream_handle(wait_for)
            _lib.check(fn(self._plan, ctypes.byref(self._buffers()), ctypes.c_void_p(stream.cuda_stream)))
            return Event(stream)
        return op

    def _create_field_source_operation(self):
        fn = self._lib.fdtd_update_j

        def op(wait_for, c, s, xmin, xmax, ymin, ymax, zmin, zmax):
            stream = self._stream_handle(wait_for)
            box = (ctypes.c_int64 * 6)(int(xmin), int(xmax), int(ymin), int(ymax), int(zmin), int(zmax))
            _lib.check(fn(self._plan, ctypes.byref(self._buffers()), ctypes.c_void_p(stream.cuda_stream),
                          float(c), float(s), box))
            return Event(stream)
        return op

    # ------------------------------------------------------------------------------------
    # additions beyond the reference
    # ------------------------------------------------------------------------------------
    def run(self, nsteps: int, point_sources=None, wait_for=None, monitor=None,
            path: str = "auto", watchdog: int = 0) -> Event:
        """Advance ``nsteps`` canonical steps (E, F, point sources, H, G, S) in one call.

        ``watchdog`` > 0 runs the steps in chunks of that many and counts the non-finite
        field values on the device after each chunk (``nonfinite_count``); the first chunk
        that leaves any raises FloatingPointError with the step reached.

        ``point_sources`` is a list of (flat_index, values) pairs: after the E update of step
        t, ``E[flat_index] += values[t]`` (fdtd.py:168-169 without the host round trip).
        values are rounded to the field dtype, as the host-side ``+=`` does.

        ``path`` picks the kernels, all giving identical fields and S:
          'auto'   'hs' where it applies (Poynting on, no Bloch boundaries), else 'plain';
          'hs'     update_E in place, then H and S in one launch reading H (and the H-side
                   CPML arrays) from one copy and writing a second: 96 B per cell per step;
          'plain'  the per-update kernels (E, H, S), optionally over L2-resident x slabs
                   (tune(slab=...));
          'fused'  E, sources, H and S in one kernel per step (no Bloch boundaries), reading
                   every field once and writing it once: 72 B per cell per step.
        The 'hs' and 'fused' paths write oS on the last step only."""
        nsteps = int(nsteps)
        if watchdog and int(watchdog) > 0:
            return self._run_watched(nsteps, int(watchdog), point_sources, wait_for, monitor, path)
        stream = self._stream_handle(wait_for)
        src = None
        keep = []
        if point_sources:
            n = len(point_sources)
            if n > 64:
                raise ValueError("at most 64 point sources")
            idx = numpy.array([int(i) for i, _ in point_sources], dtype=numpy.int64)
            if (idx < 0).any() or (idx >= 3 * self.N).any():
                raise IndexError("point source index out of range")
            # staged in pinned host memory and copied without blocking the host: the caching
            # host allocator keeps the staging block until the copy on `stream` has run
            pinned = torch.empty((max(nsteps, 1), n), dtype=self.E.dtype, pin_memory=True)
            vals = pinned.numpy()
            for k, (_, v) in enumerate(point_sources):
                v = numpy.asarray(v, dtype=numpy.float64).ravel()
                if v.size < nsteps:
                    raise ValueError("point source {} has {} values for {} steps".format(k, v.size, nsteps))
                vals[:nsteps, k] = v[:nsteps]
            with torch.cuda.stream(stream):
                val_t = pinned.to(self.device, non_blocking=True)
            idx_host = (ctypes.c_int64 * n)(*idx.tolist())
            keep = [val_t]
            src = _lib.FdtdPointSources(n, 0, ctypes.addressof(idx_host), val_t.data_ptr())
        if path not in ("auto", "hs", "plain", "fused"):
            raise ValueError("path must be 'auto', 'hs', 'plain' or 'fused'")
        hs_ok = self.do_poynting and not self.bloch_boundaries
        if path == "auto":
            path = "hs" if hs_ok else "plain"
        if path in ("hs", "fused") and self.bloch_boundaries:
            raise ValueError("the '%s' path does not support Bloch boundaries" % path)
        if path == "hs" and not self.do_poynting:
            raise ValueError("the 'hs' path needs do_poynting=True")
        mode = None if path == "plain" else path
        if mode:
            self._ensure_scratch(mode)
        bufs = self._buffers()
        self._attach_scratch(mode)
        mon = monitor.struct(nsteps) if monitor is not None else None
        _lib.check(self._lib.fdtd_run(self._plan, ctypes.byref(bufs),
                                      ctypes.c_void_p(stream.cuda_stream), nsteps,
                                      ctypes.byref(src) if src is not None else None,
                                      ctypes.byref(mon) if mon is not None else None))
        if monitor is not None:
            monitor.samples += nsteps
        for t in keep:
            t.record_stream(stream)
        self.steps_run += nsteps
        return Event(stream)

    def _run_watched(self, nsteps, every, point_sources, wait_for, monitor, path):
        if nsteps <= 0:
            return self.run(nsteps, point_sources=point_sources, wait_for=wait_for,
                            monitor=monitor, path=path)
        for k, (_, v) in enumerate(point_sources or ()):
            size = numpy.asarray(v, dtype=numpy.float64).size
            if size < nsteps:
                # the whole run is checked before the first chunk moves the fields
                raise ValueError("point source {} has {} values for {} steps".format(k, size, nsteps))
        ev = None
        for t0 in range(0, nsteps, every):
            n = min(every, nsteps - t0)
            sub = None
            if point_sources:
                sub = [(i, numpy.asarray(v, dtype=numpy.float64).ravel()[t0:t0 + n]) for i, v in point_sources]
            ev = self.run(n, point_sources=sub, wait_for=wait_for if t0 == 0 else None, monitor=monitor, path=path)
            bad = self.nonfinite_count()
            if bad:
                raise FloatingPointError("%d non-finite field values after step %d" % (bad, self.steps_run))
        return ev

    def nonfinite_count(self) -> int:
        """Number of NaN / Inf values in E and H (and F, G), counted on the device
        (fdtd_count_nonfinite) and read back (waits for the simulation's stream)."""
        if getattr(self, "_nf", None) is None:
            self._nf = torch.zeros(1, dtype=torch.int32, device=self.device)
        _lib.check(self._lib.fdtd_count_nonfinite(self._plan, ctypes.byref(self._buffers()), self._nf.data_ptr(),
                                                  ctypes.c_void_p(self.queue.cuda_stream)))
        self.queue.synchronize()
        return int(self._nf.item())

    def check_finite(self) -> bool:
        return self.nonfinite_count() == 0

    # ---- FP64 monitors --------------------------------------------------------------------
    def dft_monitor(self, points, omegas=(), record: bool = True, t0: int = None):
        """A DftMonitor on this simulation (pass it to run(monitor=...) or call sample())."""
        from .monitors import DftMonitor
        return DftMonitor(self, points, omegas, record=record,
                          t0=self.steps_run if t0 is None else t0)

    def _reduction_buffers(self):
        if getattr(self, "_red", None) is None:
            self._red = (torch.empty(1024, dtype=torch.float64, device=self.device),
                         torch.empty(1, dtype=torch.float64, device=self.device))
        return self._red

    def plane_sum(self, field: str, component: int, axis, index: int) -> float:
        """FP64 sum of one component of E, H or S over the plane ``index`` normal to ``axis``
        (a Poynting-flux integral for field 'S' and component == axis, in cell units)."""
        a = "xyz".index(axis) if isinstance(axis, str) else int(axis)
        t = getattr(self, field)
        self._check_field(t, field, 3 * self.N)
        scratch, out = self._reduction_buffers()
        _lib.check(self._lib.fdtd_plane_sum(self._plan, t.data_ptr(), int(component), a, int(index),
                                            scratch.data_ptr(), scratch.numel(), out.data_ptr(),
                                            ctypes.c_void_p(self.queue.cuda_stream)))
        self.queue.synchronize()
        return float(out.item())

    def flux(self, axis, index: int) -> float:
        """Poynting flux through plane ``index`` normal to ``axis``: sum of S_axis there."""
        if not self.do_poynting:
            raise Exception("flux needs do_poynting=True")
        a = "xyz".index(axis) if isinstance(axis, str) else int(axis)
        return self.plane_sum("S", a, a, index)

    def energy(self) -> float:
        """FP64 total field energy 1/2 sum(eps E^2 + mu H^2) (PEC cells excluded)."""
        scratch, out = self._reduction_buffers()
        _lib.check(self._lib.fdtd_energy(self._plan, ctypes.byref(self._buffers()), scratch.data_ptr(),
                                         scratch.numel(), out.data_ptr(),
                                         ctypes.c_void_p(self.queue.cuda_stream)))
        self.queue.synchronize()
        return float(out.item())

    def slab_planes(self) -> int:
        """x planes per slab of run()'s per-update schedule (whole grid when 0)."""
        v = ctypes.c_int32()
        _lib.check(self._lib.fdtd_plan_get(self._plan, _lib.FDTD_TUNE_SLAB, ctypes.byref(v)))
        return v.value or self.shape[0]

    def tune(self, xchunk: int = None, slab: int = None, fused_rows: int = None,
             fused_xchunk: int = None, hs_xchunk: int = None, hs_prefetch: bool = None,
             fused_stages: int = None, fused_tma: bool = None, fused_shape: int = None,
             hs_reverse: bool = None, hs_dft: bool = None, pdl: bool = None,
             e_form: int = None):
        """Kernel tiling and launch options (None keeps a value); results do not depend on them.

        fused_rows / fused_xchunk / fused_stages: own y rows of a one-pass step tile, x planes
        of a block, planes in its shared-memory ring (0: automatic); fused_tma: stage the rows
        of non-wrapping tiles with bulk asynchronous copies (default) or per element;
        fused_shape: block shape (1 large, 2 small, 0 automatic); hs_reverse: the H+S kernel of
        the 'hs' path takes its x chunks in descending order (default) or ascending; hs_dft:
        the step's DFT monitor sample is taken inside the H+S launch (default) instead of on a
        side stream; pdl: the E and H+S kernels of the 'hs' path use programmatic dependent
        launch (default); e_form: form of the bulk E kernel (0 next plane loaded ahead at three
        blocks per SM, 1 (default) per-plane loads at four)."""
        for key, val in ((_lib.FDTD_TUNE_XCHUNK, xchunk), (_lib.FDTD_TUNE_SLAB, slab),
                         (_lib.FDTD_TUNE_FUSED_ROWS, fused_rows),
                         (_lib.FDTD_TUNE_FUSED_XCHUNK, fused_xchunk),
                         (_lib.FDTD_TUNE_HS_XCHUNK, hs_xchunk),
                         (_lib.FDTD_TUNE_HS_PREFETCH, None if hs_prefetch is None else int(hs_prefetch)),
                         (_lib.FDTD_TUNE_FUSED_STAGES, fused_stages),
                         (_lib.FDTD_TUNE_FUSED_TMA, None if fused_tma is None else int(fused_tma)),
                         (_lib.FDTD_TUNE_FUSED_SHAPE, fused_shape),
                         (_lib.FDTD_TUNE_HS_REVERSE, None if hs_reverse is None else int(hs_reverse)),
                         (_lib.FDTD_TUNE_HS_DFT, None if hs_dft is None else int(hs_dft)),
                         (_lib.FDTD_TUNE_PDL, None if pdl is None else int(pdl)),
                         (_lib.FDTD_TUNE_E_FORM, e_form)):
            if val is not None:
                _lib.check(self._lib.fdtd_plan_tune(self._plan, key, int(val)))

    def tuning(self, key: str) -> int:
        """Current value of a tuning key ('fused_rows', 'hs_xchunk', ...) or of a read-only key:
        'last_run_path' (0 none, 1 per-update, 2 H+S, 3 one-pass), 'step_rows',
        'step_xchunk', 'step_stages', 'step_threads', 'step_shape' (tiling of the last one-pass
        launch) and 'hs_xchunk_used' (x chunk of the last H+S launch)."""
        name = key.upper()
        const = getattr(_lib, "FDTD_GET_" + name, None)
        if const is None:
            const = getattr(_lib, "FDTD_TUNE_" + name)
        v = ctypes.c_int32()
        _lib.check(self._lib.fdtd_plan_get(self._plan, const, ctypes.byref(v)))
        return v.value

    def device_status(self) -> int:
        """Bits of bounded device-side waits that ran out since the last call (0: none); waits
        for the queue. Raises FdtdError (FDTD_ERR_WATCHDOG) when any bit is set."""
        bits = ctypes.c_int32()
        _lib.check(self._lib.fdtd_device_status(self._plan, ctypes.c_void_p(self.queue.cuda_stream),
                                                ctypes.byref(bits)))
        return bits.value

    def get(self, name: str) -> numpy.ndarray:
        """Host copy of a field (what ``pyopencl.array.Array.get()`` returns)."""
        t = getattr(self, name)
        self.queue.synchronize()
        return t.detach().cpu().numpy().reshape(-1) if name != "oS" else t.detach().cpu().numpy()

    def state_dict(self) -> dict:
        """Every piece of time-stepping state: fields, CPML auxiliary arrays, step counter."""
        self.queue.synchronize()
        st = {"steps_run": self.steps_run}
        for name in ("E", "H", "F", "G", "S", "oS"):
            t = getattr(self, name)
            if t is not None:
                st[name] = t.detach().clone()
        st["psi"] = {k: [(u.detach().clone(), v.detach().clone()) for u, v in lst]
                     for k, lst in self.psi.items()}
        return st

    def load_state_dict(self, st: dict):
        self.queue.synchronize()
        for name in ("E", "H", "F", "G", "S", "oS"):
            t = getattr(self, name)
            if t is not None and name in st:
                t.copy_(st[name])
        for k, lst in self.psi.items():
            for (u, v), (su, sv) in zip(lst, st["psi"][k]):
                u.copy_(su)
                v.copy_(sv)
        self.steps_run = int(st.get("steps_run", 0))

    def save_snapshot(self, path, grid=None):
        """Write {'grid', 'E', 'H'[, 'S']} as opencl_fdtd's driver does (fdtd.py:181-191)."""
        from .snapshot import save_snapshot
        save_snapshot(self, path, grid)

    def save_checkpoint(self, path):
        from .snapshot import save_checkpoint
        save_checkpoint(self, path)

    def load_checkpoint(self, path):
        from .snapshot import load_checkpoint
        load_checkpoint(self, path)

    def close(self):
        if self._plan:
            self._lib.fdtd_plan_destroy(self._plan)
            self._plan = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
