"""
Harness for the C restatement of the reference kernels (TEST INFRASTRUCTURE).

``PortSimulation`` mirrors the reference's ``Simulation`` (opencl_fdtd/simulation.py:77-271)
on host numpy arrays and drives oracle/fdtd_port.c through ctypes. It is the checker the CUDA
path is compared with, the FP64 oracle (``float_type=numpy.float64``) for error reports, and
the checker for the two extensions the reference lacks (diagonal mu, Bloch-phase coupling).

PML psi arrays keep the reference's layout (opencl_fdtd/kernels/update_e.cl:92):
shape (T, s_u, s_v) for a face on axis r with (u, v) the other two axes in xyz order.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import warnings

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD, "libfdtd_port.so")

PML_DEFAULTS = (("thickness", 8), ("epsilon_eff", 1.0), ("mu_eff", 1.0),
                ("ln_R_per_layer", -1.6), ("m", 3.5), ("cfs_alpha", 0), ("ma", 1))


class PortDesc(ctypes.Structure):
    _fields_ = [
        ("sx", ctypes.c_int64), ("sy", ctypes.c_int64), ("sz", ctypes.c_int64),
        ("dt", ctypes.c_double),
        ("uniform", ctypes.c_int32), ("dx", ctypes.c_double),
        ("inv_de", ctypes.c_void_p * 3), ("inv_dh", ctypes.c_void_p * 3),
        ("npml", ctypes.c_int32),
        ("axis", ctypes.c_int32 * 6), ("pol", ctypes.c_int32 * 6),
        ("thick", ctypes.c_int64 * 6),
        ("pe", (ctypes.c_void_p * 3) * 6), ("ph", (ctypes.c_void_p * 3) * 6),
        ("nbloch", ctypes.c_int32), ("baxis", ctypes.c_int32 * 3),
        ("bre", ctypes.c_double * 3), ("bim", ctypes.c_double * 3),
        ("nthreads", ctypes.c_int32),
    ]


def build(force: bool = False) -> str:
    """Compile fdtd_port.c (gcc -O3 -fopenmp -ffp-contract=off) into oracle/_build/."""
    src = os.path.join(HERE, "fdtd_port.c")
    body = os.path.join(HERE, "fdtd_port_body.h")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(src), os.path.getmtime(body))):
        return LIB_PATH
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB_PATH + ".%d.tmp" % os.getpid()
    subprocess.check_call(["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
                           "-std=c11", src, "-o", tmp])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        D = ctypes.POINTER(PortDesc)
        for sfx in ("f32", "f64"):
            getattr(L, "port_update_e_" + sfx).argtypes = [D, P, P, P, ctypes.c_int, P, P]
            getattr(L, "port_update_h_" + sfx).argtypes = [D, P, P, P, ctypes.c_int, P, P, P]
            getattr(L, "port_update_s_" + sfx).argtypes = [D, P, P]
            getattr(L, "port_update_j_" + sfx).argtypes = [D, P, P, P, ctypes.c_double,
                                                          ctypes.c_double, P]
        _LIB = L
    return _LIB


def pml_tables(pml: dict, dt, dtype):
    """CPML coefficient tables, restating opencl_fdtd/simulation.py:284-307.

    Arithmetic follows numpy 1.x value-based casting, for which the reference was written:
    the depth arrays have the field dtype and every scalar (dt, kappa_max, sigma_max ...) is
    cast to that dtype before it meets them. Returns ((p0e, p1e, p2e), (p0h, p1h, p2h)).
    """
    f = numpy.dtype(dtype).type
    T = pml["thickness"]
    sigma_max = -pml["ln_R_per_layer"] / 2 * (pml["m"] + 1)
    kappa_max = float(numpy.sqrt(pml["mu_eff"] * pml["epsilon_eff"]))
    alpha_max = pml["cfs_alpha"]

    def par(x):
        scaling = (x / f(T)) ** pml["m"]
        sigma = scaling * f(sigma_max)
        kappa = f(1) + scaling * f(kappa_max - 1)
        alpha = ((f(1) - x / f(T)) ** pml["ma"]) * f(alpha_max)
        p0 = numpy.exp(-(sigma / kappa + alpha) * f(dt))
        p1 = sigma / (sigma + kappa * alpha) * (p0 - f(1))
        p2 = f(1) / kappa
        return p0.astype(dtype), p1.astype(dtype), p2.astype(dtype)

    xe = numpy.arange(1, T + 1, dtype=dtype)[::-1].copy()
    xh = numpy.arange(1, T + 1, dtype=dtype)[::-1].copy()
    if pml["polarity"] == "p":
        xe -= f(0.5)
    elif pml["polarity"] == "n":
        xh -= f(0.5)
    return par(xe), par(xh)


def _vec(f, dtype):
    return numpy.concatenate([numpy.asarray(c).ravel(order="C") for c in f]).astype(dtype)


class PortSimulation:
    """Host-memory mirror of the reference Simulation, stepping through fdtd_port.c."""

    def __init__(self, epsilon, pmls, bloch_boundaries=(), dxes=None, dt=None,
                 initial_fields=None, float_type=numpy.float32, do_poynting=True,
                 do_fieldsrc=False, mu=None, nthreads: int = 0):
        initial_fields = initial_fields or {}
        self.shape = tuple(int(s) for s in epsilon[0].shape)
        self.dtype = numpy.dtype(float_type)
        if self.dtype not in (numpy.float32, numpy.float64):
            raise Exception("Unsupported type")
        self.sfx = "f32" if self.dtype == numpy.float32 else "f64"
        self.N = int(numpy.prod(self.shape))
        self.eps = _vec(epsilon, self.dtype)
        self.mu = None if mu is None else _vec(mu, self.dtype)
        d = PortDesc()
        d.sx, d.sy, d.sz = self.shape
        self._keep = []
        if dxes is None:
            dxes = 1.0
        if isinstance(dxes, (float, int)):
            d.uniform, d.dx = 1, float(dxes)
            min_dx = dxes
        else:
            d.uniform, d.dx = 0, 0.0
            inv = [numpy.asarray(1 / numpy.asarray(dxn, dtype=numpy.float64)).astype(self.dtype)
                   for dxn in list(dxes[0]) + list(dxes[1])]
            self._keep += inv
            for r in range(3):
                d.inv_de[r] = inv[r].ctypes.data
                d.inv_dh[r] = inv[3 + r].ctypes.data
            min_dx = min(min(dxn) for dxn in list(dxes[0]) + list(dxes[1]))
        max_dt = min_dx * .99 / float(numpy.sqrt(3))
        if dt is None:
            self.dt = max_dt
        elif dt > max_dt:
            warnings.warn("Warning: unstable dt: {}".format(dt))
            self.dt = dt
        elif dt <= 0:
            raise Exception("Invalid dt: {}".format(dt))
        else:
            self.dt = dt
        d.dt = float(self.dt)

        def field(key):
            v = initial_fields.get(key)
            return numpy.zeros(3 * self.N, self.dtype) if v is None else _vec(v, self.dtype)

        self.E, self.H = field("E"), field("H")
        self.bloch = list(bloch_boundaries)
        if self.bloch:
            self.F, self.G = field("F"), field("G")
        else:
            self.F = self.G = None
        d.nbloch = len(self.bloch)
        for k, b in enumerate(self.bloch):
            d.baxis[k] = "xyz".index(b["axis"])
            d.bre[k], d.bim[k] = float(b["real"]), float(b["imag"])

        self.pmls = []
        d.npml = len(pmls)
        self.psi = {k: [] for k in "EHFG"}
        for k, pml in enumerate(pmls):
            for key, val in PML_DEFAULTS:
                pml.setdefault(key, val)
            a = "xyz".index(pml["axis"])
            d.axis[k], d.pol[k], d.thick[k] = a, 0 if pml["polarity"] == "n" else 1, pml["thickness"]
            te, th = pml_tables(pml, self.dt, self.dtype)
            self._keep += list(te) + list(th)
            for j in range(3):
                d.pe[k][j] = te[j].ctypes.data
                d.ph[k][j] = th[j].ctypes.data
            u, v = [s for s in range(3) if s != a]
            pshape = (pml["thickness"], self.shape[u], self.shape[v])
            for fk in "EHFG":
                self.psi[fk] += [numpy.zeros(pshape, self.dtype), numpy.zeros(pshape, self.dtype)]
            self.pmls.append(dict(pml))
        d.nthreads = int(nthreads) if nthreads else (os.cpu_count() or 1)
        self.desc = d

        self.do_poynting = do_poynting
        self.oS = numpy.zeros(6 * self.N, self.dtype) if do_poynting else None
        self.S = numpy.zeros(3 * self.N, self.dtype) if do_poynting else None
        if do_fieldsrc:
            self.Jr = numpy.zeros(3 * self.N, self.dtype)
            self.Ji = numpy.zeros(3 * self.N, self.dtype)

    # ---- helpers ----
    def _fn(self, name):
        return getattr(lib(), "port_%s_%s" % (name, self.sfx))

    @staticmethod
    def _p(a):
        return None if a is None else a.ctypes.data

    def _psi_arr(self, key):
        arr = (ctypes.c_void_p * max(1, len(self.psi[key])))()
        for k, p in enumerate(self.psi[key]):
            arr[k] = p.ctypes.data
        return arr

    def set_threads(self, n: int):
        self.desc.nthreads = int(n)

    # ---- the reference's operations ----
    def update_E(self, wait_for=None):
        self._fn("update_e")(ctypes.byref(self.desc), self._p(self.E), self._p(self.H),
                             self._p(self.G), 0, self._p(self.eps), self._psi_arr("E"))

    def update_F(self, wait_for=None):
        self._fn("update_e")(ctypes.byref(self.desc), self._p(self.F), self._p(self.G),
                             self._p(self.H), 1, self._p(self.eps), self._psi_arr("F"))

    def update_H(self, wait_for=None):
        self._fn("update_h")(ctypes.byref(self.desc), self._p(self.H), self._p(self.E),
                             self._p(self.F), 0, self._p(self.mu), self._psi_arr("H"),
                             self._p(self.oS))

    def update_G(self, wait_for=None):
        self._fn("update_h")(ctypes.byref(self.desc), self._p(self.G), self._p(self.F),
                             self._p(self.E), 1, self._p(self.mu), self._psi_arr("G"), None)

    def update_S(self, wait_for=None):
        self._fn("update_s")(ctypes.byref(self.desc), self._p(self.S), self._p(self.oS))

    def update_J(self, wait_for, c, s, xmin, xmax, ymin, ymax, zmin, zmax):
        box = (ctypes.c_int64 * 6)(xmin, xmax, ymin, ymax, zmin, zmax)
        self._fn("update_j")(ctypes.byref(self.desc), self._p(self.E), self._p(self.Jr),
                             self._p(self.Ji), float(c), float(s), box)

    def step(self, source=None):
        """One canonical step (opencl_fdtd fdtd.py:162-175): E, (F), source, H, (G), S.
        ``source`` is an iterable of (flat_index, value) added to E after the E update."""
        self.update_E()
        if self.F is not None:
            self.update_F()
        if source:
            for ind, val in source:
                self.E[ind] = self.E[ind] + self.dtype.type(val)
        self.update_H()
        if self.F is not None:
            self.update_G()
        if self.do_poynting:
            self.update_S()
