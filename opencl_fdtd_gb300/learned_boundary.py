"""
Learned thin absorbing boundary: a per-face MLP that stands in for the CPML layers of a
Simulation, trained on the GPU by this package's own kernels on data that plain CPML runs
generate.

The model (kernels in csrc/lbc.cu, C ABI fdtd_lbc_* / fdtd_mlp_* / fdtd_adam):
  * every column of a learned face (a cell of the face's plane) reads Ex Ey Ez Hx Hy Hz on a
    3 x 3 tangential patch two cells deep (108 values), divides them by their RMS r, and a
    108 -> 64 -> 64 -> 6 GELU network returns the six field components of the ghost cell one
    step outside the face, divided by r; scaling by r keeps the model linear in the field
    amplitude as Maxwell's equations are;
  * the grid's edges wrap, and a boundary step replaces, in the updates of the outermost cells,
    the wrapped neighbour by the ghost (fdtd_lbc_fix). Every face predicts from the pre-step
    state E^n, H^{n+1/2}: side-0 faces the H^{n+1/2} ghosts that enter the E update, side-1
    faces the E^{n+1} ghosts that enter the H update. (Along a wave leaving the grid, the
    pre-step samples lie closest to the ghost: 0.21 cells from the nearest sample for the H
    ghost, 0.43 for the E ghost at dt = 0.99 / sqrt(3), against a full cell for the E ghost
    predicted after the E update.) Every other term of every update is the plain Yee update,
    so a step is exact whenever the ghosts are.
    The two cells of the stencil's depth form the 2-cell layer that replaces an 8-cell CPML.

Teacher data (``teacher_run``): a plain run with a 16-cell CPML on every face of a larger grid
(dielectric spheres inside, a Gaussian dipole pulse of random period and polarisation). Its
interior box is the thin-boundary grid: at sampled steps the box's boundary stencils and the
teacher's fields one cell outside the box are the training pairs (normalised by the
stencil's RMS). Only the ghost components a face's fix-up uses are weighted in the
loss (tangential H outside side-0 faces, tangential E outside side-1 faces).

Training (``BoundaryNet.fit``): float32 parameters, mean squared error, Adam, all on the GPU
through fdtd_mlp_forward / fdtd_mlp_backward / fdtd_adam. Inference uses bfloat16 weights on
the tensor cores with float32 accumulation (``precision='bf16'``; 'bf16x2' also splits the
activations into two bfloat16 parts; 'f32' runs float32 weights on the CUDA cores).

Evaluation and fallback (``reflection_db``, ``evaluate``, ``thin_or_cpml``): a run with the learned
boundary is compared with a plain CPML run of a grid twice as large in every learned
direction; the reflection is the largest error seen in the shell of cells next to the learned
faces relative to the largest field that reached that shell, and a long run checks that the
error does not grow (the boundary feeds its own output back every step). A boundary that is
worse than the threshold (-40 dB by default) or grows is replaced by CPML.

Memory term: a ghost is predicted as r * MLP(x) + memory * (the previous step's ghost). With
memory = (1 - c dt) / (1 + c dt) the form contains Mur's first-order absorbing condition
(``mur_map``), and training can shrink the fitted map towards Mur's (``fit_linear(prior='mur')``).

Measured behaviour: fitted on the full 108-value stencil, the ghost maps predict the ghosts to
about 10% RMS and, over the first pass of a pulse, leave an error some 30 dB below the same
2-cell layer without the network (zero ghosts), but in closed-loop feedback they grow after
250-500 steps; fitted on Mur's stencil only (``fit_linear(support='mur')``) the layer is
stable and beats Mur's own coefficients (-22 against -18 dB in the training band). None
reaches -40 dB, so the evaluation rejects them and the simulation falls back to CPML.

opencl_fdtd has no counterpart of this module: it absorbs with CPML only
(opencl_fdtd/simulation.py:274-319).
"""
from __future__ import annotations

import ctypes
import math

import numpy

from . import _lib

FACES_ALL = 63
PRECISIONS = {"f32": _lib.FDTD_LBC_F32, "bf16": _lib.FDTD_LBC_BF16, "bf16x2": _lib.FDTD_LBC_BF16X2,
              "linear": _lib.FDTD_LBC_LINEAR}
NPARAM = _lib.FDTD_LBC_NPARAM
IN, HID, OUT = _lib.FDTD_LBC_IN, _lib.FDTD_LBC_HID, _lib.FDTD_LBC_OUT
# offsets in the parameter vector (W1 b1 W2 b2 W3 b3, row-major [in][out])
W1, B1 = 0, IN * HID
W2 = B1 + HID
B2 = W2 + HID * HID
W3 = B2 + HID
B3 = W3 + HID * OUT
DEFAULT_DT = 0.99 / math.sqrt(3)


def _torch():
    import torch
    return torch


def _shape_arg(shape):
    return (ctypes.c_int32 * 3)(*(int(s) for s in shape))


def face_mask(faces=None) -> int:
    """Mask from face names ('-x', '+x', ...) or (axis, 'n'|'p') pairs; None: all six faces."""
    if faces is None:
        return FACES_ALL
    if isinstance(faces, int):
        return faces
    m = 0
    for f in faces:
        if isinstance(f, str):
            a, side = "xyz".index(f[1]), 0 if f[0] == "-" else 1
        else:
            a, side = "xyz".index(f[0]), 0 if f[1] == "n" else 1
        m |= 1 << (2 * a + side)
    return m


def columns(shape, mask: int = FACES_ALL):
    """(number of boundary columns, first column of each face f = 2 axis + side or -1, total)."""
    lib = _lib.load()
    n = ctypes.c_int32()
    off = (ctypes.c_int32 * 7)()
    _lib.check(lib.fdtd_lbc_columns(_shape_arg(shape), int(mask), ctypes.byref(n), off))
    return n.value, list(off)


def gather(shape, mask, E, H, X=None, R=None, C=None, stream=None):
    """Stencils of every column of a float32 state (flat E, H of 3N): X [ncol][108] normalised,
    R [ncol] the RMS, C [ncol][6] the outermost cell's components (device tensors)."""
    torch = _torch()
    ncol, _ = columns(shape, mask)
    dev = E.device
    X = torch.empty((ncol, IN), dtype=torch.float32, device=dev) if X is None else X
    R = torch.empty(ncol, dtype=torch.float32, device=dev) if R is None else R
    C = torch.empty((ncol, OUT), dtype=torch.float32, device=dev) if C is None else C
    st = stream or torch.cuda.current_stream(dev)
    _lib.check(_lib.load().fdtd_lbc_gather(_shape_arg(shape), int(mask), E.data_ptr(), H.data_ptr(),
                                           X.data_ptr(), R.data_ptr(), C.data_ptr(),
                                           ctypes.c_void_p(st.cuda_stream)))
    return X, R, C


def _levi_civita(q, a, p):
    return 1.0 if (q, a, p) in ((0, 1, 2), (1, 2, 0), (2, 0, 1)) else -1.0


def _stencil_index(a, depth, offsets, comp):
    """Input index of component ``comp`` at ``depth`` with tangential offsets {axis: -1|0|1}."""
    ua, va = [r for r in range(3) if r != a]
    return ((depth * 3 + offsets.get(ua, 0) + 1) * 3 + offsets.get(va, 0) + 1) * 6 + comp


def mur_map(face: int, dt: float = DEFAULT_DT, memory: float = None):
    """[109][6] linear map (rows: the 108 stencil inputs, then the bias) that, with the memory
    term m = (1 - c dt) / (1 + c dt), gives Mur's first-order absorbing condition (Mur 1981,
    IEEE Trans. EMC 23, one-way wave equation along the face normal, c = 1, unit cells) written
    for the ghost fields:
      side 0, H ghost:  G^{n+1/2} = m G^{n-1/2} + (1 - m) H_p(0)^{n+1/2} + dt (curl E^n)_p(0)
      side 1, E ghost:  G^{n+1}   = m G^n       + (1 - m) E_p(s-1)^n      - m dt (curl H^{n+1/2})_p(s-1)
    (H_p(0)^{n-1/2} and E_p(s-1)^{n+1}, which Mur's update needs, are the stencil's values
    stepped back / forward by the Yee update, hence the curl terms; curls with forward
    differences for E, backward for H, as the Yee updates take them). Being linear, the map is
    the same on the normalised stencil."""
    m = ((1.0 - dt) / (1.0 + dt)) if memory is None else memory
    a, side = divmod(int(face), 2)
    A = numpy.zeros((IN + 1, OUT))
    for p in range(3):
        if p == a:
            continue
        if side == 0:
            o = 3 + p
            A[_stencil_index(a, 0, {}, 3 + p), o] += 1.0 - m
            for a2 in range(3):
                for q2 in range(3):
                    if len({p, a2, q2}) < 3:
                        continue
                    e = _levi_civita(p, a2, q2)
                    plus = _stencil_index(a, 1, {}, q2) if a2 == a else _stencil_index(a, 0, {a2: 1}, q2)
                    A[plus, o] += dt * e
                    A[_stencil_index(a, 0, {}, q2), o] -= dt * e
        else:
            o = p
            A[_stencil_index(a, 0, {}, p), o] += 1.0 - m
            for a2 in range(3):
                for q2 in range(3):
                    if len({p, a2, q2}) < 3:
                        continue
                    e = _levi_civita(p, a2, q2)
                    minus = _stencil_index(a, 1, {}, 3 + q2) if a2 == a else _stencil_index(a, 0, {a2: -1}, 3 + q2)
                    A[_stencil_index(a, 0, {}, 3 + q2), o] -= m * dt * e
                    A[minus, o] += m * dt * e
    return A


# ---------------------------------------------------------------------------------------------
# the network and its training
# ---------------------------------------------------------------------------------------------
class BoundaryNet:
    """Six per-face networks (face f = 2 * axis + side): float32 parameters [6][NPARAM] on the
    device with their Adam moments."""

    def __init__(self, device=None, seed: int = 0, dt: float = DEFAULT_DT, memory: float = 0.0):
        torch = _torch()
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.dt = float(dt)
        # weight of the previous step's ghost in each prediction (the teacher data's targets
        # were formed with the same value)
        self.memory = float(memory)
        rng = numpy.random.default_rng(seed)
        P = numpy.zeros((6, NPARAM), numpy.float32)
        for f in range(6):
            # He-style initial weights; a small last layer so an untrained net changes little
            P[f, W1:B1] = rng.standard_normal(IN * HID) * math.sqrt(2.0 / IN)
            P[f, W2:B2] = rng.standard_normal(HID * HID) * math.sqrt(2.0 / HID)
            P[f, W3:B3] = rng.standard_normal(HID * OUT) * 0.01 * math.sqrt(1.0 / HID)
        self.params = torch.from_numpy(P).to(self.device)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.steps = [0] * 6
        self._packed = None
        self._bufs = {}
        self._wout = {}
        self.history = {}
        # the linear map of each face whose network is an exactly embedded linear map (None
        # once Adam has changed the parameters)
        self.linear = [None] * 6
        self._linear_dev = None

    # ---- kernels ---------------------------------------------------------------------------
    def _buffers(self, B):
        torch = _torch()
        if B not in self._bufs:
            ws = ctypes.c_int64()
            _lib.check(_lib.load().fdtd_mlp_backward_workspace(int(B), ctypes.byref(ws)))
            f32 = dict(dtype=torch.float32, device=self.device)
            self._bufs[B] = dict(Y=torch.empty((B, OUT), **f32), A1=torch.empty((B, HID), **f32),
                                 A2=torch.empty((B, HID), **f32), H1=torch.empty((B, HID), **f32),
                                 H2=torch.empty((B, HID), **f32), ws=torch.empty(ws.value, **f32),
                                 grad=torch.empty(NPARAM, **f32))
        return self._bufs[B]

    def _stream(self):
        return ctypes.c_void_p(_torch().cuda.current_stream(self.device).cuda_stream)

    def forward(self, face: int, X):
        """Network output [B][6] of face ``face`` for normalised stencils X [B][108]."""
        X = X.contiguous()
        B = X.shape[0]
        b = self._buffers(B)
        _lib.check(_lib.load().fdtd_mlp_forward(self.params[face].data_ptr(), X.data_ptr(), B, b["Y"].data_ptr(),
                                                b["A1"].data_ptr(), b["A2"].data_ptr(), b["H1"].data_ptr(),
                                                b["H2"].data_ptr(), self._stream()))
        return b["Y"]

    def output_weights(self, face: int):
        """Loss weights of the six outputs for ``face``: the ghost components its fix-up uses."""
        if face not in self._wout:
            torch = _torch()
            a, side = divmod(int(face), 2)
            w = [0.0] * 6
            for p in range(3):
                if p != a:
                    w[p if side == 1 else 3 + p] = 1.0
            self._wout[face] = torch.tensor(w, dtype=torch.float32, device=self.device)
        return self._wout[face]

    def gradient(self, face: int, X, T, weighted: bool = True):
        """(loss tensor, gradient [NPARAM]) of mean(w (net(X) - T)^2) for face ``face``, w the
        output weights (all 1 when ``weighted`` is False)."""
        X = X.contiguous()
        T = T.contiguous()
        B = X.shape[0]
        b = self._buffers(B)
        Y = self.forward(face, X)
        w = self.output_weights(face) if weighted else None
        _lib.check(_lib.load().fdtd_mlp_backward(self.params[face].data_ptr(), X.data_ptr(), Y.data_ptr(),
                                                 T.data_ptr(), w.data_ptr() if w is not None else None, B,
                                                 b["A1"].data_ptr(), b["A2"].data_ptr(), b["H1"].data_ptr(),
                                                 b["H2"].data_ptr(), b["grad"].data_ptr(), b["ws"].data_ptr(),
                                                 b["ws"].numel(), self._stream()))
        d = (Y - T) ** 2
        return (d * w).mean() if w is not None else d.mean(), b["grad"]

    def adam_step(self, face: int, grad, lr: float, betas=(0.9, 0.999), eps: float = 1e-8):
        self.steps[face] += 1
        self.linear[face] = None
        self._linear_dev = None
        _lib.check(_lib.load().fdtd_adam(self.params[face].data_ptr(), grad.data_ptr(), self.m[face].data_ptr(),
                                         self.v[face].data_ptr(), NPARAM, float(lr), float(betas[0]),
                                         float(betas[1]), float(eps), self.steps[face], self._stream()))
        self._packed = None

    def fit(self, data: "TeacherData", iters: int = 3000, batch: int = 4096, lr: float = 2e-3,
            lr_final: float = 2e-5, seed: int = 0, faces=range(6), log_every: int = 0,
            input_noise: float = 0.1):
        """Adam on random batches of each face's samples, learning rate decaying
        geometrically from lr to lr_final. Gaussian noise of standard deviation ``input_noise``
        (in the normalised units, where the stencil's RMS is 1) is added to every batch's
        inputs: the boundary feeds its own output back every step, and a map that amplifies
        patterns absent from the teacher data (first at the faces' edges) grows them into an
        instability; the noise keeps the map's gain on such patterns small, as ridge
        regression does for a linear map. Returns {face: final loss over the data}."""
        torch = _torch()
        gen = torch.Generator(device=self.device)
        gen.manual_seed(int(seed))
        out = {}
        for f in faces:
            X, T = data.X[f], data.T[f]
            n = X.shape[0]
            if n == 0:
                continue
            hist = []
            B = min(batch, n)
            for it in range(iters):
                rate = lr * (lr_final / lr) ** (it / max(iters - 1, 1))
                idx = torch.randint(0, n, (B,), device=self.device, generator=gen)
                xb = X[idx]
                if input_noise > 0:
                    xb = xb + input_noise * torch.randn(xb.shape, device=self.device, generator=gen)
                loss, g = self.gradient(f, xb, T[idx])
                self.adam_step(f, g, rate)
                if log_every and it % log_every == 0:
                    hist.append((it, float(loss)))
            self.history[f] = hist
            out[f] = self.loss(f, X, T)
        return out

    def gram(self, A, B, chunk: int = 1 << 20):
        """float64 host [(K + 1) x N]: A^T B and the column sums of B (fdtd_gram, float32 on the
        device per chunk of rows, chunks summed on the host in order)."""
        torch = _torch()
        A = A.contiguous()
        B = B.contiguous()
        rows, K = A.shape
        N = B.shape[1]
        out = numpy.zeros((K + 1, N))
        o = torch.empty((K + 1) * N, dtype=torch.float32, device=self.device)
        ws_n = ctypes.c_int64()
        _lib.check(_lib.load().fdtd_gram_workspace(min(rows, chunk), K, N, ctypes.byref(ws_n)))
        ws = torch.empty(max(ws_n.value, 1), dtype=torch.float32, device=self.device)
        for a in range(0, rows, chunk):
            n = min(chunk, rows - a)
            _lib.check(_lib.load().fdtd_gram(A[a:a + n].data_ptr(), n, K, B[a:a + n].data_ptr(), N, o.data_ptr(),
                                             ws.data_ptr(), ws.numel(), self._stream()))
            out += o.cpu().numpy().astype(numpy.float64).reshape(K + 1, N)
        return out

    def embed_linear(self, face: int, A, bias_shift: float = 10.0):
        """Put the [109][6] linear map A (rows: inputs, then bias) into the network exactly: six
        hidden units per layer with a bias shift that keeps GELU in its linear range
        (gelu(a) = a Phi(a), Phi(a) > 1 - 1e-6 for a > 4.8), the output bias removing the shift;
        every other unit at zero."""
        torch = _torch()
        P = numpy.zeros(NPARAM)
        P[W1:B1].reshape(IN, HID)[:, :OUT] = A[:IN]
        P[B1:B1 + OUT] = A[IN] + bias_shift
        for o in range(OUT):
            P[W2:B2].reshape(HID, HID)[o, o] = 1.0
            P[W3:B3].reshape(HID, OUT)[o, o] = 1.0
        P[B3:B3 + OUT] = -bias_shift
        self.params[face] = torch.from_numpy(P.astype(numpy.float32)).to(self.device)
        self.m[face].zero_()
        self.v[face].zero_()
        self.steps[face] = 0
        self._packed = None
        self.linear[face] = numpy.array(A, dtype=numpy.float64)
        self._linear_dev = None

    def fit_linear(self, data: "TeacherData", ridge: float = 1e-2, faces=range(6), prior: str = None,
                   support: str = None):
        """Start of training: the regularised least-squares linear map from the normalised
        stencils to the weighted targets, embedded exactly in the network (``embed_linear``).
        Normal equations from fdtd_gram on the device (X^T X in two column halves, X^T T),
        solved on the host in float64: minimise |X A - T|^2 + ridge n |A - A0|^2 over the n
        samples, A0 = 0 or, with prior='mur', Mur's first-order map (``mur_map``; the net's
        memory must be Mur's). Shrinking towards Mur, whose layer is stable in feedback, keeps
        the map stable for a large enough ridge; shrinking towards zero does not. ``support``
        limits each output to some inputs: 'mur' to the inputs Mur's map uses for it, 'mur3x3'
        to the components those inputs carry at every tangential position of both depths.
        Returns {face: loss}."""
        out = {}
        for f in faces:
            X, T = data.X[f], data.T[f]
            n = X.shape[0]
            if n == 0:
                continue
            h = IN // 2
            G = numpy.zeros((IN + 1, IN + 1))
            G[:, :h] = self.gram(X, X[:, :h])
            G[:, h:IN] = self.gram(X, X[:, h:])
            G[:IN, IN] = G[IN, :IN]
            G[IN, IN] = n
            XT = self.gram(X, T)
            A0 = mur_map(f, self.dt, self.memory) if prior == "mur" else numpy.zeros((IN + 1, OUT))
            R = numpy.zeros((IN + 1, IN + 1))
            R[numpy.arange(IN), numpy.arange(IN)] = ridge * n
            if support is None:
                A = numpy.linalg.solve(G + R, XT + R @ A0)
            else:
                Am = mur_map(f, self.dt, self.memory)
                A = numpy.zeros((IN + 1, OUT))
                for o in range(OUT):
                    rows = numpy.flatnonzero(Am[:IN, o])
                    if rows.size == 0:
                        continue
                    if support == "mur3x3":
                        comps = sorted(set(int(r) % 6 for r in rows))
                        rows = numpy.array([k for k in range(IN) if k % 6 in comps])
                    idx = numpy.append(rows, IN)                 # and the bias
                    Gs = (G + R)[numpy.ix_(idx, idx)]
                    A[idx, o] = numpy.linalg.solve(Gs, (XT + R @ A0)[idx, o])
            w = self.output_weights(f).cpu().numpy()
            A[:, w == 0] = 0.0
            self.embed_linear(f, A)
            out[f] = self.loss(f, X, T)
        return out

    def loss(self, face: int, X, T, chunk: int = 65536, weighted: bool = True) -> float:
        """Mean over samples x 6 of w (net(X) - T)^2 (the training loss)."""
        tot = 0.0
        n = X.shape[0]
        w = self.output_weights(face) if weighted else 1.0
        for a in range(0, n, chunk):
            Y = self.forward(face, X[a:a + chunk])
            tot += float((((Y - T[a:a + chunk]) ** 2) * w).sum())
        return tot / max(n * OUT, 1)

    # ---- inference weights -----------------------------------------------------------------
    def weights(self, precision: str = "bf16"):
        """Device weights for fdtd_lbc_predict / attach in ``precision`` ('linear': the linear
        maps of a network that is an exactly embedded linear map on every face)."""
        torch = _torch()
        if precision == "f32":
            return self.params
        if precision == "linear":
            if any(a is None for a in self.linear):
                raise ValueError("'linear' inference needs a linear map on every face (embed_linear / fit_linear, "
                                 "no Adam step since)")
            if self._linear_dev is None:
                self._linear_dev = torch.from_numpy(numpy.stack(self.linear).astype(numpy.float32)).to(self.device)
            return self._linear_dev
        if self._packed is None:
            packed = torch.empty((6, _lib.FDTD_LBC_PACK_WORDS), dtype=torch.int32, device=self.device)
            _lib.check(_lib.load().fdtd_lbc_pack(self.params.data_ptr(), packed.data_ptr(), self._stream()))
            self._packed = packed
        return self._packed

    def state_dict(self) -> dict:
        st = {"params": self.params.detach().cpu().numpy(), "dt": self.dt, "memory": self.memory}
        if all(a is not None for a in self.linear):
            st["linear"] = numpy.stack(self.linear)
        return st

    def load_state_dict(self, st: dict):
        torch = _torch()
        self.params.copy_(torch.as_tensor(numpy.asarray(st["params"], numpy.float32)).to(self.device))
        self.dt = float(st.get("dt", self.dt))
        self.memory = float(st.get("memory", self.memory))
        self._packed = None
        lin = st.get("linear")
        self.linear = [None] * 6 if lin is None else [numpy.asarray(a, numpy.float64) for a in lin]
        self._linear_dev = None

    def save(self, path):
        st = self.state_dict()
        extra = {"linear": st["linear"]} if "linear" in st else {}
        numpy.savez(path, params=st["params"], dt=numpy.float64(st["dt"]), memory=numpy.float64(st["memory"]),
                    **extra)

    @classmethod
    def load(cls, path, device=None):
        z = numpy.load(path)
        memory = float(z["memory"]) if "memory" in z.files else 0.0
        net = cls(device=device, dt=float(z["dt"]), memory=memory)
        net.load_state_dict({"params": z["params"], "dt": float(z["dt"]), "memory": memory,
                             "linear": z["linear"] if "linear" in z.files else None})
        return net


# ---------------------------------------------------------------------------------------------
# teacher data
# ---------------------------------------------------------------------------------------------
class TeacherData:
    """Training pairs per face: X [n][108] normalised stencils, T [n][6] normalised increments."""

    def __init__(self, device):
        self.device = device
        self._X = [[] for _ in range(6)]
        self._T = [[] for _ in range(6)]
        self._cat = None
        self.runs = 0

    def add(self, face, X, T):
        self._X[face].append(X)
        self._T[face].append(T)
        self._cat = None

    def _concat(self):
        torch = _torch()
        if self._cat is None:
            e = torch.empty((0, IN), dtype=torch.float32, device=self.device)
            eT = torch.empty((0, OUT), dtype=torch.float32, device=self.device)
            self._cat = ([torch.cat(x) if x else e for x in self._X], [torch.cat(t) if t else eT for t in self._T])
            self._X = [[x] if x.shape[0] else [] for x in self._cat[0]]
            self._T = [[t] if t.shape[0] else [] for t in self._cat[1]]
        return self._cat

    @property
    def X(self):
        return self._concat()[0]

    @property
    def T(self):
        return self._concat()[1]

    def sizes(self):
        return [int(x.shape[0]) for x in self.X]


def dipole_pulse(period: float, polarisation, delay_periods: float = 4.0, width_periods: float = 1.0):
    """Point-dipole waveform per component: sin(2 pi t / P) exp(-((t - t0) / s)^2 / 2) times the
    polarisation's components, s = width_periods * P, t0 = delay_periods * s."""
    s = width_periods * period
    t0 = delay_periods * s

    def f(t):
        return math.sin(2 * math.pi * t / period) * math.exp(-0.5 * ((t - t0) / s) ** 2)

    return [(lambda t, k=k: polarisation[k] * f(t)) for k in range(3)]


def _box(t, shape, pad):
    """Interior box [pad, s - pad) of a flat 3-component field, contiguous."""
    sx, sy, sz = shape
    v = t.view(3, sx, sy, sz)
    return v[:, pad[0]:sx - pad[0], pad[1]:sy - pad[1], pad[2]:sz - pad[2]].contiguous().view(-1)


def _ghost_plane(t, shape, pad, box, a, side):
    """[box_u * box_v][3]: a 3-component field on the plane one cell outside face (a, side) of the
    interior box, row-major over the other two axes (the face's column order)."""
    v = t.view(3, *shape)
    idx = [slice(p, p + b) for p, b in zip(pad, box)]
    idx[a] = pad[a] - 1 if side == 0 else pad[a] + box[a]
    return v[(slice(None),) + tuple(idx)].reshape(3, -1).t()


def _select(R, off, box, gen, per_face, keep):
    """Per face: the columns whose stencil RMS passes the threshold (at most per_face, random)."""
    torch = _torch()
    rmax = float(R.max())
    keep[0] = max(keep[0], rmax)
    out = {}
    if keep[0] <= 0:
        return out
    for f in range(6):
        a = f // 2
        ua, va = [r for r in range(3) if r != a]
        lo = off[f]
        sel = torch.nonzero(R[lo:lo + box[ua] * box[va]] > keep[1] * keep[0]).flatten()
        if sel.numel() == 0:
            continue
        if sel.numel() > per_face:
            sel = sel[torch.randperm(sel.numel(), device=sel.device, generator=gen)[:per_face]]
        out[f] = sel
    return out


def sphere_epsilon_inside(shape, n, seed, lo, hi, eps_range=(1.0, 12.0), r_range=(4.0, 24.0),
                          dtype=numpy.float32):
    """Isotropic eps: vacuum with n seeded dielectric spheres lying inside the box [lo, hi) of
    every axis (radius shrunk to fit where needed)."""
    rng = numpy.random.default_rng(seed)
    eps = numpy.ones(shape, dtype)
    x, y, z = (numpy.arange(s, dtype=numpy.float32) for s in shape)
    for _ in range(int(n)):
        r = rng.uniform(*r_range)
        r = min(r, 0.5 * min(h - l for l, h in zip(lo, hi)) - 1.0)
        if r <= 1.0:
            continue
        c = [rng.uniform(l + r, h - r) for l, h in zip(lo, hi)]
        e = rng.uniform(*eps_range)
        d2 = ((x - c[0]) ** 2)[:, None, None] + ((y - c[1]) ** 2)[None, :, None] + ((z - c[2]) ** 2)[None, None, :]
        eps[d2 < r * r] = e
    return [eps, eps.copy(), eps.copy()]


def teacher_run(data: TeacherData, seed: int, size: int = 128, cpml: int = 16, steps: int = 1500,
                every: int = 25, per_face: int = 512, dt: float = DEFAULT_DT, period_range=(10.0, 30.0),
                spheres=(1, 8), rel_threshold: float = 1e-3, face_margin: int = 4, memory: float = 0.0):
    """One plain run with a ``cpml``-cell CPML on every face of a size^3 grid; at every
    ``every``-th step adds training pairs of its interior box (size - 2 cpml)^3 to ``data``:
    stencils of the pre-step state E^n, H^{n+1/2}; targets the teacher's fields one cell outside
    the box, H^{n+1/2} outside the side-0 faces and E^{n+1} (after the step's sources) outside
    the side-1 faces. The dielectric spheres stay ``face_margin`` cells inside the box, so the
    learned faces see a homogeneous exterior. Columns whose stencil RMS is below
    ``rel_threshold`` times the largest seen so far in the run are skipped, at most ``per_face``
    random columns of a face are kept per sample. With ``memory`` m the targets are the ghosts
    minus m times the previous step's ghosts (the step before each sample is made by hand too).
    Returns the box shape."""
    torch = _torch()
    from .simulation import Simulation
    rng = numpy.random.default_rng(seed)
    shape = (size, size, size)
    pad = (cpml, cpml, cpml)
    box = tuple(s - 2 * q for s, q in zip(shape, pad))
    lo = [p + face_margin for p in pad]
    hi = [p + b - face_margin for p, b in zip(pad, box)]
    eps = sphere_epsilon_inside(shape, rng.integers(spheres[0], spheres[1] + 1), int(rng.integers(1 << 31)), lo, hi)
    pmls = [{"axis": a, "polarity": p, "thickness": cpml} for a in "xyz" for p in "np"]
    sim = Simulation(epsilon=eps, pmls=pmls, dt=dt, do_poynting=False)
    # source: a point dipole inside the box, at least 4 cells from its faces
    pos = tuple(int(rng.integers(cpml + 4, size - cpml - 4)) for _ in range(3))
    pol = rng.standard_normal(3)
    pol /= numpy.linalg.norm(pol)
    period = float(rng.uniform(*period_range))
    waves = dipole_pulse(period, pol)
    N = sim.N
    cell = int(numpy.ravel_multi_index(pos, shape))
    values = [[w(t) for t in range(steps)] for w in waves]
    gen = torch.Generator(device=sim.device)
    gen.manual_seed(int(seed))
    keep = [0.0, float(rel_threshold)]
    _, off = columns(box, FACES_ALL)
    lead = 2 if memory else 1
    t = 0
    while t < steps:
        n = min(every - lead, steps - t) if every > lead else 0
        if n > 0:
            sim.run(n, point_sources=[(k * N + cell, values[k][t:t + n]) for k in range(3)])
            t += n
        if t + lead > steps:
            break
        prev = {}
        if memory:
            # the step before the sample, by hand: its ghosts are the memory term's inputs
            for a in range(3):
                prev[2 * a] = _ghost_plane(sim.H, shape, pad, box, a, 0).clone()
            sim.update_E()
            for k in range(3):
                sim.E[k * N + cell] += numpy.float32(values[k][t])
            for a in range(3):
                prev[2 * a + 1] = _ghost_plane(sim.E, shape, pad, box, a, 1).clone()
            sim.update_H()
            sim.steps_run += 1
            t += 1
        # one step by hand: stencils before it, H ghosts now, E ghosts after the E update
        X, R, _ = gather(box, FACES_ALL, _box(sim.E, shape, pad), _box(sim.H, shape, pad))
        sel = _select(R, off, box, gen, per_face, keep)
        for f, idx in sel.items():
            if f % 2 == 0:
                g = _ghost_plane(sim.H, shape, pad, box, f // 2, 0)[idx]
                if memory:
                    g = g - memory * prev[f][idx]
                data.add(f, X[off[f] + idx], _six(g, "H") / R[off[f] + idx, None])
        sim.update_E()
        for k in range(3):
            sim.E[k * N + cell] += numpy.float32(values[k][t])
        for f, idx in sel.items():
            if f % 2 == 1:
                g = _ghost_plane(sim.E, shape, pad, box, f // 2, 1)[idx]
                if memory:
                    g = g - memory * prev[f][idx]
                data.add(f, X[off[f] + idx], _six(g, "E") / R[off[f] + idx, None])
        sim.update_H()
        sim.steps_run += 1
        t += 1
    data.runs += 1
    sim.close()
    return box


def _six(g, which):
    """[n][3] ghost components into the six-output layout (the other three zero)."""
    torch = _torch()
    z = torch.zeros_like(g)
    return torch.cat([g, z], 1) if which == "E" else torch.cat([z, g], 1)


def make_teacher_data(runs: int = 200, seed: int = 0, device=None, **kw) -> TeacherData:
    torch = _torch()
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    data = TeacherData(dev)
    for k in range(int(runs)):
        teacher_run(data, seed=seed * 100003 + k, **kw)
    return data


# ---------------------------------------------------------------------------------------------
# deployment
# ---------------------------------------------------------------------------------------------
class LearnedBoundary:
    """A trained BoundaryNet attached to Simulations: fdtd_run (Simulation.run) then steps
    them with the learned boundary on the faces in ``faces``."""

    def __init__(self, net: BoundaryNet, precision: str = "bf16", faces=None):
        if precision not in PRECISIONS:
            raise ValueError("precision must be one of %s" % sorted(PRECISIONS))
        self.net = net
        self.precision = precision
        self.mask = face_mask(faces)
        self._attached = {}
        self._pred = {}

    def _check(self, sim):
        if numpy.dtype(sim.arg_type) != numpy.float32:
            raise ValueError("the learned boundary needs float32 fields")
        if sim.bloch_boundaries:
            raise ValueError("the learned boundary does not combine with Bloch boundaries")
        if abs(sim.dt - self.net.dt) > 1e-12 * max(1.0, abs(sim.dt)):
            raise ValueError("the network was trained for dt = %r, the simulation has dt = %r" % (self.net.dt, sim.dt))
        for p in sim.pmls:
            bit = 1 << (2 * "xyz".index(p["axis"]) + (0 if p["polarity"] == "n" else 1))
            if self.mask & bit:
                raise ValueError("face %s%s has a CPML and the learned boundary" % (p["polarity"], p["axis"]))

    def attach(self, sim):
        """Step ``sim`` with the learned boundary from its next run() on."""
        torch = _torch()
        self._check(sim)
        ncol, _ = columns(sim.shape, self.mask)
        pred = torch.zeros(max(ncol, 1) * OUT, dtype=torch.float32, device=sim.device)
        W = self.net.weights(self.precision)
        _lib.check(sim._lib.fdtd_lbc_attach(sim._plan, self.mask, PRECISIONS[self.precision], self.net.memory,
                                            W.data_ptr(),
                                            pred.data_ptr(), pred.numel()))
        self._attached[id(sim)] = (sim, pred, W)
        # the plan keeps raw pointers to W and pred: the simulation holds them (and this
        # boundary) until detach, whatever happens to the caller's references
        sim._lbc_keep = (self, pred, W)
        return sim

    def detach(self, sim):
        _lib.check(sim._lib.fdtd_lbc_attach(sim._plan, 0, 0, 0.0, None, None, 0))
        self._attached.pop(id(sim), None)
        sim._lbc_keep = None

    def predict(self, sim, side: int = -1, pred=None, stream=None):
        """Ghost values [ncol][6] of the faces of ``side`` (-1: all) from sim's current state
        (for stepping with update_E / update_H). With a memory term the previous ghosts are
        read from ``pred`` (default: a buffer kept per simulation, zero at first)."""
        torch = _torch()
        ncol, _ = columns(sim.shape, self.mask)
        if pred is None:
            pred = self._pred.get(id(sim))
            if pred is None or pred.shape[0] != ncol:
                pred = torch.zeros((ncol, OUT), dtype=torch.float32, device=sim.device)
                self._pred[id(sim)] = pred
        st = stream or sim.queue
        W = self.net.weights(self.precision)
        _lib.check(sim._lib.fdtd_lbc_predict(_shape_arg(sim.shape), self.mask, int(side), PRECISIONS[self.precision],
                                             self.net.memory, W.data_ptr(), sim.E.data_ptr(), sim.H.data_ptr(),
                                             pred.data_ptr(), pred.numel(), ctypes.c_void_p(st.cuda_stream)))
        outside = self._outside_rows(sim)
        if outside is not None:
            with torch.cuda.stream(st):
                pred[outside] = 0.0
        return pred

    def _outside_rows(self, sim):
        """Rows of the columns that lie inside the simulation's CPML faces (fdtd_run gives them
        zero ghosts; the plan-free predict call does not know the CPML), or None."""
        torch = _torch()
        key = ("rows", id(sim))
        if key in self._pred:
            return self._pred[key]
        lo, hi = [0, 0, 0], [0, 0, 0]
        for pml in sim.pmls:
            a = "xyz".index(pml["axis"])
            if pml["polarity"] == "n":
                lo[a] = int(pml["thickness"])
            else:
                hi[a] = int(pml["thickness"])
        rows = None
        if any(lo) or any(hi):
            _, off = columns(sim.shape, self.mask)
            sel = []
            for f in range(6):
                if off[f] < 0:
                    continue
                a = f // 2
                ua, va = [r for r in range(3) if r != a]
                u = torch.arange(sim.shape[ua]).view(-1, 1).expand(sim.shape[ua], sim.shape[va])
                v = torch.arange(sim.shape[va]).view(1, -1).expand(sim.shape[ua], sim.shape[va])
                out = (u < lo[ua]) | (u >= sim.shape[ua] - hi[ua]) | (v < lo[va]) | (v >= sim.shape[va] - hi[va])
                sel.append(torch.nonzero(out.flatten()).flatten() + off[f])
            rows = torch.cat(sel).to(sim.device) if sel else None
            if rows is not None and rows.numel() == 0:
                rows = None
        self._pred[key] = rows
        return rows

    def fix(self, sim, pred, fields: str, stream=None):
        """The fix-up of the outermost cells' updates: 'E' right after update_E, 'H' after
        update_H."""
        st = stream or sim.queue
        sim._buffers()                      # dt / eps (and dt / mu) up to date
        if fields not in ("E", "H"):
            raise ValueError("fields must be 'E' or 'H'")
        f = _lib.FDTD_LBC_FIX_E if fields == "E" else _lib.FDTD_LBC_FIX_H
        cm = sim._cm if sim.mu is not None else None
        _lib.check(sim._lib.fdtd_lbc_fix(_shape_arg(sim.shape), self.mask, f, pred.data_ptr(), sim.E.data_ptr(),
                                         sim.H.data_ptr(), sim._ce.data_ptr(),
                                         cm.data_ptr() if cm is not None else None, float(sim.dt),
                                         ctypes.c_void_p(st.cuda_stream)))

    def step(self, sim, point_sources=None):
        """One step through the reference-style per-update entry points: the ghosts of every
        face from the pre-step state, update_E, E fix-up, the soft sources (flat index, value),
        update_H, H fix-up."""
        pred = self.predict(sim)
        sim.update_E()
        self.fix(sim, pred, "E")
        for idx, val in point_sources or ():
            sim.E.view(-1)[int(idx)] += numpy.float32(val)
        sim.update_H()
        self.fix(sim, pred, "H")


def reflection_db(boundary: LearnedBoundary, shape=(64, 64, 64), steps: int = 400, every: int = 10,
                  period: float = 20.0, polarisation=(0.3, 1.0, 0.2), epsilon=None, cpml: int = 16,
                  source=None, shell: int = 8, cpml_other: int = 0):
    """Reflection of a boundary in dB: the same dipole pulse in (a) ``shape`` with the boundary
    on the faces of its mask and (b) a plain run on a grid twice as large in every learned
    direction (``shape`` centred) with a ``cpml``-cell CPML. Over samples every ``every`` steps,
    in the L2 norm over the shell of cells within ``shell`` cells of the learned faces,
    20 log10(max_t |E_a - E_b| / max_t |E_b|): the wave sent back by the boundary against the
    wave that reached it. epsilon: the small grid's [3] arrays (the large grid extends them by
    edge replication); default vacuum. boundary None: no boundary treatment at all (the grid's
    edges wrap), on every face. cpml_other > 0: the faces without the learned layer carry a
    CPML of that thickness in both grids (as a deployment that mixes the two would), instead of
    wrapping. Also returns the same ratio over the whole grid and the series [(step, shell
    error, shell reference)]."""
    torch = _torch()
    from .simulation import Simulation
    mask = boundary.mask if boundary is not None else FACES_ALL
    pad = [0, 0, 0]
    for a in range(3):
        if mask & (3 << (2 * a)):
            pad[a] = shape[a] // 2
    if epsilon is None:
        epsilon = [numpy.ones(shape, numpy.float32) for _ in range(3)]
    big_shape = tuple(s + 2 * p for s, p in zip(shape, pad))
    big_eps = [numpy.pad(numpy.asarray(e, numpy.float32), [(p, p) for p in pad], mode="edge") for e in epsilon]
    pol = numpy.asarray(polarisation, numpy.float64)
    pol = pol / numpy.linalg.norm(pol)
    waves = dipole_pulse(period, pol)
    src = tuple(s // 2 for s in shape) if source is None else tuple(source)
    dt = boundary.net.dt if boundary is not None else DEFAULT_DT
    other = [{"axis": "xyz"[a], "polarity": p, "thickness": cpml_other}
             for a in range(3) for side, p in ((0, "n"), (1, "p"))
             if cpml_other > 0 and not mask & (1 << (2 * a + side))]
    small = Simulation(epsilon=[numpy.asarray(e, numpy.float32) for e in epsilon], pmls=[dict(o) for o in other],
                       dt=dt, do_poynting=False)
    big_pmls = [{"axis": "xyz"[a], "polarity": p, "thickness": cpml} for a in range(3) if pad[a] for p in "np"]
    big_pmls += [dict(o) for o in other if not pad["xyz".index(o["axis"])]]
    big = Simulation(epsilon=big_eps, pmls=big_pmls, dt=dt, do_poynting=False)
    if boundary is not None:
        boundary.attach(small)
    cs = int(numpy.ravel_multi_index(src, shape))
    cb = int(numpy.ravel_multi_index(tuple(c + p for c, p in zip(src, pad)), big_shape))
    vals = [[w(t) for t in range(steps)] for w in waves]
    # shell mask over the small grid
    m = torch.zeros(shape, dtype=torch.bool, device=small.device)
    for a in range(3):
        for side in range(2):
            if mask & (1 << (2 * a + side)):
                idx = [slice(None)] * 3
                idx[a] = slice(0, shell) if side == 0 else slice(shape[a] - shell, shape[a])
                m[tuple(idx)] = True
    err_max = ref_max = all_err = all_ref = 0.0
    series = []
    t = 0
    while t < steps:
        n = min(every, steps - t)
        small.run(n, point_sources=[(k * small.N + cs, vals[k][t:t + n]) for k in range(3)])
        big.run(n, point_sources=[(k * big.N + cb, vals[k][t:t + n]) for k in range(3)])
        t += n
        Es = small.E.view(3, *shape)
        Eb = big.E.view(3, *big_shape)[:, pad[0]:pad[0] + shape[0], pad[1]:pad[1] + shape[1],
                                       pad[2]:pad[2] + shape[2]]
        d = (Es - Eb).double()
        e = float(torch.linalg.vector_norm(d[:, m]))
        r = float(torch.linalg.vector_norm(Eb.double()[:, m]))
        ea = float(torch.linalg.vector_norm(d))
        ra = float(torch.linalg.vector_norm(Eb.double()))
        if not math.isfinite(e):
            e = ea = float("inf")
        err_max, ref_max = max(err_max, e), max(ref_max, r)
        all_err, all_ref = max(all_err, ea), max(all_ref, ra)
        series.append((t, e, r))
    if boundary is not None:
        boundary.detach(small)
    small.close()
    big.close()

    def db(e, r):
        if not r > 0:
            return math.nan
        return 20 * math.log10(e / r) if e > 0 else -math.inf

    return {"reflection_db": db(err_max, ref_max), "grid_db": db(all_err, all_ref), "series": series,
            "shape": tuple(shape), "big_shape": big_shape}


def evaluate(boundary: LearnedBoundary, shape=(96, 96, 96), steps: int = 400, periods=(20.0, 68.0),
             stability_shape=(64, 64, 64), stability_steps: int = 3000, threshold_db: float = -40.0,
             growth_db: float = 0.0, cpml_other: int = 0):
    """The boundary's verdict: the worst reflection (``reflection_db`` over ``steps`` steps, one
    run per pulse period) and a long run (``stability_steps``) whose shell error, relative to the
    largest field that reached the shell, must stay at most ``growth_db`` at its end (a boundary
    that feeds back its own errors grows them without bound). Accepted when both hold and the
    reflection is at most ``threshold_db``. ``cpml_other``: see ``reflection_db``."""
    refl = {}
    for per in periods:
        refl[per] = reflection_db(boundary, shape=shape, steps=steps, every=10, period=per,
                                  cpml_other=cpml_other)["reflection_db"]
    long = reflection_db(boundary, shape=stability_shape, steps=stability_steps, every=50, period=periods[0],
                         cpml_other=cpml_other)
    ref = max(r for _, _, r in long["series"]) or 1.0
    t_end, e_end, _ = long["series"][-1]
    end_db = 20 * math.log10(e_end / ref) if e_end > 0 and math.isfinite(e_end) else (math.inf if e_end else -math.inf)
    onset = next((t for t, e, _ in long["series"] if not math.isfinite(e) or e > ref), None)
    worst = max(refl.values())
    stable = end_db <= growth_db
    return {"reflection_db": worst, "reflection_by_period": refl, "stable": stable,
            "final_error_db": end_db, "growth_onset_step": onset, "stability_steps": stability_steps,
            "accepted": bool(stable and math.isfinite(worst) and worst <= threshold_db)}


def thin_or_cpml(kwargs: dict, boundary: LearnedBoundary, reflection_db_value: float = None, threshold_db: float = -40.0,
                 cpml_thickness: int = 8, verdict: dict = None):
    """A Simulation for ``kwargs`` (constructor arguments without CPML on the boundary's faces):
    with the learned boundary attached when it passed (``verdict['accepted']`` from ``evaluate``,
    or ``reflection_db_value`` at most ``threshold_db`` when no verdict is given), else with a
    ``cpml_thickness``-cell CPML on those faces instead. Returns (sim, 'learned' | 'cpml')."""
    from .simulation import Simulation
    kw = dict(kwargs)
    if verdict is not None:
        ok = bool(verdict.get("accepted"))
    else:
        ok = reflection_db_value is not None and math.isfinite(reflection_db_value) and reflection_db_value <= threshold_db
    if ok:
        sim = Simulation(**kw)
        boundary.attach(sim)
        return sim, "learned"
    pmls = list(kw.get("pmls", []))
    for a in range(3):
        for side, pol in ((0, "n"), (1, "p")):
            if boundary.mask & (1 << (2 * a + side)):
                pmls.append({"axis": "xyz"[a], "polarity": pol, "thickness": cpml_thickness})
    kw["pmls"] = pmls
    return Simulation(**kw), "cpml"


MUR_MEMORY = (1.0 - DEFAULT_DT) / (1.0 + DEFAULT_DT)   # -(c dt - dx) / (c dt + dx), vacuum, unit cells


def train(runs: int = 200, seed: int = 0, ridge: float = 1.0, finetune_iters: int = 0,
          finetune_lr: float = 1e-4, input_noise: float = 0.1, device=None, memory: float = None,
          prior: str = "mur", data=None, **teacher_kw):
    """The training pipeline: ``runs`` teacher runs (``teacher_run``, targets formed with the
    memory term, Mur's by default), the regularised least-squares start shrunk towards
    ``prior`` (``BoundaryNet.fit_linear``) and an optional Adam fine-tune with input noise
    (``BoundaryNet.fit``). Returns (net, data, {face: loss after the start},
    {face: loss after the fine-tune})."""
    memory = MUR_MEMORY if memory is None else memory
    if data is None:
        data = make_teacher_data(runs=runs, seed=seed, device=device, memory=memory, **teacher_kw)
    net = BoundaryNet(device=device, seed=seed + 1, memory=memory)
    start = net.fit_linear(data, ridge=ridge, prior=prior)
    fin = net.fit(data, iters=finetune_iters, batch=4096, lr=finetune_lr, lr_final=finetune_lr * 1e-2,
                  input_noise=input_noise) if finetune_iters > 0 else dict(start)
    return net, data, start, fin
