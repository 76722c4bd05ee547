"""
CPU oracle of the learned thin absorbing boundary (float64 numpy). Test infrastructure only:
the tests import it to check the CUDA kernels of opencl_fdtd_gb300/csrc/lbc.cu; nothing in the
package calls it.

The reference (opencl_fdtd) absorbs outgoing waves only with CPML (simulation.py:274-319,
kernels/update_e.cl / update_h.cl psi terms); the learned boundary has no counterpart there,
so this oracle is pinned by mathematics instead of reference outputs: the backward pass is
checked against central finite differences of the forward pass, the column layout against a
direct enumeration of the faces' cells, and the fix-up against the Yee step of a larger grid
(with the exact ghosts, a boundary step of the interior box equals the larger grid's step
there; the Yee step is the oracle port of the reference kernels, oracle/port.py).

Definitions restated here (the CUDA side follows the same ones):
  * faces f = 2 * axis + side (side 0: index 0, side 1: index s - 1), visited in that order;
    a face's prediction columns span its whole plane (the two other axes, u, v in xyz order);
    the fix-up visits every outer cell once (``owned_faces``) and adds every face's term;
  * the stencil of column (u, v): depth d in {0, 1} (cells s_a - 1 - d on side 1), tangential
    offsets du, dv in {-1, 0, 1} clamped to the grid, components Ex Ey Ez Hx Hy Hz; flat index
    ((d * 3 + du + 1) * 3 + dv + 1) * 6 + component;
  * r = RMS of the 108 values, x = stencil / r (x = 0 where r = 0);
  * MLP: a1 = x W1 + b1, h1 = gelu(a1), a2 = h1 W2 + b2, h2 = gelu(a2), y = h2 W3 + b3,
    gelu(a) = a Phi(a) (exact, erf form), parameters packed W1 b1 W2 b2 W3 b3 row-major
    [in][out];
  * prediction: the six components of the ghost cell one step outside the face, r * y, at the
    stencil's time level; ``fix`` puts them into the Yee updates of the outermost cells in place
    of the wrapped neighbours of a grid whose edges wrap.
"""
from __future__ import annotations

import numpy
from scipy.special import erf

IN, HID, OUT = 108, 64, 6
W1 = 0
B1 = W1 + IN * HID
W2 = B1 + HID
B2 = W2 + HID * HID
W3 = B2 + HID
B3 = W3 + HID * OUT
NPARAM = B3 + OUT


def _other(a):
    return (1, 2) if a == 0 else ((0, 2) if a == 1 else (0, 1))


def faces(shape, face_mask):
    """Prediction columns: [(axis, side, u0, nu, v0, nv, col0)] covering each learned face's whole
    plane (u, v: the other axes in xyz order, row-major), and the total column count."""
    out = []
    ncol = 0
    for a in range(3):
        for side in range(2):
            if not face_mask & (1 << (2 * a + side)):
                continue
            ua, va = _other(a)
            out.append((a, side, 0, shape[ua], 0, shape[va], ncol))
            ncol += shape[ua] * shape[va]
    return out, ncol


def owned_faces(shape, face_mask):
    """The same planes with the rows of earlier faces (x, y, z; side 0 first) removed: every
    outer cell once."""
    owned = [[False, False] for _ in range(3)]
    out = []
    ncol = 0
    for a in range(3):
        for side in range(2):
            if not face_mask & (1 << (2 * a + side)):
                continue
            ua, va = _other(a)
            u0, u1, v0, v1 = 0, shape[ua], 0, shape[va]
            if owned[ua][0]:
                u0 = 1
            if owned[ua][1]:
                u1 -= 1
            if owned[va][0]:
                v0 = 1
            if owned[va][1]:
                v1 -= 1
            nu, nv = max(u1 - u0, 0), max(v1 - v0, 0)
            out.append((a, side, u0, nu, v0, nv, ncol))
            ncol += nu * nv
            owned[a][side] = True
    return out, ncol


def _cells_of(shape, fl, ncol):
    cells = numpy.empty(ncol, numpy.int64)
    face_of = numpy.empty(ncol, numpy.int64)
    for a, side, u0, nu, v0, nv, col0 in fl:
        ua, va = _other(a)
        u, v = numpy.meshgrid(numpy.arange(u0, u0 + nu), numpy.arange(v0, v0 + nv), indexing="ij")
        c = [None, None, None]
        c[a] = numpy.full(u.shape, shape[a] - 1 if side else 0)
        c[ua], c[va] = u, v
        cells[col0:col0 + nu * nv] = numpy.ravel_multi_index(c, shape).ravel()
        face_of[col0:col0 + nu * nv] = 2 * a + side
    return cells, face_of


def column_cells(shape, face_mask):
    """Flat cell index of every prediction column's depth-0 centre, and its face number."""
    fl, ncol = faces(shape, face_mask)
    return _cells_of(shape, fl, ncol)


def owned_cells(shape, face_mask):
    fl, ncol = owned_faces(shape, face_mask)
    return _cells_of(shape, fl, ncol)


def stencil_cells(shape, face_mask):
    """[ncol][18] flat cell indices of the stencil cells, order (d, du, dv)."""
    fl, ncol = faces(shape, face_mask)
    out = numpy.empty((ncol, 18), numpy.int64)
    for a, side, u0, nu, v0, nv, col0 in fl:
        ua, va = _other(a)
        u, v = numpy.meshgrid(numpy.arange(u0, u0 + nu), numpy.arange(v0, v0 + nv), indexing="ij")
        u, v = u.ravel(), v.ravel()
        k = 0
        for d in range(2):
            for du in (-1, 0, 1):
                for dv in (-1, 0, 1):
                    c = [None, None, None]
                    c[a] = numpy.full(u.shape, shape[a] - 1 - d if side else d)
                    c[ua] = numpy.clip(u + du, 0, shape[ua] - 1)
                    c[va] = numpy.clip(v + dv, 0, shape[va] - 1)
                    out[col0:col0 + nu * nv, k] = numpy.ravel_multi_index(c, shape)
                    k += 1
    return out


def gather(shape, face_mask, E, H):
    """X [ncol][108] (stencil / r), R [ncol], C [ncol][6] (depth-0 centre components)."""
    N = int(numpy.prod(shape))
    E = numpy.asarray(E, numpy.float64).reshape(3, N)
    H = numpy.asarray(H, numpy.float64).reshape(3, N)
    idx = stencil_cells(shape, face_mask)
    vals = numpy.concatenate([E[:, idx], H[:, idx]], axis=0)     # [6][ncol][18]
    raw = vals.transpose(1, 2, 0).reshape(idx.shape[0], IN)       # [ncol][(cell, comp)]
    R = numpy.sqrt((raw * raw).mean(axis=1))
    inv = numpy.where(R > 0, 1.0 / numpy.where(R > 0, R, 1.0), 0.0)
    X = raw * inv[:, None]
    C = raw[:, 24:30].copy()
    return X, R, C


def gelu(a):
    return 0.5 * a * (1.0 + erf(a / numpy.sqrt(2.0)))


def gelu_d(a):
    return 0.5 * (1.0 + erf(a / numpy.sqrt(2.0))) + a * numpy.exp(-0.5 * a * a) / numpy.sqrt(2.0 * numpy.pi)


def unpack(P):
    P = numpy.asarray(P, numpy.float64)
    return (P[W1:B1].reshape(IN, HID), P[B1:W2], P[W2:B2].reshape(HID, HID), P[B2:W3],
            P[W3:B3].reshape(HID, OUT), P[B3:NPARAM])


def forward(P, X):
    w1, b1, w2, b2, w3, b3 = unpack(P)
    X = numpy.asarray(X, numpy.float64)
    a1 = X @ w1 + b1
    h1 = gelu(a1)
    a2 = h1 @ w2 + b2
    h2 = gelu(a2)
    y = h2 @ w3 + b3
    return y, (X, a1, h1, a2, h2)


def loss(P, X, T, w=None):
    """mean over batch x 6 of w_o (Y - T)^2 (w = 1 when None)."""
    y, _ = forward(P, X)
    w = numpy.ones(OUT) if w is None else numpy.asarray(w, numpy.float64)
    return float((w * (y - T) ** 2).mean())


def backward(P, X, T, w=None):
    """Gradient of ``loss`` with respect to the parameter vector."""
    w1, b1, w2, b2, w3, b3 = unpack(P)
    y, (X, a1, h1, a2, h2) = forward(P, X)
    B = X.shape[0]
    w = numpy.ones(OUT) if w is None else numpy.asarray(w, numpy.float64)
    dy = 2.0 * w * (y - numpy.asarray(T, numpy.float64)) / (B * OUT)
    d2 = (dy @ w3.T) * gelu_d(a2)
    d1 = (d2 @ w2.T) * gelu_d(a1)
    g = numpy.zeros(NPARAM)
    g[W1:B1] = (X.T @ d1).ravel()
    g[B1:W2] = d1.sum(0)
    g[W2:B2] = (h1.T @ d2).ravel()
    g[B2:W3] = d2.sum(0)
    g[W3:B3] = (h2.T @ dy).ravel()
    g[B3:NPARAM] = dy.sum(0)
    return g


def adam(P, G, M, V, lr, b1, b2, eps, step):
    """One bias-corrected Adam step (Kingma and Ba 2015); returns new (P, M, V)."""
    M = b1 * M + (1 - b1) * G
    V = b2 * V + (1 - b2) * G * G
    P = P - lr * (M / (1 - b1 ** step)) / (numpy.sqrt(V / (1 - b2 ** step)) + eps)
    return P, M, V


def predict(shape, face_mask, params, E, H, side=None):
    """[ncol][6] ghost values r * net(x) of the faces (of one side when ``side`` is 0 or 1;
    other rows are zero); params [6][NPARAM] (face 2 * axis + side)."""
    X, R, C = gather(shape, face_mask, E, H)
    _, face_of = column_cells(shape, face_mask)
    out = numpy.zeros_like(C)
    for f in numpy.unique(face_of):
        if side is not None and f % 2 != side:
            continue
        sel = face_of == f
        y, _ = forward(numpy.asarray(params)[f], X[sel])
        out[sel] = y * R[sel, None]
    return out


def levi_civita(q, a, p):
    return 1.0 if (q, a, p) in ((0, 1, 2), (1, 2, 0), (2, 0, 1)) else -1.0


def fix(shape, face_mask, fields, pred, E, H, ce, ch):
    """The fix-up of the updates of the outermost cells, in place on flat E, H ([3N]): for every
    learned face (a, side) and every cell c of its plane, component q != a, p the third axis,
      side 0, 'E' in fields: E_q(c) += -e_qap ce_q(c) (ghost H_p - H_p(c with index s_a - 1)),
      side 1, 'H' in fields: H_q(c) += -e_qap ch_q(c) (ghost E_p - E_p(c with index 0)),
    ghost = pred[column of c in the face] (components Ex Ey Ez Hx Hy Hz). This is what the Yee
    update (E_q += ce sum e_qap d_a H_p with backward differences, H_q -= ch sum e_qap d_a E_p
    with forward differences, unit cells) gives when the neighbour across the face is the
    ghost instead of the wrapped cell. ce, ch: [3N] arrays or scalars."""
    N = int(numpy.prod(shape))
    st = (shape[1] * shape[2], shape[2], 1)
    fl, _ = faces(shape, face_mask)
    ce = numpy.broadcast_to(numpy.asarray(ce, numpy.float64), (3 * N,))
    ch = numpy.broadcast_to(numpy.asarray(ch, numpy.float64), (3 * N,))
    dE = numpy.zeros(3 * N)
    dH = numpy.zeros(3 * N)
    for a, side, u0, nu, v0, nv, col0 in fl:
        cells, _ = _cells_of(shape, [(a, side, u0, nu, v0, nv, 0)], nu * nv)
        g = pred[col0:col0 + nu * nv]
        wrapped = cells + (shape[a] - 1) * st[a] if side == 0 else cells - (shape[a] - 1) * st[a]
        for q in range(3):
            if q == a:
                continue
            p = 3 - a - q
            e = levi_civita(q, a, p)
            if side == 0 and "E" in fields:
                numpy.add.at(dE, q * N + cells, -e * (g[:, 3 + p] - H[p * N + wrapped]))
            if side == 1 and "H" in fields:
                numpy.add.at(dH, q * N + cells, -e * (g[:, p] - E[p * N + wrapped]))
    if "E" in fields:
        E += ce * dE
    if "H" in fields:
        H += ch * dH
