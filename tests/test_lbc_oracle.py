"""The learned-boundary oracle (oracle/lbc.py) on the CPU: its backward pass against central
finite differences of its forward pass, its column layout against a direct enumeration of the
grid's outer cells, its gather against per-column loops, its fix-up against the Yee step of a
larger grid (the oracle port of the reference kernels), and Adam against the closed form of
the first step."""
import itertools

import numpy
import pytest

from oracle import lbc


def _params(seed, scale=0.3):
    rng = numpy.random.default_rng(seed)
    P = rng.standard_normal(lbc.NPARAM) * scale
    return P


def test_layout_sizes():
    assert lbc.NPARAM == 108 * 64 + 64 + 64 * 64 + 64 + 64 * 6 + 6 == 11526


def test_backward_matches_finite_differences():
    rng = numpy.random.default_rng(1)
    P = _params(2, 0.2)
    X = rng.standard_normal((7, lbc.IN))
    T = rng.standard_normal((7, lbc.OUT))
    g = lbc.backward(P, X, T)
    # a sample of parameters from every block, plus every bias of the last layer
    idx = list(rng.choice(lbc.B1, 12, replace=False)) + list(range(lbc.B1, lbc.B1 + 3)) + \
        list(rng.choice(numpy.arange(lbc.W2, lbc.B2), 8, replace=False)) + [lbc.B2 + 5] + \
        list(rng.choice(numpy.arange(lbc.W3, lbc.B3), 6, replace=False)) + list(range(lbc.B3, lbc.NPARAM))
    h = 1e-6
    for i in idx:
        Pp, Pm = P.copy(), P.copy()
        Pp[i] += h
        Pm[i] -= h
        fd = (lbc.loss(Pp, X, T) - lbc.loss(Pm, X, T)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])


def test_weighted_backward_matches_finite_differences():
    rng = numpy.random.default_rng(6)
    P = _params(7, 0.2)
    X = rng.standard_normal((5, lbc.IN))
    T = rng.standard_normal((5, lbc.OUT))
    w = numpy.array([0.0, 1.0, 0.5, 0.0, 2.0, 1.0])
    g = lbc.backward(P, X, T, w)
    h = 1e-6
    for i in list(rng.choice(lbc.NPARAM, 20, replace=False)) + list(range(lbc.B3, lbc.NPARAM)):
        Pp, Pm = P.copy(), P.copy()
        Pp[i] += h
        Pm[i] -= h
        fd = (lbc.loss(Pp, X, T, w) - lbc.loss(Pm, X, T, w)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])
    assert g[lbc.B3] == 0.0 and g[lbc.B3 + 3] == 0.0


def test_gelu_derivative():
    a = numpy.linspace(-6, 6, 101)
    h = 1e-6
    fd = (lbc.gelu(a + h) - lbc.gelu(a - h)) / (2 * h)
    assert numpy.max(numpy.abs(fd - lbc.gelu_d(a))) < 1e-8


@pytest.mark.parametrize("shape,mask", [((5, 4, 3), 63), ((6, 5, 4), 0b110011), ((4, 4, 4), 0b001100),
                                        ((3, 7, 2), 63)])
def test_columns_cover_each_outer_cell_once(shape, mask):
    cells, face_of = lbc.owned_cells(shape, mask)
    assert len(numpy.unique(cells)) == len(cells)
    want = set()
    for c in itertools.product(*(range(s) for s in shape)):
        for a in range(3):
            for side in range(2):
                if mask & (1 << (2 * a + side)) and c[a] == (shape[a] - 1 if side else 0):
                    want.add(numpy.ravel_multi_index(c, shape))
    assert set(cells.tolist()) == want
    # each cell is owned by the first face (x before y before z, side 0 before side 1)
    for cell, f in zip(cells, face_of):
        c = numpy.unravel_index(cell, shape)
        first = min(2 * a + s for a in range(3) for s in range(2)
                    if mask & (1 << (2 * a + s)) and c[a] == (shape[a] - 1 if s else 0))
        assert f == first
    # prediction columns: every face's whole plane, row-major over its two other axes
    pc, pf = lbc.column_cells(shape, mask)
    for f in range(6):
        a, side = divmod(f, 2)
        if not mask & (1 << f):
            assert not (pf == f).any()
            continue
        ua, va = [r for r in range(3) if r != a]
        want = []
        for u in range(shape[ua]):
            for v in range(shape[va]):
                c = [0, 0, 0]
                c[a] = shape[a] - 1 if side else 0
                c[ua], c[va] = u, v
                want.append(numpy.ravel_multi_index(c, shape))
        assert pc[pf == f].tolist() == want


def test_gather_against_loops():
    shape = (4, 5, 3)
    N = numpy.prod(shape)
    rng = numpy.random.default_rng(3)
    E = rng.standard_normal(3 * N)
    H = rng.standard_normal(3 * N)
    X, R, C = lbc.gather(shape, 63, E, H)
    fl, ncol = lbc.faces(shape, 63)
    assert X.shape == (ncol, 108)
    for a, side, u0, nu, v0, nv, col0 in fl:
        ua, va = (1, 2) if a == 0 else ((0, 2) if a == 1 else (0, 1))
        for j in range(nu * nv):
            u, v = u0 + j // nv, v0 + j % nv
            raw = []
            for d in range(2):
                for du in (-1, 0, 1):
                    for dv in (-1, 0, 1):
                        c = [0, 0, 0]
                        c[a] = shape[a] - 1 - d if side else d
                        c[ua] = min(max(u + du, 0), shape[ua] - 1)
                        c[va] = min(max(v + dv, 0), shape[va] - 1)
                        i = numpy.ravel_multi_index(c, shape)
                        raw += [E[q * N + i] for q in range(3)] + [H[q * N + i] for q in range(3)]
            raw = numpy.array(raw)
            r = numpy.sqrt(numpy.mean(raw ** 2))
            numpy.testing.assert_allclose(R[col0 + j], r, rtol=1e-14)
            numpy.testing.assert_allclose(X[col0 + j], raw / r, rtol=1e-13)
            numpy.testing.assert_array_equal(C[col0 + j], raw[24:30])


def _ghosts(big, pad, shape, mask):
    """[ncol][6] with the big grid's E and H one cell outside each face of the interior box."""
    sb = big.shape
    N = int(numpy.prod(sb))
    fl, ncol = lbc.faces(shape, mask)
    out = numpy.zeros((ncol, 6))
    for a, side, u0, nu, v0, nv, col0 in fl:
        ua, va = [r for r in range(3) if r != a]
        u, v = numpy.meshgrid(numpy.arange(nu), numpy.arange(nv), indexing="ij")
        idx = [None, None, None]
        idx[a] = numpy.full((nu, nv), pad[a] - 1 if side == 0 else pad[a] + shape[a])
        idx[ua], idx[va] = u + pad[ua], v + pad[va]
        cells = numpy.ravel_multi_index(idx, sb).ravel()
        for q in range(3):
            out[col0:col0 + nu * nv, q] = big.E[q * N + cells]
            out[col0:col0 + nu * nv, 3 + q] = big.H[q * N + cells]
    return out


def _box(arr, sb, pad, shape):
    v = arr.reshape(3, *sb)
    return v[:, pad[0]:pad[0] + shape[0], pad[1]:pad[1] + shape[1], pad[2]:pad[2] + shape[2]].reshape(-1).copy()


@pytest.mark.parametrize("mask", [63, 0b000011, 0b001100, 0b110000, 0b001111, 0b110011])
def test_fix_with_exact_ghosts_reproduces_the_larger_grid(mask):
    """A grid's interior box stepped on its own (edges wrapping) with the fix-up fed the larger
    grid's values just outside it equals the larger grid's step inside the box. Axes without a
    learned face are not padded, and wrap in both grids."""
    from oracle.port import PortSimulation
    shape = (7, 6, 5)
    pad = [2 if mask & (3 << (2 * a)) else 0 for a in range(3)]
    sb = tuple(s + 2 * p for s, p in zip(shape, pad))
    box = tuple(slice(p, p + s) for p, s in zip(pad, shape))
    rng = numpy.random.default_rng(mask)
    eps_b = [rng.uniform(1, 5, sb) for _ in range(3)]
    init = {k: [rng.standard_normal(sb) for _ in range(3)] for k in "EH"}
    dt = 0.5
    kw = dict(dt=dt, float_type=numpy.float64, do_poynting=False)
    big = PortSimulation(eps_b, [], initial_fields=init, **kw)
    eps_s = [e[box] for e in eps_b]
    init_s = {k: [x[box] for x in v] for k, v in init.items()}
    small = PortSimulation(eps_s, [], initial_fields=init_s, **kw)
    plain = PortSimulation(eps_s, [], initial_fields=init_s, **kw)
    ce = numpy.concatenate([dt / e.ravel() for e in eps_s])
    for _ in range(3):
        gh0 = _ghosts(big, pad, shape, mask)            # H^{n+1/2} outside the side-0 faces
        small.update_E()
        lbc.fix(shape, mask, "E", gh0, small.E, small.H, ce, dt)
        big.update_E()
        gh1 = _ghosts(big, pad, shape, mask)            # E^{n+1} outside the side-1 faces
        small.update_H()
        lbc.fix(shape, mask, "H", gh1, small.E, small.H, ce, dt)
        big.update_H()
        plain.step()
        numpy.testing.assert_allclose(small.E, _box(big.E, sb, pad, shape), rtol=0, atol=1e-12)
        numpy.testing.assert_allclose(small.H, _box(big.H, sb, pad, shape), rtol=0, atol=1e-12)
    # without the fix-up the box differs (the wrapped neighbours are wrong)
    assert not numpy.allclose(plain.E, small.E)


def test_prediction_is_homogeneous_in_the_fields():
    """r * f(x / r): scaling every field by a scales the predicted ghosts by a."""
    shape = (4, 4, 4)
    rng = numpy.random.default_rng(5)
    E = rng.standard_normal(3 * 64)
    H = rng.standard_normal(3 * 64)
    P = rng.standard_normal((6, lbc.NPARAM)) * 0.1
    d1 = lbc.predict(shape, 63, P, E, H)
    d2 = lbc.predict(shape, 63, P, 3.5 * E, 3.5 * H)
    numpy.testing.assert_allclose(d2, 3.5 * d1, rtol=1e-12, atol=1e-12)


def test_adam_first_step_is_lr_times_sign():
    P = numpy.array([1.0, -2.0, 0.5])
    G = numpy.array([0.3, -4.0, 0.0])
    P1, M, V = lbc.adam(P, G, numpy.zeros(3), numpy.zeros(3), 0.01, 0.9, 0.999, 1e-12, 1)
    numpy.testing.assert_allclose(P1, P - 0.01 * numpy.sign(G), atol=1e-9)


def _mur_1d_run(direction, comp, steps):
    """A Gaussian plane-wave pulse along x starting at the centre of a 60-cell box with Mur's map
    (memory form) on both x faces, against the same pulse in a 240-cell grid; float64 oracle
    port and oracle fix-up. Returns the max error over the box per step and the box's fields."""
    from oracle.port import PortSimulation
    from opencl_fdtd_gb300.learned_boundary import mur_map, MUR_MEMORY
    dt = 0.99 / numpy.sqrt(3)
    sb, pad, box = (240, 1, 1), 90, (60, 1, 1)
    x = numpy.arange(sb[0], dtype=numpy.float64)
    x0 = 120.0
    q, a = comp, 0
    p = 3 - a - q
    s = lbc.levi_civita(q, a, p)
    E = [numpy.zeros(sb) for _ in range(3)]
    H = [numpy.zeros(sb) for _ in range(3)]
    E[q][:, 0, 0] = numpy.exp(-0.5 * ((x - x0) / 4.0) ** 2)
    xh = x + 0.5 + direction * 0.5 * dt
    H[p][:, 0, 0] = (s if direction < 0 else -s) * numpy.exp(-0.5 * ((xh - x0) / 4.0) ** 2)
    kw = dict(dt=dt, float_type=numpy.float64, do_poynting=False)
    big = PortSimulation([numpy.ones(sb)] * 3, [], initial_fields={"E": E, "H": H}, **kw)
    sl = (slice(pad, pad + box[0]), slice(None), slice(None))
    small = PortSimulation([numpy.ones(box)] * 3, [], initial_fields={"E": [e[sl] for e in E],
                                                                      "H": [h[sl] for h in H]}, **kw)
    mask = 0b000011
    fl, ncol = lbc.faces(box, mask)
    A = {f: mur_map(f) for f in (0, 1)}
    ghost = numpy.zeros((ncol, 6))
    err = []
    for _ in range(steps):
        X, R, _ = lbc.gather(box, mask, small.E, small.H)
        new = numpy.zeros_like(ghost)
        for a_, side, u0, nu, v0, nv, col0 in fl:
            rows = slice(col0, col0 + nu * nv)
            f = 2 * a_ + side
            new[rows] = (X[rows] @ A[f][:108] + A[f][108]) * R[rows, None]
        ghost = new + MUR_MEMORY * ghost
        small.update_E()
        lbc.fix(box, mask, "E", ghost, small.E, small.H, dt, dt)
        small.update_H()
        lbc.fix(box, mask, "H", ghost, small.E, small.H, dt, dt)
        big.step()
        Eb = big.E.reshape(3, *sb)[:, pad:pad + box[0]]
        err.append(numpy.abs(small.E.reshape(3, *box) - Eb).max())
    return numpy.array(err), small


@pytest.mark.parametrize("direction,comp", [(-1, 1), (1, 2)])
def test_mur_map_absorbs_a_plane_wave_and_stays_stable(direction, comp):
    """Mur's first-order map in the memory form, in closed loop: a normally incident pulse
    (peak 1, 9.4 cells FWHM) leaves the box with an error below 1% of its peak against the
    larger grid (before that grid's own wrapped pulse returns), and 1000 further steps leave no
    growing field in the box."""
    err, _ = _mur_1d_run(direction, comp, 160)
    assert err.max() < 0.01, err.max()
    _, small = _mur_1d_run(direction, comp, 1200)
    assert numpy.abs(small.E).max() < 1e-3
