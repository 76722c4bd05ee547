"""Learned thin boundary on the GPU: the column layout, stencil gather, MLP forward, backward
and Adam kernels against the float64 CPU oracle (oracle/lbc.py); the tensor-core inference
against the float32 one; the boundary step of fdtd_run against the same step made by hand; a
short training run that lowers the loss and absorbs better than the thin layer without the
network; and the CPML fallback."""
import copy
import ctypes
import math

import numpy
import pytest

torch = pytest.importorskip("torch")

from oracle import lbc as O  # noqa: E402

pytestmark = pytest.mark.gpu


def _L():
    from opencl_fdtd_gb300 import learned_boundary
    return learned_boundary


def _fields(shape, seed, scale=1.0):
    rng = numpy.random.default_rng(seed)
    N = int(numpy.prod(shape))
    E = (scale * rng.standard_normal(3 * N)).astype(numpy.float32)
    H = (scale * rng.standard_normal(3 * N)).astype(numpy.float32)
    return E, H


def _cuda(a):
    return torch.from_numpy(numpy.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("shape,mask", [((12, 9, 7), 63), ((10, 6, 5), 0b110011), ((5, 8, 3), 0b001100),
                                        ((3, 4, 2), 63)])
def test_columns_and_gather_match_oracle(shape, mask):
    L = _L()
    fl, ncol = O.faces(shape, mask)
    n, off = L.columns(shape, mask)
    assert n == ncol
    for a, side, u0, nu, v0, nv, col0 in fl:
        assert off[2 * a + side] == col0
    E, H = _fields(shape, 1)
    X, R, C = L.gather(shape, mask, _cuda(E), _cuda(H))
    Xo, Ro, Co = O.gather(shape, mask, E, H)
    numpy.testing.assert_allclose(R.cpu().numpy(), Ro, rtol=1e-5)
    numpy.testing.assert_allclose(X.cpu().numpy(), Xo, rtol=1e-5, atol=1e-6)
    numpy.testing.assert_array_equal(C.cpu().numpy(), Co.astype(numpy.float32))


def _net(seed=0, scale_last=1.0):
    L = _L()
    net = L.BoundaryNet(seed=seed)
    if scale_last != 1.0:
        net.params[:, L.W3:L.B3] *= scale_last
    net.params[:, L.B1:L.W2] = 0.05
    net.params[:, L.B3:] = 0.01
    return net


def test_forward_matches_oracle():
    net = _net(1, 100.0)
    rng = numpy.random.default_rng(2)
    X = rng.standard_normal((300, 108)).astype(numpy.float32)
    for f in (0, 5):
        Y = net.forward(f, _cuda(X)).cpu().numpy()
        Yo, _ = O.forward(net.params[f].cpu().numpy().astype(numpy.float64), X)
        assert numpy.max(numpy.abs(Y - Yo)) <= 1e-5 * max(1.0, numpy.max(numpy.abs(Yo)))


@pytest.mark.parametrize("B", [1, 37, 256, 1000])
def test_backward_matches_oracle_and_is_deterministic(B):
    net = _net(3, 100.0)
    rng = numpy.random.default_rng(B)
    X = rng.standard_normal((B, 108)).astype(numpy.float32)
    T = rng.standard_normal((B, 6)).astype(numpy.float32)
    loss, g = net.gradient(2, _cuda(X), _cuda(T))
    g1 = g.clone()
    P = net.params[2].cpu().numpy().astype(numpy.float64)
    w = net.output_weights(2).cpu().numpy().astype(numpy.float64)
    go = O.backward(P, X, T, w)
    scale = numpy.max(numpy.abs(go))
    err = numpy.abs(g1.cpu().numpy() - go)
    assert numpy.max(err) <= 1e-5 * scale, (numpy.max(err), scale)
    # per block of parameters too (small blocks would hide behind a large global scale)
    for a, b in ((O.W1, O.B1), (O.B1, O.W2), (O.W2, O.B2), (O.B2, O.W3), (O.W3, O.B3), (O.B3, O.NPARAM)):
        s = max(numpy.max(numpy.abs(go[a:b])), 1e-30)
        assert numpy.max(err[a:b]) <= 1e-4 * s + 1e-6 * scale
    assert abs(float(loss) - O.loss(P, X, T, w)) <= 1e-5 * O.loss(P, X, T, w)
    _, g2 = net.gradient(2, _cuda(X), _cuda(T))
    assert torch.equal(g1, g2)
    # unweighted
    _, g3 = net.gradient(2, _cuda(X), _cuda(T), weighted=False)
    go3 = O.backward(P, X, T)
    assert numpy.max(numpy.abs(g3.cpu().numpy() - go3)) <= 1e-5 * numpy.max(numpy.abs(go3))


def test_adam_matches_oracle():
    net = _net(4)
    rng = numpy.random.default_rng(5)
    P0 = net.params[1].cpu().numpy().astype(numpy.float64)
    M = numpy.zeros(O.NPARAM)
    V = numpy.zeros(O.NPARAM)
    P = P0.copy()
    for step in range(1, 4):
        G = rng.standard_normal(O.NPARAM).astype(numpy.float32)
        net.adam_step(1, _cuda(G), 1e-3)
        P, M, V = O.adam(P, G.astype(numpy.float64), M, V, 1e-3, 0.9, 0.999, 1e-8, step)
    numpy.testing.assert_allclose(net.params[1].cpu().numpy(), P, rtol=0, atol=1e-6)
    # the other faces are untouched
    assert net.steps == [0, 3, 0, 0, 0, 0]


def _predict(L, shape, mask, precision, W, E, H, side=-1, memory=0.0, prev=None):
    n, _ = L.columns(shape, mask)
    pred = torch.zeros((n, 6), dtype=torch.float32, device="cuda") if prev is None else _cuda(prev)
    lib = L._lib.load()
    L._lib.check(lib.fdtd_lbc_predict(L._shape_arg(shape), mask, side, L.PRECISIONS[precision], memory,
                                      W.data_ptr(), E.data_ptr(), H.data_ptr(), pred.data_ptr(), pred.numel(),
                                      ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
    return pred.cpu().numpy()


@pytest.mark.parametrize("shape,mask,side", [((14, 11, 9), 63, -1), ((40, 3, 17), 0b101010, -1),
                                             ((6, 70, 5), 63, 0), ((9, 8, 7), 0b110110, 1)])
def test_predict_f32_matches_oracle(shape, mask, side):
    L = _L()
    net = _net(6, 300.0)
    E, H = _fields(shape, 7, 0.01)
    pred = _predict(L, shape, mask, "f32", net.params, _cuda(E), _cuda(H), side)
    po = O.predict(shape, mask, net.params.cpu().numpy().astype(numpy.float64), E, H,
                   None if side < 0 else side)
    assert numpy.max(numpy.abs(po)) > 0
    assert numpy.max(numpy.abs(pred - po)) <= 2e-5 * numpy.max(numpy.abs(po))


@pytest.mark.parametrize("shape", [(14, 11, 9), (33, 20, 17), (5, 130, 6)])
def test_predict_tensor_cores_match_float32(shape):
    """bfloat16 weights on the tensor cores against the same (bfloat16-rounded) weights in
    float32 on the CUDA cores: the activations' rounding is the only difference."""
    L = _L()
    net = _net(8, 300.0)
    net.params.copy_(net.params.to(torch.bfloat16).to(torch.float32))
    net._packed = None
    E, H = _fields(shape, 9, 0.02)
    Ed, Hd = _cuda(E), _cuda(H)
    p32 = _predict(L, shape, 63, "f32", net.params, Ed, Hd)
    scale = numpy.max(numpy.abs(p32))
    assert scale > 0
    for prec, tol in (("bf16", 3e-2), ("bf16x2", 2e-4)):
        p = _predict(L, shape, 63, prec, net.weights(prec), Ed, Hd)
        err = numpy.max(numpy.abs(p - p32)) / scale
        assert err <= tol, (prec, err)
        # side filter: the other side's rows stay untouched (zero)
        p0 = _predict(L, shape, 63, prec, net.weights(prec), Ed, Hd, side=0)
        _, face_of = O.column_cells(shape, 63)
        assert not p0[face_of % 2 == 1].any()
        numpy.testing.assert_array_equal(p0[face_of % 2 == 0], p[face_of % 2 == 0])


@pytest.mark.parametrize("precision", ["f32", "bf16", "bf16x2"])
def test_predict_memory_term(precision):
    """pred = r * net + memory * (previous pred), rows of the other side untouched."""
    L = _L()
    shape = (10, 9, 8)
    net = _net(40, 200.0)
    net.params.copy_(net.params.to(torch.bfloat16).to(torch.float32))
    net._packed = None
    E, H = _fields(shape, 41, 0.05)
    Ed, Hd = _cuda(E), _cuda(H)
    W = net.weights(precision)
    n, _ = L.columns(shape)
    prev = numpy.random.default_rng(42).standard_normal((n, 6)).astype(numpy.float32)
    p0 = _predict(L, shape, 63, precision, W, Ed, Hd)
    p1 = _predict(L, shape, 63, precision, W, Ed, Hd, memory=0.27, prev=prev)
    numpy.testing.assert_allclose(p1, p0 + numpy.float32(0.27) * prev, rtol=1e-5, atol=1e-6)
    _, face_of = O.column_cells(shape, 63)
    p2 = _predict(L, shape, 63, precision, W, Ed, Hd, side=1, memory=0.5, prev=prev)
    numpy.testing.assert_array_equal(p2[face_of % 2 == 0], prev[face_of % 2 == 0])


@pytest.mark.parametrize("mask,fields", [(63, "E"), (63, "H"), (0b011011, "H"), (0b110100, "E")])
def test_fix_matches_oracle(mask, fields):
    L = _L()
    shape = (9, 7, 6)
    N = int(numpy.prod(shape))
    E, H = _fields(shape, 10)
    rng = numpy.random.default_rng(11)
    ce = rng.uniform(0.1, 0.6, 3 * N).astype(numpy.float32)
    cm = rng.uniform(0.1, 0.6, 3 * N).astype(numpy.float32)
    n, _ = L.columns(shape, mask)
    pred = rng.standard_normal((n, 6)).astype(numpy.float32)
    pred_d, ce_d, cm_d = _cuda(pred), _cuda(ce), _cuda(cm)
    for with_mu in (False, True):
        Ed, Hd = _cuda(E), _cuda(H)
        lib = L._lib.load()
        f = 1 if fields == "E" else 2
        L._lib.check(lib.fdtd_lbc_fix(L._shape_arg(shape), mask, f, pred_d.data_ptr(), Ed.data_ptr(),
                                      Hd.data_ptr(), ce_d.data_ptr(), cm_d.data_ptr() if with_mu else None, 0.5,
                                      ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
        Eo, Ho = E.astype(numpy.float64), H.astype(numpy.float64)
        O.fix(shape, mask, fields, pred.astype(numpy.float64), Eo, Ho, ce.astype(numpy.float64),
              cm.astype(numpy.float64) if with_mu else 0.5)
        numpy.testing.assert_allclose(Ed.cpu().numpy(), Eo, rtol=1e-6, atol=1e-6)
        numpy.testing.assert_allclose(Hd.cpu().numpy(), Ho, rtol=1e-6, atol=1e-6)
        if "E" in fields:
            assert not numpy.array_equal(Ed.cpu().numpy(), E)


def test_exact_ghosts_reproduce_the_larger_grid():
    """The teacher's ghost planes fed through the fix-up: a box stepped on its own equals the
    larger grid (with CPML beyond the box) inside the box, to float32 rounding."""
    from opencl_fdtd_gb300 import Simulation
    L = _L()
    sb, pad = (20, 18, 16), (4, 4, 4)
    box = tuple(s - 2 * p for s, p in zip(sb, pad))
    rng = numpy.random.default_rng(20)
    eps = [rng.uniform(1, 4, sb).astype(numpy.float32) for _ in range(3)]
    init = {k: [0.1 * rng.standard_normal(sb).astype(numpy.float32) for _ in range(3)] for k in "EH"}
    dt = 0.99 / math.sqrt(3)
    big = Simulation(epsilon=eps, pmls=[{"axis": a, "polarity": p, "thickness": 4} for a in "xyz" for p in "np"],
                     initial_fields=init, dt=dt, do_poynting=False)
    sl = tuple(slice(p, p + b) for p, b in zip(pad, box))
    small = Simulation(epsilon=[e[sl].copy() for e in eps], pmls=[], dt=dt, do_poynting=False,
                       initial_fields={k: [x[sl].copy() for x in v] for k, v in init.items()})
    lb = L.LearnedBoundary(_net(21), "f32")
    n, off = L.columns(box)
    pred = torch.zeros((n, 6), dtype=torch.float32, device="cuda")

    def ghosts(side):
        for a in range(3):
            f = 2 * a + side
            g = torch.cat([L._ghost_plane(big.E, sb, pad, box, a, side),
                           L._ghost_plane(big.H, sb, pad, box, a, side)], dim=1)
            pred[off[f]:off[f] + g.shape[0]] = g

    for _ in range(4):
        ghosts(0)
        small.update_E()
        lb.fix(small, pred, "E")
        big.update_E()
        ghosts(1)
        small.update_H()
        lb.fix(small, pred, "H")
        big.update_H()
    torch.cuda.synchronize()
    for name in ("E", "H"):
        want = getattr(big, name).view(3, *sb)[(slice(None),) + sl].reshape(-1)
        got = getattr(small, name)
        assert torch.max(torch.abs(got - want)).item() <= 2e-6


def _sim_kwargs(shape, seed, poynting=False):
    rng = numpy.random.default_rng(seed)
    eps = [rng.uniform(1, 4, shape).astype(numpy.float32) for _ in range(3)]
    init = {k: [0.1 * rng.standard_normal(shape).astype(numpy.float32) for _ in range(3)] for k in "EH"}
    return dict(epsilon=eps, pmls=[], initial_fields=init, do_poynting=poynting,
                dt=0.99 / math.sqrt(3))


@pytest.mark.parametrize("precision,memory", [("f32", 0.0), ("bf16", 0.27), ("bf16x2", 0.0)])
def test_run_with_boundary_equals_manual_steps(precision, memory):
    from opencl_fdtd_gb300 import Simulation
    L = _L()
    shape = (16, 12, 10)
    net = _net(11, 50.0)
    net.memory = memory
    lb = L.LearnedBoundary(net, precision)
    a = Simulation(**_sim_kwargs(shape, 12))
    b = Simulation(**_sim_kwargs(shape, 12))
    src = int(numpy.ravel_multi_index((8, 6, 5), shape)) + a.N
    vals = [0.3 * math.sin(0.4 * t) for t in range(6)]
    lb.attach(a)
    a.run(6, point_sources=[(src, vals)])
    for t in range(6):
        lb.step(b, point_sources=[(src, vals[t])])
    torch.cuda.synchronize()
    assert torch.equal(a.E, b.E) and torch.equal(a.H, b.H)
    # the outermost cells did change from the plain step's values
    c = Simulation(**_sim_kwargs(shape, 12))
    c.run(6, point_sources=[(src, vals)])
    assert not torch.equal(a.E, c.E)


def test_run_with_cpml_on_other_faces_equals_manual_steps():
    """A learned layer on the z faces with CPML on x and y: fdtd_run (zero ghosts for the
    columns inside the CPML) and the hand-made steps agree bit for bit."""
    from opencl_fdtd_gb300 import Simulation
    L = _L()
    shape = (16, 14, 12)
    net = _net(17, 50.0)
    lb = L.LearnedBoundary(net, "f32", faces=["-z", "+z"])
    kw = _sim_kwargs(shape, 18)
    kw["pmls"] = [{"axis": a, "polarity": p, "thickness": 3} for a in "xy" for p in "np"]
    a = Simulation(**copy.deepcopy(kw))
    b = Simulation(**copy.deepcopy(kw))
    lb.attach(a)
    a.run(5)
    for _ in range(5):
        lb.step(b)
    torch.cuda.synchronize()
    assert torch.equal(a.E, b.E) and torch.equal(a.H, b.H)


def test_boundary_on_the_hs_path_matches_plain_path():
    from opencl_fdtd_gb300 import Simulation
    L = _L()
    shape = (18, 10, 12)
    lb = L.LearnedBoundary(_net(13, 50.0), "bf16")
    a = Simulation(**_sim_kwargs(shape, 14, poynting=True))
    b = Simulation(**_sim_kwargs(shape, 14, poynting=True))
    lb.attach(a)
    lb.attach(b)
    a.run(5, path="hs")
    b.run(5, path="plain")
    torch.cuda.synchronize()
    assert torch.equal(a.E, b.E) and torch.equal(a.H, b.H)


def test_attach_rejections():
    from opencl_fdtd_gb300 import Simulation
    L = _L()
    lb = L.LearnedBoundary(_net(15), "bf16", faces=["-x", "+x"])
    kw = _sim_kwargs((8, 8, 8), 16)
    kw["pmls"] = [{"axis": "x", "polarity": "p", "thickness": 2}]
    with pytest.raises(ValueError):
        lb.attach(Simulation(**kw))
    kw = _sim_kwargs((8, 8, 8), 16)
    kw["dt"] = 0.3
    with pytest.raises(ValueError):
        lb.attach(Simulation(**kw))
    kw = _sim_kwargs((8, 8, 8), 16)
    kw["float_type"] = numpy.float64
    kw["epsilon"] = [e.astype(numpy.float64) for e in kw["epsilon"]]
    kw["initial_fields"] = {k: [x.astype(numpy.float64) for x in v] for k, v in kw["initial_fields"].items()}
    with pytest.raises(ValueError):
        lb.attach(Simulation(**kw))
    with pytest.raises(ValueError):
        L.LearnedBoundary(_net(15), "fp8")


@pytest.fixture(scope="module")
def small_training():
    """Teacher data from 4 plain runs at 40^3 with an 8-cell CPML (24^3 interior boxes), the
    ridge least-squares start and a short Adam fine-tune: what the full-size pipeline does,
    small enough for a test."""
    L = _L()
    data = L.make_teacher_data(runs=4, seed=1, size=40, cpml=8, steps=260, every=5, per_face=256,
                               period_range=(10.0, 20.0), spheres=(1, 2), face_margin=2)
    net = L.BoundaryNet(seed=2)
    before = {f: net.loss(f, data.X[f], data.T[f]) for f in range(6)}
    start = net.fit_linear(data, ridge=1e-2)
    after = net.fit(data, iters=200, batch=1024, lr=1e-4, lr_final=1e-6, input_noise=0.1)
    return L, data, net, before, start, after


def test_gram_matches_numpy():
    L = _L()
    net = _net(30)
    rng = numpy.random.default_rng(31)
    A = rng.standard_normal((3000, 108)).astype(numpy.float32)
    B = rng.standard_normal((3000, 54)).astype(numpy.float32)
    g = net.gram(_cuda(A), _cuda(B), chunk=1024)
    want = numpy.vstack([A.astype(numpy.float64).T @ B, B.sum(0, dtype=numpy.float64)[None, :]])
    assert numpy.max(numpy.abs(g - want)) <= 1e-3 * numpy.max(numpy.abs(want))


def test_linear_start_is_the_least_squares_map(small_training):
    """The embedded linear map reproduces the ridge least-squares solution solved in float64
    on the host from the same data (the GELU units stay in their linear range)."""
    L, data, net, before, start, after = small_training
    f = 1
    X = data.X[f].double().cpu().numpy()
    T = data.T[f].double().cpu().numpy()
    X1 = numpy.hstack([X, numpy.ones((X.shape[0], 1))])
    G = X1.T @ X1
    G[numpy.arange(108), numpy.arange(108)] += 1e-2 * X.shape[0]
    A = numpy.linalg.solve(G, X1.T @ T)
    lin = L.BoundaryNet(seed=2)
    lin.fit_linear(data, ridge=1e-2, faces=[f])
    Y = lin.forward(f, data.X[f][:500]).double().cpu().numpy()
    w = lin.output_weights(f).cpu().numpy() > 0
    Yl = X1[:500] @ A
    assert numpy.max(numpy.abs(Y[:, w] - Yl[:, w])) <= 1e-3 * numpy.max(numpy.abs(Yl[:, w]))


def test_training_lowers_the_loss(small_training):
    L, data, net, before, start, after = small_training
    assert min(data.sizes()) > 1000
    for f in range(6):
        assert start[f] < 0.05 * before[f], (f, before[f], start[f])
        assert after[f] <= 1.1 * start[f], (f, start[f], after[f])


def test_trained_network_absorbs_better_than_the_layer_without_it(small_training):
    """First pass of a pulse against a plain run on a doubled grid with CPML: the trained
    network's 2-cell layer against the same layer whose network predicts zero ghosts, and
    against no layer at all (the grid's wrapped edges)."""
    L, data, net, before, start, after = small_training
    kw = dict(shape=(24, 24, 24), steps=60, every=4, period=14.0, cpml=8, shell=4)
    trained = L.reflection_db(L.LearnedBoundary(net, "bf16x2"), **kw)["reflection_db"]
    zero = L.BoundaryNet(seed=3)
    zero.params.zero_()
    held = L.reflection_db(L.LearnedBoundary(zero, "bf16x2"), **kw)["reflection_db"]
    wrapped = L.reflection_db(None, **kw)["reflection_db"]
    assert trained < held - 10.0, (trained, held)
    assert trained < wrapped - 10.0, (trained, wrapped)


@pytest.fixture(scope="module")
def mur_training():
    """Teacher data with Mur's memory term (4 runs at 40^3, 24^3 boxes) and the least-squares
    map on Mur's stencil."""
    L = _L()
    data = L.make_teacher_data(runs=4, seed=3, size=40, cpml=8, steps=260, every=5, per_face=256,
                               period_range=(10.0, 20.0), spheres=(1, 2), face_margin=2, memory=L.MUR_MEMORY)
    net = L.BoundaryNet(seed=4, memory=L.MUR_MEMORY)
    net.fit_linear(data, ridge=0.0, prior="mur", support="mur")
    mur = L.BoundaryNet(seed=4, memory=L.MUR_MEMORY)
    for f in range(6):
        mur.embed_linear(f, L.mur_map(f))
    return L, data, net, mur


def test_learned_map_on_murs_stencil_is_stable_and_fits_better_than_mur(mur_training):
    """The fitted coefficients lower the one-step error below Mur's own, the layer stays bounded
    over 1500 closed-loop steps and absorbs better than the layer without the network."""
    L, data, net, mur = mur_training
    for f in range(6):
        assert net.loss(f, data.X[f], data.T[f]) < mur.loss(f, data.X[f], data.T[f])
    kw = dict(shape=(24, 24, 24), period=14.0, cpml=8, shell=4)
    long = L.reflection_db(L.LearnedBoundary(net, "bf16x2"), steps=1500, every=50, **kw)
    ref = max(r for _, _, r in long["series"])
    assert all(math.isfinite(e) for _, e, _ in long["series"])
    assert long["series"][-1][1] < 0.1 * ref
    first = L.reflection_db(L.LearnedBoundary(net, "bf16x2"), steps=60, every=4, **kw)["reflection_db"]
    zero = L.BoundaryNet(seed=3, memory=L.MUR_MEMORY)
    zero.params.zero_()
    held = L.reflection_db(L.LearnedBoundary(zero, "bf16x2"), steps=60, every=4, **kw)["reflection_db"]
    assert first < held - 10.0, (first, held)


def test_linear_inference_matches_the_network(mur_training):
    """A network that is an exactly embedded linear map gives the same ghosts through the
    'linear' kernel as through the float32 MLP kernel (GELU kept in its linear range)."""
    L, data, net, mur = mur_training
    shape = (14, 11, 9)
    E, H = _fields(shape, 50, 0.05)
    Ed, Hd = _cuda(E), _cuda(H)
    n, _ = L.columns(shape)
    prev = numpy.random.default_rng(51).standard_normal((n, 6)).astype(numpy.float32) * 0.01
    w = numpy.concatenate([net.output_weights(f).cpu().numpy()[None, :].repeat(1, 0) for f in range(6)])
    p32 = _predict(L, shape, 63, "f32", net.params, Ed, Hd, memory=net.memory, prev=prev)
    plin = _predict(L, shape, 63, "linear", net.weights("linear"), Ed, Hd, memory=net.memory, prev=prev)
    _, face_of = O.column_cells(shape, 63)
    used = w[face_of] > 0
    scale = numpy.max(numpy.abs(p32[used]))
    assert numpy.max(numpy.abs(p32[used] - plin[used])) <= 1e-4 * scale
    # an Adam step leaves no linear map behind
    net2 = L.BoundaryNet(seed=4, memory=L.MUR_MEMORY)
    net2.embed_linear(0, L.mur_map(0))
    with pytest.raises(ValueError):
        net2.weights("linear")


def test_reflection_with_cpml_on_the_other_faces(mur_training):
    """A learned layer on the z faces with CPML on x and y, as deployed: the thin and the
    doubled grid both carry the x/y CPML, so the shell error measures the z layer."""
    L, data, net, mur = mur_training
    lb = L.LearnedBoundary(mur, "f32", faces=["-z", "+z"])
    r = L.reflection_db(lb, shape=(24, 24, 24), steps=60, every=4, period=14.0, cpml=8, shell=4, cpml_other=6)
    assert r["big_shape"] == (24, 24, 48)
    assert math.isfinite(r["reflection_db"]) and r["reflection_db"] < 0.0


def test_evaluation_and_fallback(small_training):
    """The evaluation's verdict decides between the learned layer and CPML."""
    L, data, net, before, start, after = small_training
    lb = L.LearnedBoundary(net, "bf16x2")
    v = L.evaluate(lb, shape=(24, 24, 24), steps=60, periods=(14.0,), stability_shape=(24, 24, 24),
                stability_steps=200)
    assert set(v) >= {"reflection_db", "stable", "accepted", "growth_onset_step"}
    kw = dict(epsilon=[numpy.ones((12, 12, 12), numpy.float32)] * 3, pmls=[], do_poynting=False,
              dt=L.DEFAULT_DT)
    sim, used = L.thin_or_cpml(kw, lb, verdict=v)
    assert used == ("learned" if v["accepted"] else "cpml")
    sim, used = L.thin_or_cpml(kw, lb, verdict={"accepted": False})
    assert used == "cpml" and len(sim.pmls) == 6
    sim, used = L.thin_or_cpml(kw, lb, reflection_db_value=-45.0)
    assert used == "learned" and sim.pmls == []
