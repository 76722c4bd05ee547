"""The one-pass step kernel (Simulation.run(path='fused')) against the per-call drop-in loop and
the oracle: bit-identical E, H, S and CPML state for every tiling (rows per tile, x chunk, stage
count), with the rows of non-wrapping tiles staged by bulk copies or by per-element copies,
including tiles of one row, chunks of one plane and z faces whose thickness is not a multiple
of the 16-byte unit."""
import copy
import math
import os

import numpy
import pytest

torch = pytest.importorskip("torch")

from oracle import port  # noqa: E402
from opencl_fdtd_gb300 import geometry  # noqa: E402
from tests.golden import cases  # noqa: E402

pytestmark = pytest.mark.gpu


def _gpu(**kw):
    from opencl_fdtd_gb300 import Simulation
    return Simulation(**kw)


def _np(a):
    return a.detach().cpu().numpy().reshape(-1)


def _sources(kw, loop, nsteps):
    shape = kw["epsilon"][0].shape
    N = int(numpy.prod(shape))
    return [(int(numpy.ravel_multi_index(p, shape)) + c * N,
             [cases._WAVES[w](t) for t in range(nsteps)]) for p, c, w in loop["sources"]]


def _same_state(a, b, poynting):
    for k in ("E", "H") + (("S", "oS") if poynting else ()):
        x, y = _np(getattr(a, k)), _np(getattr(b, k))
        bad = numpy.flatnonzero(x != y)
        assert bad.size == 0, (k, bad[:5], x[bad[:5]], y[bad[:5]])
    for fld in "EH":
        for (u1, v1), (u2, v2) in zip(a.psi[fld], b.psi[fld]):
            assert torch.equal(u1, u2) and torch.equal(v1, v2), fld


# (rows per tile, x chunk, stages, bulk copies, block shape)
TILINGS = [(0, 0, 0, 1, 0), (1, 3, 2, 1, 2), (2, 1, 3, 0, 1), (3, 2, 0, 1, 2), (5, 7, 2, 0, 1), (4, 5, 4, 1, 1),
           (0, 0, 0, 1, 1), (0, 4, 3, 1, 2)]


def _tune(sim, tiling):
    rows, xc, ns, tma, shape = tiling
    sim.tune(fused_rows=rows, fused_xchunk=xc, fused_stages=ns, fused_tma=bool(tma), fused_shape=shape)


@pytest.mark.parametrize("name", ["c1_small", "pml_mixed", "periodic_pec_poynting", "nonuniform",
                                  "dx_half", "f64_mixed"])
@pytest.mark.parametrize("tiling", TILINGS)
@pytest.mark.parametrize("nsteps", [7, 10])
def test_fused_equals_per_call_loop(name, tiling, nsteps):
    kw, loop = cases.build(name)
    src = _sources(kw, loop, nsteps)
    a = _gpu(**copy.deepcopy(kw))
    b = _gpu(**copy.deepcopy(kw))
    _tune(b, tiling)
    a.run(nsteps, point_sources=src, path="plain")
    b.run(nsteps, point_sources=src, path="fused")
    assert b.tuning("last_run_path") == 3
    assert b.device_status() == 0
    _same_state(a, b, kw.get("do_poynting", True))


@pytest.mark.parametrize("shape,faces,T", [((9, 40, 37), "xyz", (3, 5, 6)), ((6, 23, 18), "yz", (2, 4, 7)),
                                           ((7, 31, 20), "z", (0, 0, 9)), ((5, 17, 11), "", (0, 0, 0))])
@pytest.mark.parametrize("tiling", [(1, 2, 2, 1, 2), (3, 4, 3, 1, 1), (6, 0, 0, 1, 0), (2, 3, 4, 0, 2),
                                    (0, 0, 0, 1, 2)])
@pytest.mark.parametrize("dtype,mu", [(numpy.float32, False), (numpy.float32, True), (numpy.float64, True)])
def test_fused_many_tiles(shape, faces, T, tiling, dtype, mu):
    """Grids with many tiles, most of them staged by bulk copies, CPML faces of uneven
    thickness (the 'p' side one cell thinner), a PEC row, mu and two point sources."""
    rng = numpy.random.default_rng(sum(shape) + 7 * len(faces))
    eps = [rng.uniform(1, 5, shape).astype(dtype) for _ in range(3)]
    eps[1][shape[0] // 2, shape[1] // 3, :3] = numpy.inf
    kw = dict(epsilon=eps, do_poynting=True,
              pmls=[{"axis": a, "polarity": p, "thickness": max(1, T["xyz".index(a)] - (p == "p"))}
                    for a in faces for p in "np"],
              initial_fields={k: [rng.standard_normal(shape).astype(dtype) for _ in range(3)] for k in "EH"})
    if mu:
        kw["mu"] = [rng.uniform(1, 2, shape).astype(dtype) for _ in range(3)]
    N = int(numpy.prod(shape))
    steps = 9
    srcs = [(int(numpy.ravel_multi_index((shape[0] // 2, 1, shape[2] - 1), shape)) + 2 * N,
             [math.sin(0.4 * t) for t in range(steps)]),
            (int(numpy.ravel_multi_index((0, shape[1] - 2, 0), shape)) + 1 * N, [0.25] * steps)]
    a = _gpu(**copy.deepcopy(kw))
    b = _gpu(**copy.deepcopy(kw))
    _tune(b, tiling)
    a.run(steps, point_sources=srcs, path="plain")
    b.run(steps, point_sources=srcs, path="fused")
    assert b.tuning("last_run_path") == 3
    assert b.device_status() == 0
    _same_state(a, b, True)


def test_fused_matches_oracle_with_mu_and_sources():
    shape = (18, 16, 20)
    eps, mu = geometry.sphere_inclusions(shape, n=4, rmin=2, rmax=5, seed=21, pec_index=0)
    pmls = [{"axis": a, "polarity": p, "thickness": 3} for a in "xyz" for p in "np"]
    N = int(numpy.prod(shape))
    steps = 25
    srcs = [(int(numpy.ravel_multi_index((9, 8, 10), shape)) + 2 * N, [math.sin(0.4 * t) for t in range(steps)]),
            (int(numpy.ravel_multi_index((4, 12, 5), shape)) + 0 * N, [math.cos(0.3 * t) for t in range(steps)]),
            (int(numpy.ravel_multi_index((9, 8, 10), shape)) + 2 * N, [0.5] * steps)]
    kw = dict(epsilon=eps, mu=mu, pmls=pmls, do_poynting=True)
    g = _gpu(**copy.deepcopy(kw))
    g.tune(fused_rows=3, fused_xchunk=4)
    g.run(steps, point_sources=srcs, path="fused")
    assert g.tuning("last_run_path") == 3
    c = port.PortSimulation(nthreads=os.cpu_count(), **copy.deepcopy(kw))
    for t in range(steps):
        c.update_E()
        for ind, vals in srcs:
            c.E[ind] = c.E[ind] + numpy.float32(vals[t])
        c.update_H()
        c.update_S()
    for k in ("E", "H", "S", "oS"):
        assert numpy.array_equal(_np(getattr(g, k)), getattr(c, k).reshape(-1)), k


def test_fused_then_per_call_continue_identically():
    """State left by a fused run (odd step count: copied back from the scratch buffers) is
    the full state: per-call steps after it match an all-per-call history."""
    kw, loop = cases.build("pml_mixed")
    src = _sources(kw, loop, 9)
    a = _gpu(**copy.deepcopy(kw))
    b = _gpu(**copy.deepcopy(kw))
    a.run(9, point_sources=src, path="plain")
    b.run(9, point_sources=src, path="fused")
    for s in (a, b):
        for _ in range(4):
            s.update_E([])
            s.update_H([])
            s.update_S([])
    _same_state(a, b, True)


SLAB_CASES = [n for n in cases.CASE_NAMES if n != "fieldsrc"]


@pytest.mark.parametrize("name", SLAB_CASES)
@pytest.mark.parametrize("slab", [1, 2, 5, 0])
def test_slab_schedule_equals_per_call_loop(name, slab):
    """run(path='plain') advances the update kernels over x slabs (E, then H one plane
    behind, then S); every slab width gives the per-call loop's state bit for bit."""
    kw, loop = cases.build(name)
    n = loop["steps"]
    a = cases.run_case(_gpu, name)
    b = _gpu(**copy.deepcopy(kw))
    b.tune(slab=slab)
    b.run(n, point_sources=_sources(kw, loop, n), path="plain")
    for k, v in cases.outputs(a, name).items():
        assert numpy.array_equal(v, _np(getattr(b, k))), k
    for fld in ("EHFG" if kw.get("bloch_boundaries") else "EH"):
        for (u1, v1), (u2, v2) in zip(a.psi[fld], b.psi[fld]):
            assert torch.equal(u1, u2) and torch.equal(v1, v2), fld


def test_slab_schedule_bloch_mu():
    shape = (14, 12, 20)
    rng = numpy.random.default_rng(8)
    eps, mu = geometry.sphere_inclusions(shape, n=3, rmin=2, rmax=4, seed=4)
    init = {k: [rng.standard_normal(shape).astype(numpy.float32) for _ in range(3)] for k in "EHFG"}
    bloch = [{"axis": "x", "real": math.cos(0.3), "imag": math.sin(0.3)},
             {"axis": "z", "real": math.cos(0.7), "imag": math.sin(0.7)}]
    pmls = [{"axis": "y", "polarity": p, "thickness": 3} for p in "np"]
    kw = dict(epsilon=eps, mu=mu, pmls=pmls, bloch_boundaries=bloch, initial_fields=init, do_poynting=True)
    a = _gpu(**copy.deepcopy(kw))
    for _ in range(12):
        a.update_E([]); a.update_F([]); a.update_H([]); a.update_G([]); a.update_S([])
    for slab in (1, 3, 0):
        b = _gpu(**copy.deepcopy(kw))
        b.tune(slab=slab)
        b.run(12, path="plain")
        for k in ("E", "H", "F", "G", "S"):
            assert torch.equal(getattr(a, k), getattr(b, k)), (slab, k)


HS_SHAPES = [((16, 14, 12), 3), ((10, 9, 200), 3), ((6, 5, 511), 2), ((9, 11, 100), 4), ((7, 6, 300), 1),
             ((5, 6, 224), 2), ((6, 7, 73), 2)]


@pytest.mark.parametrize("shape,T", HS_SHAPES)
@pytest.mark.parametrize("xchunk", [1, 3, 8])
@pytest.mark.parametrize("nsteps", [5, 8])
def test_hs_path_equals_per_call_loop(shape, T, xchunk, nsteps):
    """run(path='hs'): H and S in one launch, with blocks of whole z rows so that several
    blocks (and, for sz > 149, one-row blocks) recompute their first row's y-1 products; rows
    longer than 224 cells take the per-update kernels."""
    rng = numpy.random.default_rng(sum(shape) + T)
    eps = [rng.uniform(1, 4, shape).astype(numpy.float32) for _ in range(3)]
    eps[1][1:3, 2:4, 5:9] = numpy.inf
    init = {k: [rng.standard_normal(shape).astype(numpy.float32) for _ in range(3)] for k in "EH"}
    pmls = [{"axis": a, "polarity": p, "thickness": T} for a in "xyz" for p in "np"
            if 2 * T <= shape["xyz".index(a)]]
    kw = dict(epsilon=eps, pmls=pmls, initial_fields=init, do_poynting=True)
    N = int(numpy.prod(shape))
    src = [(int(rng.integers(0, 3 * N)), [math.sin(0.3 * t) for t in range(nsteps)])]
    a = _gpu(**copy.deepcopy(kw))
    b = _gpu(**copy.deepcopy(kw))
    b.tune(hs_xchunk=xchunk, hs_prefetch=bool(xchunk % 2))
    a.run(nsteps, point_sources=src, path="plain")
    b.run(nsteps, point_sources=src, path="hs")
    _same_state(a, b, True)


@pytest.mark.parametrize("shape,T", HS_SHAPES[:4] + HS_SHAPES[6:])
@pytest.mark.parametrize("xchunk", [0, 1, 3, 8])
@pytest.mark.parametrize("pdl", [False, True])
def test_hs_path_launch_options_equal_per_call_loop(shape, T, xchunk, pdl):
    """H+S path with and without programmatic dependent launches of the E and H+S kernels,
    at the automatic (0) and at fixed x chunks: the per-call loop's bits, with point sources
    added by the E kernel."""
    rng = numpy.random.default_rng(sum(shape) + 7 * T)
    eps = [rng.uniform(1, 4, shape).astype(numpy.float32) for _ in range(3)]
    eps[0][1:3, 2:4, 1:4] = numpy.inf
    init = {k: [rng.standard_normal(shape).astype(numpy.float32) for _ in range(3)] for k in "EH"}
    pmls = [{"axis": a, "polarity": p, "thickness": T} for a in "xyz" for p in "np"
            if 2 * T <= shape["xyz".index(a)]]
    kw = dict(epsilon=eps, pmls=pmls, initial_fields=init, do_poynting=True)
    N = int(numpy.prod(shape))
    nsteps = 7
    src = [(int(rng.integers(0, 3 * N)), [math.sin(0.3 * t) for t in range(nsteps)])]
    a = _gpu(**copy.deepcopy(kw))
    b = _gpu(**copy.deepcopy(kw))
    b.tune(hs_xchunk=xchunk, pdl=pdl)
    assert (b.tuning("hs_xchunk"), b.tuning("pdl")) == (xchunk, int(pdl))
    a.run(nsteps, point_sources=src, path="plain")
    b.run(nsteps, point_sources=src, path="hs")
    # rows longer than 224 cells take the per-update kernels
    assert b.tuning("last_run_path") == (2 if shape[2] <= 224 else 1)
    _same_state(a, b, True)


@pytest.mark.parametrize("name", ["c1_small", "pml_mixed", "nonuniform", "f64_mixed"])
def test_hs_path_launch_options_cases(name):
    """The default launch options (programmatic dependent launch, DFT sample in the H+S
    launch) on golden cases with non-uniform spacing and float64: the per-call loop's bits."""
    kw, loop = cases.build(name)
    kw["do_poynting"] = True
    n = loop["steps"]
    src = _sources(kw, loop, n)
    a = _gpu(**copy.deepcopy(kw))
    b = _gpu(**copy.deepcopy(kw))
    b.tune(pdl=True, hs_dft=True)
    a.run(n, point_sources=src, path="plain")
    b.run(n, point_sources=src, path="hs")
    _same_state(a, b, True)


@pytest.mark.parametrize("form", [0])
@pytest.mark.parametrize("name", cases.CASE_NAMES)
def test_e_kernel_forms_equal_default(name, form):
    """The bulk E kernel's other form (0: next plane loaded ahead at three blocks per SM)
    against the default (per-plane loads at four blocks per SM): every golden case (Bloch F/G,
    non-uniform spacing, float64, overlapping faces) through the per-call loop, and the run
    path, bit for bit."""
    from opencl_fdtd_gb300 import Simulation

    def tuned(**kw):
        s = Simulation(**kw)
        s.tune(e_form=form)
        assert s.tuning("e_form") == form
        return s

    a = cases.run_case(Simulation, name)
    b = cases.run_case(tuned, name)
    oa, ob = cases.outputs(a, name), cases.outputs(b, name)
    for k in oa:
        assert numpy.array_equal(oa[k], ob[k]), (name, k)
    kw, loop = cases.build(name)
    if not kw.get("bloch_boundaries"):
        kw["do_poynting"] = True
        n = loop["steps"]
        src = _sources(kw, loop, n)
        c = _gpu(**copy.deepcopy(kw))
        d = tuned(**copy.deepcopy(kw))
        c.run(n, point_sources=src)
        d.run(n, point_sources=src)
        _same_state(c, d, True)


@pytest.mark.parametrize("name", ["c1_small", "pml_mixed", "periodic_pec_poynting", "nonuniform", "dx_half", "f64_mixed"])
def test_hs_path_cases(name):
    kw, loop = cases.build(name)
    if not kw.get("do_poynting", True):
        kw["do_poynting"] = True
    n = loop["steps"]
    src = _sources(kw, loop, n)
    a = _gpu(**copy.deepcopy(kw))
    b = _gpu(**copy.deepcopy(kw))
    a.run(n, point_sources=src, path="plain")
    b.run(n, point_sources=src, path="hs")
    _same_state(a, b, True)


def test_hs_path_with_mu():
    shape = (18, 16, 20)
    eps, mu = geometry.sphere_inclusions(shape, n=4, rmin=2, rmax=5, seed=31, pec_index=2)
    pmls = [{"axis": a, "polarity": p, "thickness": 3} for a in "xyz" for p in "np"]
    kw = dict(epsilon=eps, mu=mu, pmls=pmls, do_poynting=True)
    N = int(numpy.prod(shape))
    src = [(int(numpy.ravel_multi_index((9, 8, 10), shape)) + 2 * N, [math.sin(0.4 * t) for t in range(21)])]
    a = _gpu(**copy.deepcopy(kw))
    b = _gpu(**copy.deepcopy(kw))
    a.run(21, point_sources=src, path="plain")
    b.run(21, point_sources=src, path="hs")
    _same_state(a, b, True)


@pytest.mark.parametrize("kind", ["same_cell", "components", "many"])
def test_hs_path_point_sources_equal_per_call_loop(kind):
    """On the H+S path the E kernel adds up to 8 point sources itself (more fall back to the
    separate launch): repeated sources on one cell component add in list order, sources on
    the three components of one cell, and 11 sources all give the per-call loop's bits."""
    rng = numpy.random.default_rng(31)
    shape = (18, 15, 13)
    eps = [rng.uniform(1, 4, shape).astype(numpy.float32) for _ in range(3)]
    pmls = [{"axis": a, "polarity": p, "thickness": 3} for a in "xyz" for p in "np"]
    kw = dict(epsilon=eps, pmls=pmls, do_poynting=True)
    N = int(numpy.prod(shape))
    n = 9
    cell = int(numpy.ravel_multi_index((9, 7, 6), shape))
    if kind == "same_cell":
        inds = [cell + N, cell + N, cell + N]
    elif kind == "components":
        inds = [cell, cell + N, cell + 2 * N, cell + N]
    else:
        inds = [int(i) for i in rng.integers(0, 3 * N, 11)]
    src = [(i, [float(rng.standard_normal()) * 10.0 ** -k for _ in range(n)]) for k, i in enumerate(inds)]
    a = _gpu(**copy.deepcopy(kw))
    b = _gpu(**copy.deepcopy(kw))
    a.run(n, point_sources=src, path="plain")
    b.run(n, point_sources=src, path="hs")
    assert b.tuning("last_run_path") == 2
    _same_state(a, b, True)
