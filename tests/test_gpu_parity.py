"""GPU parity: the CUDA drop-in against the oracle (bit for bit, same inputs, same host) and
against the golden fixtures the reference itself wrote (1e-5 relative L2, the tolerance for
float32 fields; the fixtures come from another host whose numpy may round the float32 CPML
tables differently)."""
import json
import os

import numpy
import pytest

torch = pytest.importorskip("torch")

from oracle import port  # noqa: E402
from tests.golden import cases  # noqa: E402
from tests.golden.make_golden import c1_full, summary  # noqa: E402

pytestmark = pytest.mark.gpu

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
GOLD = numpy.load(os.path.join(HERE, "golden_cases.npz"))
REL_L2_TOL = 1e-5


def _gpu(**kw):
    from opencl_fdtd_gb300 import Simulation
    return Simulation(**kw)


def _port(**kw):
    return port.PortSimulation(nthreads=os.cpu_count(), **kw)


def rel_l2(a, b):
    a = a.astype(numpy.float64)
    b = b.astype(numpy.float64)
    return float(numpy.linalg.norm(a - b) / max(numpy.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("name", cases.CASE_NAMES)
def test_dropin_matches_oracle_bitwise(name):
    g = cases.outputs(cases.run_case(_gpu, name), name)
    c = cases.outputs(cases.run_case(_port, name), name)
    for k in c:
        assert g[k].dtype == c[k].dtype
        bad = numpy.flatnonzero(g[k] != c[k])
        assert bad.size == 0, (name, k, bad[:5], g[k][bad[:5]], c[k][bad[:5]])


@pytest.mark.parametrize("name", cases.CASE_NAMES)
def test_dropin_matches_reference_golden(name):
    g = cases.outputs(cases.run_case(_gpu, name), name)
    for k, v in g.items():
        assert rel_l2(v, GOLD["%s__%s" % (name, k)]) <= REL_L2_TOL, (name, k)


def test_config1_full_size():
    """Config 1 (64^3, 8-cell CPML x6, slab, Ez source, 500 steps): bitwise against the
    oracle, and within 1e-5 relative L2 of the reference's own run."""
    g = c1_full(_gpu)
    c = c1_full(_port)
    ge, gh = cases.to_numpy(g.E), cases.to_numpy(g.H)
    assert numpy.array_equal(ge, c.E) and numpy.array_equal(gh, c.H)
    with open(os.path.join(HERE, "golden_c1_full.json")) as f:
        gold = json.load(f)
    for k, a in (("E", ge), ("H", gh)):
        s = summary(a)
        for comp in range(3):
            assert abs(s["l2"][comp] - gold[k]["l2"][comp]) <= REL_L2_TOL * max(gold[k]["l2"]) + 1e-12
        assert rel_l2(numpy.asarray(s["sample"]), numpy.asarray(gold[k]["sample"])) <= REL_L2_TOL
    # error of the float32 result against the same 500 steps in float64
    d = c1_full(_gpu, float_type=numpy.float64)
    err = {k: float(numpy.linalg.norm(a.astype(numpy.float64) - cases.to_numpy(getattr(d, k))) /
                    numpy.linalg.norm(cases.to_numpy(getattr(d, k))))
           for k, a in (("E", ge), ("H", gh))}
    print("config1 float32 vs float64 relative L2 after 500 steps:", err)
    assert all(v < 1e-4 for v in err.values()), err


@pytest.mark.parametrize("name", ["pml_mixed", "periodic_pec_poynting", "bloch_trivial"])
def test_run_equals_canonical_loop(name):
    """Simulation.run(n, point_sources) advances exactly like the per-call loop."""
    kw, loop = cases.build(name)
    a = cases.run_case(_gpu, name)
    import copy
    b = _gpu(**copy.deepcopy(kw))
    shape = kw["epsilon"][0].shape
    N = int(numpy.prod(shape))
    src = [(int(numpy.ravel_multi_index(p, shape)) + c * N,
            [cases._WAVES[w](t) for t in range(loop["steps"])]) for p, c, w in loop["sources"]]
    b.run(loop["steps"], point_sources=src).wait()
    for k, v in cases.outputs(a, name).items():
        assert numpy.array_equal(v, cases.to_numpy(getattr(b, k))), k


def test_psi_layout_is_a_permutation_of_the_reference_layout():
    a = cases.run_case(_gpu, "pml_mixed")
    c = cases.run_case(_port, "pml_mixed")
    kw, _ = cases.build("pml_mixed")
    for f, p in enumerate(kw["pmls"]):
        r = "xyz".index(p["axis"])
        perm = {0: (0, 1, 2), 1: (1, 0, 2), 2: (2, 0, 1)}[r]
        for fld in "EH":
            for j in range(2):
                mine = a.psi[fld][f][j].cpu().numpy().transpose(perm)
                assert numpy.array_equal(mine, c.psi[fld][2 * f + j]), (f, fld, j)


def test_pec_cells_stay_zero():
    shape = (12, 12, 12)
    eps = [numpy.full(shape, 2.0, numpy.float32) for _ in range(3)]
    for e in eps:
        e[4:8, 4:8, 4:8] = numpy.inf
    sim = _gpu(epsilon=eps, pmls=[], do_poynting=True)
    N = 12 ** 3
    ind = int(numpy.ravel_multi_index((2, 2, 2), shape)) + N
    for t in range(40):
        sim.update_E([])
        sim.E[ind] += float(numpy.sin(0.5 * t))
        sim.update_H([])
        sim.update_S([])
    E = sim.get("E").reshape(3, *shape)
    assert numpy.abs(E).max() > 0
    assert numpy.all(E[:, 4:8, 4:8, 4:8] == 0)


def test_api_semantics():
    from opencl_fdtd_gb300 import Simulation, Event
    shape = (8, 8, 8)
    eps = [numpy.ones(shape, numpy.float32)] * 3
    pm = [{"axis": "x", "polarity": "n"}]
    sim = Simulation(eps, pm, do_poynting=False)
    assert pm[0]["thickness"] == 8 and pm[0]["ma"] == 1  # setdefault on the caller's dict
    assert sim.update_S is None and sim.update_F is None and sim.update_J is None
    assert isinstance(sim.E, torch.Tensor) and sim.E.shape == (3 * 512,) and sim.E.is_cuda
    e = sim.update_E([])
    assert isinstance(e, Event)
    e2 = sim.update_H([e])
    e2.wait()
    assert abs(sim.dt - 0.99 / numpy.sqrt(3)) < 1e-15
    sim2 = Simulation(eps, [], do_poynting=True)
    assert sim2.oS.shape == (3 * 512, 2) and sim2.S.shape == (3 * 512,)
    assert "E" in sim2.sources and "S" in sim2.sources


def test_constructor_errors():
    from opencl_fdtd_gb300 import Simulation
    shape = (6, 6, 6)
    one = numpy.ones(shape, numpy.float32)
    with pytest.raises(Exception, match="length of 3"):
        Simulation([one, one], [])
    with pytest.raises(Exception, match="same shape"):
        Simulation([one, one, numpy.ones((6, 6, 5), numpy.float32)], [])
    with pytest.raises(Exception, match="Invalid dt"):
        Simulation([one] * 3, [], dt=-1.0)
    with pytest.warns(UserWarning, match="unstable dt"):
        Simulation([one] * 3, [], dt=1.0)
    with pytest.raises(Exception, match="Duplicate pml"):
        Simulation([one] * 3, [{"axis": "x", "polarity": "n"}, {"axis": "x", "polarity": "n"}])
    with pytest.raises(Exception, match="Unsupported type"):
        Simulation([one] * 3, [], float_type=numpy.float16)


def test_snapshot_and_checkpoint_resume(tmp_path):
    """The driver's snapshot dict, and a checkpoint that resumes bit for bit."""
    from opencl_fdtd_gb300 import snapshot
    kw, loop = cases.build("pml_mixed")
    import copy
    a = _gpu(**copy.deepcopy(kw))
    a.run(10)
    a.save_snapshot(tmp_path / "snap.xz")
    d = snapshot.load_snapshot(tmp_path / "snap.xz")
    shape = kw["epsilon"][0].shape
    assert d["E"].shape == (3, *shape) and numpy.array_equal(d["E"].reshape(-1), a.get("E"))
    assert numpy.array_equal(d["S"].reshape(-1), a.get("S"))
    a.save_checkpoint(tmp_path / "ck.pt")
    a.run(7)
    b = _gpu(**copy.deepcopy(kw))
    b.load_checkpoint(tmp_path / "ck.pt")
    b.run(7)
    for k in ("E", "H", "S"):
        assert torch.equal(getattr(a, k), getattr(b, k)), k
    assert b.steps_run == 17
