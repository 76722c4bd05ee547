"""Batched stepping of several variants in one persistent launch (BatchSimulation): float32
storage is bit-identical to stepping each variant with Simulation.run, for every tile shape,
through CUDA-graph replays and monitor series; 16-bit storage with per-tile exponents stays
close to the float32 result, its encode/decode round trip is within the format's rounding,
and on the seeded cavity variants its error against float64 stays within stated bounds."""
import copy
import math

import numpy
import pytest

torch = pytest.importorskip("torch")

from opencl_fdtd_gb300 import geometry  # noqa: E402

pytestmark = pytest.mark.gpu

SHAPES = [((20, 18, 16), 4), ((13, 11, 23), 3), ((9, 25, 7), 2), ((16, 16, 1), 2)]


def _variant(shape, T, seed):
    rng = numpy.random.default_rng(seed)
    eps = [rng.uniform(1, 6, shape).astype(numpy.float32) for _ in range(3)]
    eps[0][tuple(slice(1, max(2, s // 4)) for s in shape)] = numpy.inf
    init = {k: [0.1 * rng.standard_normal(shape).astype(numpy.float32) for _ in range(3)] for k in "EH"}
    pmls = [{"axis": a, "polarity": p, "thickness": T} for a in "xyz" for p in "np"
            if 2 * T <= shape["xyz".index(a)]]
    return dict(epsilon=eps, pmls=pmls, initial_fields=init, do_poynting=False)


def _sims(kws):
    from opencl_fdtd_gb300 import Simulation
    return [Simulation(**copy.deepcopy(k)) for k in kws]


def _sources(sims, nsteps, seed):
    rng = numpy.random.default_rng(seed)
    out = []
    for s in sims:
        out.append([(int(rng.integers(0, 3 * s.N)), [math.sin(0.2 * t + k) for t in range(nsteps)])
                    for k in range(2)])
    return out


def _monitors(sims, seed):
    rng = numpy.random.default_rng(seed)
    return [[int(rng.integers(0, 3 * s.N)) for _ in range(3)] for s in sims]


def _same(a, b):
    for k in ("E", "H"):
        x, y = getattr(a, k), getattr(b, k)
        assert torch.equal(x, y), (k, int((x != y).sum()))
    for fld in "EH":
        for (u1, v1), (u2, v2) in zip(a.psi[fld], b.psi[fld]):
            assert torch.equal(u1, u2) and torch.equal(v1, v2), fld


@pytest.mark.parametrize("tiles", [(8, 0, "launches"), (1, 0, "launches"), (8, 0, "persistent"),
                                   (1, 1, "persistent"), (3, 2, "persistent"), (64, 0, "launches")])
def test_batch_f32_equals_per_variant_runs(tiles):
    from opencl_fdtd_gb300.batch import BatchSimulation
    kws = [_variant(s, T, 10 + i) for i, (s, T) in enumerate(SHAPES)]
    n = 9
    ref = _sims(kws)
    got = _sims(kws)
    src = _sources(ref, n, 5)
    mon = _monitors(ref, 6)
    series_ref = []
    for sim, ps, ms in zip(ref, src, mon):
        m = sim.dft_monitor([(i // sim.N, numpy.unravel_index(i % sim.N, sim.shape)) for i in ms], ())
        sim.run(n, point_sources=ps, monitor=m, path="plain")
        series_ref.append(m.series())
    b = BatchSimulation(got, storage="f32", sources=src, monitors=mon, steps=n)
    b.tune(*tiles)
    b.run(4)
    b.run(5)
    torch.cuda.synchronize()
    assert b.step_counter() == n
    for r, g, sr, sg in zip(ref, got, series_ref, b.series):
        _same(r, g)
        assert numpy.array_equal(sr, sg.cpu().numpy())


def test_batch_graph_replay_equals_run():
    from opencl_fdtd_gb300.batch import BatchSimulation
    kws = [_variant(s, T, 30 + i) for i, (s, T) in enumerate(SHAPES[:3])]
    a_s, b_s = _sims(kws), _sims(kws)
    src = _sources(a_s, 12, 7)
    a = BatchSimulation(a_s, sources=src, steps=12)
    b = BatchSimulation(b_s, sources=src, steps=12)
    a.tune(8, 0, "persistent")
    a.run(12)
    b.capture(4)
    for _ in range(3):
        b.replay()
    torch.cuda.synchronize()
    assert b.step_counter() == 12
    for x, y in zip(a_s, b_s):
        _same(x, y)


@pytest.mark.parametrize("storage,tol", [("bf16", 5e-2), ("fp16", 1e-2), ("bf16u", 5e-2)])
def test_batch_16bit_storage_tracks_f32(storage, tol):
    from opencl_fdtd_gb300.batch import BatchSimulation
    kws = [_variant(s, T, 50 + i) for i, (s, T) in enumerate(SHAPES[:3])]
    ref, got = _sims(kws), _sims(kws)
    src = _sources(ref, 20, 8)
    BatchSimulation(ref, storage="f32", sources=src, steps=20).run(20)
    b = BatchSimulation(got, storage=storage, sources=src, steps=20)
    b.run(20)
    b.sync()
    torch.cuda.synchronize()
    for r, g in zip(ref, got):
        for k in ("E", "H"):
            x = getattr(r, k).double()
            y = getattr(g, k).double()
            fin = torch.isfinite(x)
            err = torch.linalg.norm((x - y)[fin]) / torch.linalg.norm(x[fin])
            assert err < tol, (storage, k, float(err))


@pytest.mark.parametrize("storage,bits", [("bf16", 8), ("fp16", 11), ("bf16u", 8)])
def test_batch_encode_decode_round_trip(storage, bits):
    """Per-tile exponents keep every tile at full 16-bit precision, whatever its level: tiles
    whose values span 1e-30 .. 1e3 decode within half an ulp of the format."""
    from opencl_fdtd_gb300 import Simulation
    from opencl_fdtd_gb300.batch import BatchSimulation
    shape = (6, 20, 40)
    sim = Simulation(epsilon=[numpy.ones(shape, numpy.float32)] * 3, pmls=[], do_poynting=False)
    rng = numpy.random.default_rng(3)
    N = sim.N
    levels = 10.0 ** rng.uniform(-30, 3, size=3 * N)
    vals = (rng.standard_normal(3 * N) * levels).astype(numpy.float32)
    sim.E.copy_(torch.from_numpy(vals))
    b = BatchSimulation([sim], storage=storage)
    sim.E.zero_()
    b.sync()
    torch.cuda.synchronize()
    got = sim.E.cpu().numpy().astype(numpy.float64)
    want = vals.astype(numpy.float64)
    # within a tile (32 cells) the step is 2^-bits of the tile's largest magnitude
    syz = shape[1] * shape[2]
    for c in range(3):
        for x in range(shape[0]):
            for jt in range((syz + 31) // 32):
                lo = c * N + x * syz + jt * 32
                hi = min(lo + 32, c * N + (x + 1) * syz)
                m = numpy.abs(want[lo:hi]).max()
                assert numpy.abs(got[lo:hi] - want[lo:hi]).max() <= m * 2.0 ** (-bits)


def test_bf16_without_exponents_matches_bf16_with_them():
    """Power-of-two tile exponents commute with bfloat16 rounding in the normal range, so the
    'bf16u' storage (no exponents) steps to the same bits as 'bf16', and its round trip is
    plain bfloat16 rounding."""
    from opencl_fdtd_gb300.batch import BatchSimulation
    kws = [_variant(s, T, 70 + i) for i, (s, T) in enumerate(SHAPES[:3])]
    a, b = _sims(kws), _sims(kws)
    src = _sources(a, 15, 9)
    ba = BatchSimulation(a, storage="bf16", sources=src, steps=15)
    bb = BatchSimulation(b, storage="bf16u", sources=src, steps=15)
    ba.run(15)
    bb.run(15)
    ba.sync()
    bb.sync()
    torch.cuda.synchronize()
    for x, y in zip(a, b):
        assert torch.equal(x.E, y.E) and torch.equal(x.H, y.H)
    vals = (torch.randn(3 * b[0].N, device="cuda") * 10.0 ** torch.empty(3 * b[0].N, device="cuda").uniform_(-20, 3))
    b[0].E.copy_(vals)
    bb.load()
    b[0].E.zero_()
    bb.sync()
    torch.cuda.synchronize()
    assert torch.equal(b[0].E, vals.to(torch.bfloat16).to(torch.float32))


def test_batch_rejects_unsupported_simulations():
    from opencl_fdtd_gb300 import Simulation
    from opencl_fdtd_gb300.batch import BatchSimulation
    shape = (10, 10, 10)
    eps, mu = geometry.sphere_inclusions(shape, n=2, rmin=2, rmax=3, seed=1)
    with pytest.raises(ValueError):
        BatchSimulation([Simulation(epsilon=eps, mu=mu, pmls=[], do_poynting=False)])
    with pytest.raises(ValueError):
        BatchSimulation([Simulation(epsilon=eps, pmls=[], do_poynting=True)])
    with pytest.raises(ValueError):
        BatchSimulation([Simulation(epsilon=eps, pmls=[], do_poynting=False)], storage="int8")


def test_autotune_restores_state_and_caches(tmp_path):
    from opencl_fdtd_gb300.batch import BatchSimulation
    kws = [_variant(s, T, 70 + i) for i, (s, T) in enumerate(SHAPES[:3])]
    a_s, b_s = _sims(kws), _sims(kws)
    src = _sources(a_s, 8, 9)
    mon = _monitors(a_s, 10)
    a = BatchSimulation(a_s, sources=src, monitors=mon, steps=8)
    b = BatchSimulation(b_s, sources=src, monitors=mon, steps=8)
    a.run(3)
    b.run(3)
    cache = str(tmp_path / "tune.json")
    choice = b.autotune(steps=2, cache_path=cache, xchunks=(2, 8), blocks=(1, 2))
    assert not choice["cached"] and len(choice["timings"]) == 6
    assert b.step_counter() == 3
    a.run(5)
    b.run(5)
    torch.cuda.synchronize()
    for x, y, sa, sb in zip(a_s, b_s, a.series, b.series):
        _same(x, y)
        assert torch.equal(sa, sb)
    again = b.autotune(steps=2, cache_path=cache, xchunks=(2, 8), blocks=(1, 2))
    assert again["cached"] and again["xchunk"] == choice["xchunk"]


@pytest.mark.parametrize("schedule", ["launches", "persistent"])
def test_batch_f32_variant_equals_oracle(schedule):
    """One variant of the batch stepped by the batched kernels against the oracle's per-call
    loop (update_E, the sources added in list order, update_H) bit for bit."""
    import os
    from oracle import port
    from opencl_fdtd_gb300.batch import BatchSimulation
    kws = [_variant(s, T, 30 + i) for i, (s, T) in enumerate(SHAPES[:3])]
    n = 11
    got = _sims(kws)
    src = _sources(got, n, 7)
    b = BatchSimulation(got, storage="f32", sources=src, monitors=None, steps=n)
    b.tune(4, 0, schedule)
    b.run(n)
    torch.cuda.synchronize()
    for v in (0, 2):
        c = port.PortSimulation(nthreads=os.cpu_count(), **copy.deepcopy(kws[v]))
        for t in range(n):
            c.update_E()
            for ind, vals in src[v]:
                c.E[ind] = c.E[ind] + numpy.float32(vals[t])
            c.update_H()
        for k in ("E", "H"):
            x = getattr(got[v], k).detach().cpu().numpy().reshape(-1)
            assert numpy.array_equal(x, getattr(c, k).reshape(-1)), (v, k)


def _cavity_errors(storages, n_variants=4, steps=400):
    """Relative L2 of E against a float64 run of each of the first n_variants seeded c4 cavity
    variants after `steps` steps of the centre dipole pulse, per storage (the setting of the
    benchmark's batched section)."""
    from opencl_fdtd_gb300 import Simulation, workloads
    from opencl_fdtd_gb300.batch import BatchSimulation
    variants = workloads.c4(n=n_variants, steps=steps)
    wave = numpy.array([variants[0]["wave"](t) for t in range(steps)], dtype=numpy.float64)
    refs = []
    for var in variants:
        kw64, ind = workloads.c4_kwargs(var, float_type=numpy.float64)
        s64 = Simulation(**kw64)
        s64.run(steps, point_sources=[(ind, wave)], path="plain")
        refs.append(s64.E.clone())
        del s64
    out = {}
    for storage in storages:
        sims, idx = [], []
        for var in variants:
            kw, ind = workloads.c4_kwargs(var)
            sims.append(Simulation(**kw))
            idx.append(ind)
        b = BatchSimulation(sims, storage=storage, sources=[[(i, wave)] for i in idx], steps=steps)
        b.run(steps)
        b.sync()
        torch.cuda.synchronize()
        errs = []
        for s, ref in zip(sims, refs):
            fin = torch.isfinite(ref)
            errs.append(float(torch.linalg.norm((s.E.double() - ref)[fin]) / torch.linalg.norm(ref[fin])))
        out[storage] = errs
        b.close()
        del b, sims
    return out


# Bounds of the relative L2 of E against float64 (median, max over the variants) after 400
# steps on the cavity variants, about twice the measured values (float32 0.8-1.2e-7, bfloat16
# with or without tile exponents 4.0-6.5e-3, float16 5.4-7.0e-4); the benchmark's batched
# section reports the same quantity (bfloat16 without exponents: 5.1e-3 / 5.7e-3 on 16 of
# the variants). bfloat16 with and without exponents differ in the bits here: the pulse's
# leading edge holds float32-subnormal values, where a tile exponent changes the rounding.
CAVITY_BOUNDS = {"f32": (3e-7, 3e-7), "bf16": (1e-2, 1.3e-2), "bf16u": (1e-2, 1.3e-2), "fp16": (1.5e-3, 1.5e-3)}


def test_batch_16bit_error_vs_float64_on_cavity_variants():
    errs = _cavity_errors(tuple(CAVITY_BOUNDS))
    print({k: ["%.3g" % e for e in v] for k, v in errs.items()})
    for storage, (med, mx) in CAVITY_BOUNDS.items():
        e = numpy.array(errs[storage])
        assert numpy.median(e) <= med and e.max() <= mx, (storage, e)
