"""The snapshot layout helpers (no GPU needed): unvec/vec round trip and the example
script's (fdtd.py) {'grid', 'E', 'H', 'S'} file format."""
import lzma
import pickle

import numpy

from opencl_fdtd_gb300 import snapshot


def test_vec_unvec_round_trip():
    shape = (4, 5, 6)
    f = [numpy.random.default_rng(k).standard_normal(shape) for k in range(3)]
    v = snapshot.vec(f)
    u = snapshot.unvec(v, shape)
    assert u.shape == (3, *shape)
    for k in range(3):
        assert numpy.array_equal(u[k], f[k])
    assert numpy.array_equal(snapshot.vec(u), v)


def test_snapshot_file_is_an_lzma_pickle(tmp_path):
    d = {"grid": {"shape": (2, 2, 2)}, "E": numpy.zeros((3, 2, 2, 2)), "H": numpy.ones((3, 2, 2, 2))}
    p = tmp_path / "saved_simulation"
    with lzma.open(p, "wb") as f:
        pickle.dump(d, f)
    back = snapshot.load_snapshot(p)
    assert set(back) == {"grid", "E", "H"} and numpy.array_equal(back["H"], d["H"])
