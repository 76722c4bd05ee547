"""Host-side logic of the learned boundary, without a GPU: the library's column layout against
the oracle, face-mask parsing, the structure of Mur's map and the teacher-data bookkeeping."""
import numpy
import pytest

from oracle import lbc as O


def _L():
    from opencl_fdtd_gb300 import learned_boundary
    return learned_boundary


@pytest.mark.parametrize("shape,mask", [((12, 9, 7), 63), ((10, 6, 5), 0b110011), ((5, 8, 3), 0b001100),
                                        ((3, 4, 2), 63), ((2, 2, 2), 0b000001), ((7, 7, 7), 0)])
def test_columns_match_the_oracle(shape, mask):
    L = _L()
    n, off = L.columns(shape, mask)
    fl, ncol = O.faces(shape, mask)
    assert n == ncol
    want = [-1] * 6 + [ncol]
    for a, side, u0, nu, v0, nv, col0 in fl:
        want[2 * a + side] = col0
    assert off == want


def test_columns_rejects_bad_arguments():
    L = _L()
    from opencl_fdtd_gb300 import _lib
    with pytest.raises(Exception):
        L.columns((1, 5, 5), 63)
    with pytest.raises(Exception):
        L.columns((5, 5, 5), 64)
    assert _lib.FDTD_LBC_NPARAM == O.NPARAM


def test_face_mask_parsing():
    L = _L()
    assert L.face_mask(None) == 63
    assert L.face_mask(["-x", "+x"]) == 0b000011
    assert L.face_mask([("y", "n"), ("z", "p")]) == 0b100100
    assert L.face_mask(17) == 17


def test_mur_map_structure():
    """Mur's map uses, for each tangential ghost component, its own field at depth 0 with
    weight 1 - m, and the curl of the other field (entries of weight dt); nothing else, no
    bias, and the faces of one side map onto each other under axis permutation."""
    L = _L()
    m, dt = L.MUR_MEMORY, L.DEFAULT_DT
    assert abs(m - (1 - dt) / (1 + dt)) < 1e-15
    for f in range(6):
        a, side = divmod(f, 2)
        A = L.mur_map(f)
        assert A.shape == (109, 6)
        assert not A[108].any()
        used = [o for o in range(6) if A[:, o].any()]
        assert used == ([3 + p for p in range(3) if p != a] if side == 0 else [p for p in range(3) if p != a])
        for o in used:
            p = o % 3
            own = L._stencil_index(a, 0, {}, o)
            assert abs(A[own, o] - (1 - m)) < 1e-12
            others = numpy.flatnonzero(A[:, o])
            comps = set(int(k) % 6 for k in others if k != own)
            # the curl of E for an H ghost, of H for an E ghost, never the ghost's own field type
            assert comps <= ({0, 1, 2} if side == 0 else {3, 4, 5})
            scale = dt if side == 0 else m * dt
            vals = A[[k for k in others if k != own], o]
            assert numpy.allclose(numpy.abs(vals), scale)
            # a curl: the entries sum to zero
            assert abs(vals.sum()) < 1e-12


def test_teacher_data_bookkeeping():
    torch = pytest.importorskip("torch")
    L = _L()
    d = L.TeacherData(torch.device("cpu"))
    assert d.sizes() == [0] * 6
    d.add(2, torch.ones(3, 108), torch.zeros(3, 6))
    d.add(2, torch.full((2, 108), 2.0), torch.ones(2, 6))
    d.add(5, torch.ones(1, 108), torch.ones(1, 6))
    assert d.sizes() == [0, 0, 5, 0, 0, 1]
    assert d.X[2].shape == (5, 108) and float(d.X[2][4, 0]) == 2.0
    d.add(2, torch.ones(1, 108), torch.ones(1, 6))
    assert d.sizes()[2] == 6


def test_dipole_pulse_shape():
    L = _L()
    w = L.dipole_pulse(20.0, (0.0, 1.0, 0.0))
    assert [float(f(0)) for f in w][0] == 0.0
    vals = numpy.array([w[1](t) for t in range(200)])
    # peak of the envelope at t0 = 4 periods' widths (width = 1 period): |values| largest near t = 80
    assert 60 <= int(numpy.argmax(numpy.abs(vals))) <= 100
    assert abs(vals[0]) < 1e-3
