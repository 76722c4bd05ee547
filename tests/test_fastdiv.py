"""The magic-number division the kernels use to decode flat indices (csrc/yee_common.cuh
FastDiv), emulated in integer arithmetic on the host over edge and random cases."""
import numpy
import pytest


def make(d):
    l = 0
    while (1 << l) < d:
        l += 1
    m = (((1 << 32) * ((1 << l) - d)) // d) + 1
    assert 0 < m < (1 << 32) or d == 1
    return m, l


def div(n, m, l):
    t = (m * n) >> 32
    return (t + n) >> l


@pytest.mark.parametrize("d", [1, 2, 3, 5, 7, 64, 73, 345, 25185, 65535, 65536, 1 << 20,
                               (1 << 31) - 1, (1 << 31) + 1, (1 << 32) - 1])
def test_fastdiv_edges(d):
    m, l = make(d)
    ns = [0, 1, d - 1, d, d + 1, 2 * d - 1, 2 * d, (1 << 32) - 1, (1 << 32) - 2, (1 << 31)]
    rng = numpy.random.default_rng(d)
    ns += [int(v) for v in rng.integers(0, 1 << 32, 2000, dtype=numpy.uint64)]
    for n in ns:
        if 0 <= n < (1 << 32):
            assert div(n, m, l) == n // d, (n, d)


def test_fastdiv_random_divisors():
    rng = numpy.random.default_rng(0)
    for d in rng.integers(1, 1 << 32, 300, dtype=numpy.uint64):
        d = int(d)
        m, l = make(d)
        for n in rng.integers(0, 1 << 32, 200, dtype=numpy.uint64):
            n = int(n)
            assert div(n, m, l) == n // d
