"""The parallel replay of the CV loss sum equals a serial left-to-right FP64
sum bit for bit, including ties, binade crossings, zeros and subnormals."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def serial(v):
    m = 0.0
    for x in v.tolist():
        m = m + x
    return m


@pytest.mark.parametrize("kind", range(7))
def test_sequential_sum_bit_identical(gpu, kind):
    rng = np.random.default_rng(100 + kind)
    for n in (1, 7, 1023, 1024, 1025, 5000, 1 << 17):
        if kind == 0:
            v = rng.random(n)
        elif kind == 1:
            v = rng.random(n) ** 8 * 10.0 ** rng.integers(-300, 300)
        elif kind == 2:
            v = np.round(rng.random(n) * 16) / 16          # exact values, many ties
        elif kind == 3:
            v = np.concatenate([[1e30], rng.random(n - 1)])  # huge first term
        elif kind == 4:
            v = rng.random(n) * 1e-310                      # subnormal terms
        elif kind == 5:
            v = np.where(rng.random(n) < 0.5, 0.0, rng.random(n) * 2.0 ** rng.integers(-60, 60, n))
        else:
            v = np.full(n, 0.1)                              # constant terms
        assert gpu.sequential_sum(v) == serial(v), (kind, n)
