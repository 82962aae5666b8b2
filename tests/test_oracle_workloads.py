"""The oracle's restatement of the synthetic workloads' generators against the
library's host generators, bit for bit (CPU only).

The reference arm of the benchmark builds its inputs with the restatement, so
that the reference's host multiply runs without the library loaded; these
tests pin that it multiplies the same matrices the library's arm does."""
import numpy as np
import pytest

import matrixmultiplicationcuda_gb300 as m
from oracle import oracle


@pytest.mark.parametrize("pattern,param", [(0, 0.0), (1, 8.0), (2, 256.0), (3, 1.5)])
@pytest.mark.parametrize("bR", [16, 32, 64])
def test_structure_bit_identical(pattern, param, bR):
    for density, seed in ((0.01, 3), (0.05, 11), (0.2, 12345)):
        a = oracle.gen_structure(2048, 4096, bR, pattern, density, param, seed=seed)
        b = m.gen_structure(2048, 4096, bR, pattern, density, param, seed=seed)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


@pytest.mark.parametrize("dist", [0, 1, 2])
def test_values_bit_identical(dist):
    x = oracle.gen_values(257, 64, 16, dist, seed=5)
    y = m.gen_values(257, 64, 16, dist, seed=5)
    assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
    x = oracle.gen_dense(129, 96, dist, seed=6)
    y = m.gen_dense(129, 96, dist, seed=6)
    assert np.array_equal(x.view(np.uint32), y.view(np.uint32))


def test_headline_structure_matches():
    """The 16384^2, 64x16, 2 % random structure the benchmark runs."""
    a = oracle.gen_structure(16384, 16384, 64, oracle.PATTERN_RANDOM, 0.02, 0, seed=20240)
    b = m.gen_structure(16384, 16384, 64, m.PATTERN_RANDOM, 0.02, 0, seed=20240)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert len(a[1]) == 5161


def test_bad_arguments_rejected():
    with pytest.raises(ValueError):
        oracle.gen_structure(100, 64, 64, 0, 0.1)        # M not a multiple of bR
    with pytest.raises(ValueError):
        oracle.gen_structure(128, 64, 64, 7, 0.1)        # unknown pattern


def test_f64_product_threads_agree():
    rp, ci = oracle.gen_structure(512, 512, 32, 0, 0.1, seed=1)
    v = oracle.gen_values(len(ci), 32, 16, 0, seed=2).astype(np.float64)
    B = oracle.gen_dense(512, 64, 2, seed=3).astype(np.float64)
    one = oracle.bcsr_matmul_f64(rp, ci, v, 32, 16, B)
    many = oracle.bcsr_matmul_f64(rp, ci, v, 32, 16, B, threads=4)
    assert np.array_equal(one, many)
