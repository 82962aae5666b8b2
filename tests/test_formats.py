"""File formats (no GPU): Matrix Market files as scipy's mmwrite writes them
(the writer the reference's generator uses), loaded densely and straight into
BCSR, and the binary BCSR file."""
import os

import numpy as np
import pytest

import matrixmultiplicationcuda_gb300 as m
from oracle import oracle

scipy_io = pytest.importorskip("scipy.io")
sparse = pytest.importorskip("scipy.sparse")


def half_bits(x):
    return np.asarray(x, np.float32).astype(np.float16).view(np.uint16)


@pytest.mark.parametrize("kind", ["general", "symmetric", "pattern", "integer", "array", "skew"])
def test_mtx_load_matches_scipy(tmp_path, kind):
    rng = np.random.default_rng(3)
    n = 96
    A = (rng.uniform(size=(n, n)) < 0.1) * rng.uniform(-1, 1, (n, n))
    path = os.path.join(str(tmp_path), "a.mtx")
    if kind == "symmetric":
        A = np.triu(A) + np.triu(A, 1).T
        scipy_io.mmwrite(path, sparse.coo_matrix(A), symmetry="symmetric")
    elif kind == "skew":
        A = np.triu(A, 1) - np.triu(A, 1).T
        scipy_io.mmwrite(path, sparse.coo_matrix(A), symmetry="skew-symmetric")
    elif kind == "pattern":
        A = (A != 0).astype(np.float64)
        scipy_io.mmwrite(path, sparse.coo_matrix(A), field="pattern")
    elif kind == "integer":
        A = np.round(A * 10)
        scipy_io.mmwrite(path, sparse.coo_matrix(A), field="integer")
    elif kind == "array":
        scipy_io.mmwrite(path, A)
    else:
        scipy_io.mmwrite(path, sparse.coo_matrix(A))
    got, nz = m.mtx_load(path)
    ref = np.asarray(scipy_io.mmread(path).todense() if kind != "array" else scipy_io.mmread(path), np.float32)
    np.testing.assert_array_equal(got, half_bits(ref))
    assert nz == int(np.count_nonzero(ref))


def test_mtx_bcsr_equals_dense_conversion(tmp_path):
    """Loading into BCSR directly gives the arrays the BCSR constructor builds
    from the densely loaded matrix (blocks of 16x16 and 32x16; rows and columns
    past the last whole block are dropped as the constructor does)."""
    rng = np.random.default_rng(5)
    rows, cols = 120, 200
    keep = np.repeat(np.repeat(rng.uniform(size=(8, 13)) < 0.3, 16, 0), 16, 1)[:rows, :cols]
    A = keep * rng.uniform(-1, 1, (rows, cols)) * (rng.uniform(size=(rows, cols)) < 0.5)
    A[3, 5] = 1e-9                      # rounds to fp16 zero: does not keep its block
    path = os.path.join(str(tmp_path), "b.mtx")
    scipy_io.mmwrite(path, sparse.coo_matrix(A))
    dense, _ = m.mtx_load(path)
    for bR in (16, 32):
        r, c, rp, ci, vals = m.mtx_load_bcsr(path, bR, 16)
        assert (r, c) == (rows, cols)
        hdr, idx, data = oracle.bcsr(dense[:rows - rows % bR, :cols - cols % 16], bR, 16)
        np.testing.assert_array_equal(rp, hdr)
        np.testing.assert_array_equal(ci, idx)
        np.testing.assert_array_equal(vals, data)


def test_mtx_roundtrip_and_errors(tmp_path):
    rng = np.random.default_rng(7)
    A = ((rng.uniform(size=(40, 56)) < 0.2) * rng.uniform(-4, 4, (40, 56))).astype(np.float32)
    A = A + np.float32(0.0)            # -0 is not stored by a sparse format: compare with +0
    path = os.path.join(str(tmp_path), "c.mtx")
    m.mtx_save(path, A)
    got, nz = m.mtx_load(path)
    np.testing.assert_array_equal(got, half_bits(A))
    assert nz == int(np.count_nonzero(A))
    np.testing.assert_allclose(np.asarray(scipy_io.mmread(path).todense()), A, rtol=1e-7)
    bad = os.path.join(str(tmp_path), "bad.mtx")
    with open(bad, "w") as f:
        f.write("%%MatrixMarket matrix coordinate real general\n4 4 1\n5 1 1.0\n")
    with pytest.raises(m.SpmmError):
        m.mtx_load(bad)
    with open(bad, "w") as f:
        f.write("not a matrix\n")
    with pytest.raises(m.SpmmError):
        m.mtx_load(bad)
    with pytest.raises(m.SpmmError):
        m.mtx_load(os.path.join(str(tmp_path), "missing.mtx"))


@pytest.mark.parametrize("dtype", [0, 1, 2, 3])
def test_bcsr_binary_roundtrip(tmp_path, dtype):
    rng = np.random.default_rng(dtype)
    rp, ci = m.gen_structure(256, 512, 64, m.PATTERN_RANDOM, 0.1, 0, seed=4)
    nv = len(ci) * 64 * 16
    vals = rng.integers(0, 255 if dtype == 2 else 65535, nv).astype(np.uint8 if dtype == 2 else np.uint16)
    lo = rng.integers(0, 65535, nv).astype(np.uint16) if dtype == 3 else None
    sc = rng.uniform(0.1, 2, len(ci)).astype(np.float32) if dtype == 2 else None
    path = os.path.join(str(tmp_path), "a.bcsr")
    m.bcsr_save(path, 256, 512, 64, 16, rp, ci, vals, dtype, lo, sc)
    M, K, bR, bC, dt, rp2, ci2, v2, lo2, sc2 = m.bcsr_load(path)
    assert (M, K, bR, bC, dt) == (256, 512, 64, 16, dtype)
    np.testing.assert_array_equal(rp2, rp)
    np.testing.assert_array_equal(ci2, ci)
    np.testing.assert_array_equal(v2, vals)
    if lo is not None:
        np.testing.assert_array_equal(lo2, lo)
    if sc is not None:
        np.testing.assert_array_equal(sc2, sc)
    with open(path, "r+b") as f:
        f.write(b"XXXX")
    with pytest.raises(m.SpmmError):
        m.bcsr_load(path)
