"""GPU generators against the host generators (same counter-based streams)
and the reference generator's patterns."""
import numpy as np
import pytest

import matrixmultiplicationcuda_gb300 as m
from oracle import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M,K,bR,pattern,dens,param", [
    (2048, 4096, 16, m.PATTERN_RANDOM, 0.05, 0.0), (4096, 2048, 64, m.PATTERN_RANDOM, 0.2, 0.0),
    (2048, 2048, 32, m.PATTERN_BAND, 0.05, 8.0), (8192, 8192, 64, m.PATTERN_BAND, 0.01, 3.0),
    (1024, 4096, 16, m.PATTERN_BLOCKDIAG, 0.0, 256.0), (768, 768, 64, m.PATTERN_BLOCKDIAG, 0.0, 128.0)])
def test_structure_bit_identical_to_host(dev, M, K, bR, pattern, dens, param):
    rp_h, ci_h = m.gen_structure(M, K, bR, pattern, dens, param, seed=17)
    rp_d, ci_d = m.gpu_gen_structure(M, K, bR, pattern, dens, param, seed=17, device=dev)
    np.testing.assert_array_equal(rp_d.cpu().numpy(), rp_h)
    np.testing.assert_array_equal(ci_d.cpu().numpy(), ci_h)


def test_lognormal_structure_matches_host_rowwise(dev):
    """Log-normal row counts use device log / exp: rows whose count agrees with
    the host's (nearly all) hold the same columns, and every row is a valid
    ascending set."""
    M, K, bR = 16384, 16384, 64
    rp_h, ci_h = m.gen_structure(M, K, bR, m.PATTERN_LOGNORMAL, 0.05, 1.5, seed=5)
    rp_d, ci_d = m.gpu_gen_structure(M, K, bR, m.PATTERN_LOGNORMAL, 0.05, 1.5, seed=5, device=dev)
    rp_d, ci_d = rp_d.cpu().numpy(), ci_d.cpu().numpy()
    cnt_h, cnt_d = np.diff(rp_h), np.diff(rp_d)
    same = cnt_h == cnt_d
    assert same.mean() >= 0.99
    for r in np.nonzero(same)[0][:64]:
        np.testing.assert_array_equal(ci_d[rp_d[r]:rp_d[r + 1]], ci_h[rp_h[r]:rp_h[r + 1]])
    for r in range(0, M // bR, 7):
        row = ci_d[rp_d[r]:rp_d[r + 1]]
        assert np.all(np.diff(row) > 0) and (len(row) == 0 or (row[0] >= 0 and row[-1] < K // 16))


def test_values_match_host(dev):
    u_h = m.gen_values(1000, 64, 16, m.DIST_UNIFORM, seed=9)
    u_d = m.gpu_gen_values(1000, 64, 16, m.DIST_UNIFORM, seed=9, device=dev).cpu().numpy()
    np.testing.assert_array_equal(u_d, u_h)
    d_h = m.gen_dense(300, 200, m.DIST_UNIFORM, seed=4)
    d_d = m.gpu_gen_dense(300, 200, m.DIST_UNIFORM, seed=4, device=dev).cpu().numpy()
    np.testing.assert_array_equal(d_d, d_h)
    for dist in (m.DIST_SCALED_NORMAL, m.DIST_NORMAL):
        n_h = m.gen_values(500, 64, 16, dist, seed=3)
        n_d = m.gpu_gen_values(500, 64, 16, dist, seed=3, device=dev).cpu().numpy()
        assert np.mean(n_h == n_d) >= 0.999
        np.testing.assert_allclose(n_d, n_h, rtol=1e-6, atol=0)


@pytest.mark.parametrize("pattern", ["random", "checkerboard", "diagonal", "blockdiagonal", "blockrandom",
                                     "pattern64by16", "pattern32by16"])
def test_reference_patterns(dev, pattern):
    R, Cn, bs, sp = 512, 384, 16, 0.8
    A = m.gpu_generate_matrix(R, Cn, sp, pattern, bs, seed=11, device=dev).float().cpu().numpy()
    nz = A != 0
    assert np.abs(A).max() <= 1.0
    r, c = np.meshgrid(np.arange(R), np.arange(Cn), indexing="ij")
    if pattern == "checkerboard":
        assert np.array_equal(nz, (((r // bs) % 2) ^ ((c // bs) % 2)) == 0)
    elif pattern == "diagonal":
        assert np.array_equal(nz, r == c)
    elif pattern == "blockdiagonal":
        assert np.array_equal(nz, r // bs == c // bs)
    elif pattern == "random":
        assert abs(nz.mean() - (1 - sp)) < 0.01
    else:
        brow = {"blockrandom": bs, "pattern64by16": 64, "pattern32by16": 32}[pattern]
        bcol = bs if pattern == "blockrandom" else 16
        blk = nz.reshape(R // brow, brow, Cn // bcol, bcol).any(axis=(1, 3))
        full = nz.reshape(R // brow, brow, Cn // bcol, bcol).all(axis=(1, 3))
        assert np.array_equal(blk, full)              # kept blocks are dense
        assert abs(blk.mean() - (1 - sp)) < 0.06
    with pytest.raises(m.SpmmError):
        m.gpu_generate_matrix(16, 16, 0.5, "spiral", 16, seed=1, device=dev)


def test_device_only_pipeline(dev):
    """Generate, convert and multiply without a host round trip; the product
    matches an FP64 product of the generated values."""
    A = m.gpu_generate_matrix(1024, 1024, 0.9, "blockrandom", 16, seed=123, device=dev)
    rp, ci, vals = m.dense_to_bcsr(A, 16, 16)
    B = m.gpu_gen_dense(1024, 512, m.DIST_UNIFORM, seed=456, device=dev).half()
    C = m.spmm(m.BCSR(1024, 1024, 16, 16, rp, ci, vals), B)
    m.device_error_check()
    ref = A.double().cpu().numpy() @ B.double().cpu().numpy()
    mx, fr = oracle.rel_errors(C.cpu().numpy(), ref)
    assert mx <= 1e-5 and fr <= 1e-5
