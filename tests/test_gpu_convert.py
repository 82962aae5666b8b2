"""GPU dense -> BCSR conversion, bit-exact to the reference BCSRMatrix ctor
(formats/BCSRMatrix.cu:22-74) restated by the oracle."""
import numpy as np
import pytest
import torch

import matrixmultiplicationcuda_gb300 as m
from oracle import oracle

pytestmark = pytest.mark.gpu


def gpu_convert(A_bits, bR, bC, dev, lda=None):
    M, K = A_bits.shape
    if lda is None:
        t = torch.from_numpy(A_bits.view(np.float16).copy()).to(dev)
    else:
        big = np.zeros((M, lda), np.uint16)
        big[:, :K] = A_bits
        t = torch.from_numpy(big.view(np.float16)).to(dev)[:, :K]
    rp, ci, vals = m.dense_to_bcsr(t, bR, bC)
    torch.cuda.synchronize()
    return rp.cpu().numpy(), ci.cpu().numpy(), vals.cpu().numpy().view(np.uint16)


@pytest.mark.parametrize("bR,bC", [(16, 16), (32, 16), (64, 16), (16, 32), (32, 32), (48, 64)])
@pytest.mark.parametrize("pattern,sp", [("blockrandom", 0.8), ("random", 0.995), ("checkerboard", 0.0),
                                        ("diagonal", 0.0), ("pattern64by16", 0.7)])
def test_bit_exact(dev, bR, bC, pattern, sp):
    A = oracle.f32_to_f16(oracle.generate_matrix(384, 320, sp, pattern, 16, 31))
    exp = oracle.bcsr(A, bR, bC)
    got = gpu_convert(A, bR, bC, dev)
    for g, e in zip(got, exp):
        assert np.array_equal(g, e)


def test_special_values_and_strided_input(dev, golden):
    A = golden["bcsr/special/A"]
    got = gpu_convert(A, 16, 16, dev, lda=72)
    assert np.array_equal(got[0], golden["bcsr/special/hdr"])
    assert np.array_equal(got[1], golden["bcsr/special/idx"])
    assert np.array_equal(got[2], golden["bcsr/special/data"])


def test_c1_structure(dev, golden):
    A = oracle.f32_to_f16(oracle.generate_matrix(1024, 1024, 0.9, "blockrandom", 16, 123))
    rp, ci, vals = gpu_convert(A, 16, 16, dev)
    assert np.array_equal(rp, golden["c1/hdr"]) and np.array_equal(ci, golden["c1/idx"])
    import hashlib
    assert hashlib.sha256(vals.tobytes()).digest() == golden["c1/data_sha256"].tobytes()


def test_empty_full_and_truncated(dev):
    Z = np.zeros((64, 64), np.uint16)
    rp, ci, vals = gpu_convert(Z, 16, 16, dev)
    assert list(rp) == [0] * 5 and len(ci) == 0
    F = np.full((64, 64), 0x3c00, np.uint16)
    rp, ci, vals = gpu_convert(F, 16, 16, dev)
    assert list(rp) == [0, 4, 8, 12, 16]
    # sizes that are not whole blocks are truncated like the ctor (:37-38)
    T = oracle.f32_to_f16(oracle.generate_matrix(100, 90, 0.3, "random", 16, 2))
    exp = oracle.bcsr(T[:, :88].copy(), 16, 16)
    got = gpu_convert(T[:, :88].copy(), 16, 16, dev)
    for g, e in zip(got, exp):
        assert np.array_equal(g, e)


def test_rejects_bad_block_sizes(dev):
    t = torch.zeros((32, 32), dtype=torch.float16, device=dev)
    with pytest.raises(m.SpmmError):
        m.dense_to_bcsr(t, 8, 16)
    with pytest.raises(m.SpmmError):
        m.dense_to_bcsr(t, 16, 24)


def test_large_convert_matches_oracle(dev):
    M = K = 4096
    rp0, ci0 = m.gen_structure(M, K, 64, m.PATTERN_LOGNORMAL, 0.05, 1.5, seed=9)
    vals = m.gen_values(len(ci0), 64, 16, m.DIST_UNIFORM, seed=9).astype(np.float16)
    A = np.zeros((M, K), np.float16)
    blocks = vals.reshape(-1, 64, 16)
    for br in range(len(rp0) - 1):
        for k in range(rp0[br], rp0[br + 1]):
            A[br * 64:(br + 1) * 64, ci0[k] * 16:(ci0[k] + 1) * 16] = blocks[k]
    got = gpu_convert(A.view(np.uint16), 64, 16, dev)
    exp = oracle.bcsr(A.view(np.uint16), 64, 16)
    for g, e in zip(got, exp):
        assert np.array_equal(g, e)
