"""The CPU oracle pinned against fixtures written by the reference's own code."""
import hashlib

import numpy as np
import pytest

from oracle import oracle


def _gen_keys(golden):
    return [k for k in golden.files if k.startswith("gen/")]


def test_generator_matches_reference(golden):
    keys = _gen_keys(golden)
    assert len(keys) == 21
    for k in keys:
        _, pat, spec = k.split("/")
        r, c, sp, bs, seed = spec.split("_")
        got = oracle.generate_matrix(int(r), int(c), float(sp), pat, int(bs), int(seed))
        assert np.array_equal(got.view(np.uint32), golden[k]), k


def test_unknown_pattern_rejected():
    with pytest.raises(ValueError):
        oracle.generate_matrix(16, 16, 0.5, "spiral", 16, 1)


def test_float_to_half_matches_reference(golden):
    x = golden["f16/in"].view(np.float32)
    assert np.array_equal(oracle.f32_to_f16(x), golden["f16/out"])
    # and back: every finite half maps to the float numpy gives it
    h = np.arange(0, 1 << 16, dtype=np.uint32).astype(np.uint16)
    f = oracle.f16_to_f32(h)
    fin = np.isfinite(h.view(np.float16))
    assert np.array_equal(f[fin], h.view(np.float16)[fin].astype(np.float32))


def test_bcsr_matches_reference(golden):
    keys = sorted({k.rsplit("/", 1)[0] for k in golden.files if k.startswith("bcsr/") and k.endswith("/hdr")})
    assert len(keys) >= 5
    for key in keys:
        A = golden[key + "/A"]
        if key.endswith("special"):
            bR = bC = 16
        else:
            bR, bC = (int(x) for x in key.split("/")[-1].split("_")[2:4])
        hdr, idx, data = oracle.bcsr(A, bR, bC)
        assert np.array_equal(hdr, golden[key + "/hdr"]), key
        assert np.array_equal(idx, golden[key + "/idx"]), key
        assert np.array_equal(data, golden[key + "/data"]), key
        if key + "/nonZeros" in golden.files:
            assert int(golden[key + "/nonZeros"][0]) == len(idx) * bR * bC


def test_bcsr_special_values(golden):
    # a block of only -0 is dropped; NaN, subnormal and -inf blocks are kept
    hdr = golden["bcsr/special/hdr"]
    idx = golden["bcsr/special/idx"]
    assert list(hdr) == [0, 1, 3]
    assert list(idx) == [1, 2, 3]


def test_bcsr_rejects_block_sizes(golden):
    assert list(golden["bcsr/reject"]) == [1, 1]
    A = golden["bcsr/special/A"]
    assert oracle.bcsr(A, 8, 16) is None
    assert oracle.bcsr(A, 16, 24) is None


def test_c1_workload_structure(golden):
    A = oracle.f32_to_f16(oracle.generate_matrix(1024, 1024, 0.9, "blockrandom", 16, 123))
    hdr, idx, data = oracle.bcsr(A, 16, 16)
    assert np.array_equal(hdr, golden["c1/hdr"])
    assert np.array_equal(idx, golden["c1/idx"])
    assert hashlib.sha256(data.tobytes()).digest() == golden["c1/data_sha256"].tobytes()
    B = oracle.f32_to_f16(oracle.generate_matrix(1024, 1024, 0.0, "random", 16, 456))
    assert hashlib.sha256(B.tobytes()).digest() == golden["c1/B_sha256"].tobytes()


def test_metrics_match_reference(golden):
    a, b = golden["metrics/a"], golden["metrics/b"]
    md, ar, rm = golden["metrics/values"]
    assert oracle.maxdiff(a, b) == pytest.approx(md, rel=1e-6)
    assert oracle.avgrelerr(a, b) == pytest.approx(ar, rel=1e-6)
    assert oracle.rmse(a, b) == pytest.approx(rm, rel=1e-12)


def test_cpu_matmul_ref_small_exact():
    # integer-valued fp16 inputs: every product and partial sum is exact in fp32
    rng = np.random.default_rng(0)
    A = rng.integers(-3, 4, (48, 64)).astype(np.float16)
    B = rng.integers(-3, 4, (64, 40)).astype(np.float16)
    C = oracle.cpu_matmul_ref(A.view(np.uint16), B.view(np.uint16))
    assert np.array_equal(C, A.astype(np.float32) @ B.astype(np.float32))
    C2 = oracle.cpu_matmul_ref(A.view(np.uint16), B.view(np.uint16), 8, 40, threads=3)
    assert np.array_equal(C2, C[8:40])


def test_fp64_bcsr_product_matches_dense():
    rng = np.random.default_rng(1)
    A = (rng.standard_normal((64, 48)) * (rng.random((64, 48)) < 0.3)).astype(np.float16)
    hdr, idx, data = oracle.bcsr(A.view(np.uint16), 16, 16)
    B = rng.standard_normal((48, 24))
    vals = data.view(np.float16).astype(np.float64)
    C = oracle.bcsr_matmul_f64(hdr, idx, vals, 16, 16, B)
    np.testing.assert_allclose(C, A.astype(np.float64) @ B, rtol=0, atol=1e-12)
    mx, fr = oracle.rel_errors(C.astype(np.float32), C)
    assert mx < 1e-6 and fr < 1e-6


def test_block_sparse_host_baseline_exact():
    """The block-sparse host multiply (the bench's all-core CPU baseline) on
    integer-valued inputs, where every sum is exact in fp32, and its row split."""
    rng = np.random.default_rng(2)
    A = (rng.integers(-3, 4, (128, 96)) * (rng.random((128, 96)) < 0.2)).astype(np.float16)
    hdr, idx, data = oracle.bcsr(A.view(np.uint16), 32, 16)
    B = rng.integers(-3, 4, (96, 40)).astype(np.float32)
    want = A.astype(np.float32) @ B
    for threads in (1, 3):
        C = oracle.bcsr_matmul_f32_mt(hdr, idx, data, 32, B, threads=threads)
        assert np.array_equal(C, want)
    assert np.array_equal(oracle.bcsr_matmul_f32_mt(hdr, idx, data, 32, B, 1, 3, threads=2), want[32:96])


@pytest.mark.skipif(oracle.ref_lib() is None, reason="reference tree not built here")
def test_oracle_against_live_reference_build():
    R = oracle.ref_lib()
    import ctypes
    for seed in (1, 99):
        for pat, bs in (("blockrandom", 16), ("pattern64by16", 16), ("checkerboard", 32)):
            m = np.empty((192, 160), np.float32)
            R.ref_generate_matrix(192, 160, 0.75, pat.encode(), bs, seed, ctypes.c_void_p(m.ctypes.data))
            assert np.array_equal(m, oracle.generate_matrix(192, 160, 0.75, pat, bs, seed))
