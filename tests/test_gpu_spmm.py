"""GPU parity of the BCSR SpMM kernels against the oracle (through the C ABI).

Tolerances: fp16 inputs with fp32 accumulation, compared with the restated
reference host multiply at |diff| <= 1e-2 absolute (the reference harness's own
check, nvbench_main.cu:357-364), and with the FP64 product at a normwise
relative error <= 1e-5 (max) / 1e-5 (Frobenius) -- the fp16-rounded inputs are
exact in FP64, so only the fp32 accumulation order differs.
"""
import ctypes

import numpy as np
import pytest
import torch

import matrixmultiplicationcuda_gb300 as m
from oracle import oracle

pytestmark = pytest.mark.gpu


def to_dev(a, dev):
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def make_problem(M, K, N, pattern, sparsity, bs, bR, seedA=123, seedB=456):
    A = oracle.f32_to_f16(oracle.generate_matrix(M, K, sparsity, pattern, bs, seedA))
    B = oracle.f32_to_f16(oracle.generate_matrix(K, N, 0.0, "random", bs, seedB))
    hdr, idx, data = oracle.bcsr(A, bR, 16)
    return A, B, hdr, idx, data


def fp64_ref(hdr, idx, data, bR, B):
    return oracle.bcsr_matmul_f64(hdr, idx, data.view(np.float16).astype(np.float64), bR, 16,
                                  B.view(np.float16).astype(np.float64))


LAUNCH = {16: m.sparseMatrixMulTensor, 32: m.sparseMatrixMulTensor32x16, 64: m.sparseMatrixMulTensor64x16}


def run_ref_shaped(bR, hdr, idx, data, B, M, N, K, dev, poison=True):
    C = torch.full((M, N), float("nan") if poison else 0.0, dtype=torch.float32, device=dev)
    LAUNCH[bR](to_dev(hdr, dev), to_dev(idx, dev), to_dev(data.view(np.float16), dev),
               to_dev(B.view(np.float16), dev), C, M, N, K)
    m.device_error_check()
    return C.cpu().numpy()


def test_c1_workload_matches_host_multiply(dev):
    """1024 x 1024, 16x16 blocks, 10% of blocks (seed 123), B dense (seed 456), N = 1024:
    the exact inputs of the reference harness's prepare_buffers (nvbench_main.cu:139-175)."""
    A, B, hdr, idx, data = make_problem(1024, 1024, 1024, "blockrandom", 0.9, 16, 16)
    got = run_ref_shaped(16, hdr, idx, data, B, 1024, 1024, 1024, dev)
    ref = oracle.cpu_matmul_ref(A, B, threads=8)
    assert np.isfinite(got).all()
    assert float(np.max(np.abs(got - ref))) <= 1e-2
    mx, fr = oracle.rel_errors(got, fp64_ref(hdr, idx, data, 16, B))
    assert mx <= 1e-5 and fr <= 1e-5


@pytest.mark.parametrize("bR,pattern", [(16, "blockrandom"), (32, "pattern32by16"), (64, "pattern64by16")])
@pytest.mark.parametrize("N", [8, 24, 64, 136, 512])
def test_block_shapes_and_widths(dev, bR, pattern, N):
    M, K = 256, 192
    A, B, hdr, idx, data = make_problem(M, K, N, pattern, 0.6, 16, bR, seedA=N + bR)
    got = run_ref_shaped(bR, hdr, idx, data, B, M, N, K, dev)
    ref = oracle.cpu_matmul_ref(A, B)
    assert np.isfinite(got).all()
    assert float(np.max(np.abs(got - ref))) <= 1e-2
    mx, fr = oracle.rel_errors(got, fp64_ref(hdr, idx, data, bR, B))
    assert mx <= 1e-5 and fr <= 1e-5


@pytest.mark.parametrize("bR", [16, 32, 64])
@pytest.mark.parametrize("n_tile,stages", [(64, 4), (128, 4), (128, 8), (256, 4)])
def test_every_mma_config(dev, bR, n_tile, stages):
    M, K, N = 512, 1024, 512
    rp, ci = m.gen_structure(M, K, bR, m.PATTERN_LOGNORMAL, 0.08, 1.5, seed=bR)
    vals = m.gen_values(len(ci), bR, 16, m.DIST_UNIFORM, seed=7)
    A = m.BCSR.from_host(M, K, bR, rp, ci, vals, m.DType.F16)
    Bf = m.gen_dense(K, N, m.DIST_UNIFORM, seed=8)
    Bh = torch.from_numpy(Bf).to(dev).half()
    cfg = m.Config(kernel=1, n_tile=n_tile, stages=stages)
    try:
        C = m.spmm(A, Bh, cfg=cfg)
    except m.SpmmError as e:
        assert e.status == m.Status.UNSUPPORTED
        pytest.skip("config not instantiated")
    m.device_error_check()
    vh = vals.astype(np.float16).astype(np.float64)
    ref = oracle.bcsr_matmul_f64(rp, ci, vh, bR, 16, Bf.astype(np.float16).astype(np.float64))
    mx, fr = oracle.rel_errors(C.cpu().numpy(), ref)
    assert mx <= 1e-5 and fr <= 1e-5


def test_empty_and_degenerate_structures(dev):
    M, K, N = 128, 64, 40
    B = oracle.f32_to_f16(oracle.generate_matrix(K, N, 0.0, "random", 16, 1))
    # no stored blocks at all: C must be all zeros (every C element written)
    hdr = np.zeros(M // 16 + 1, np.int32)
    got = run_ref_shaped(16, hdr, np.zeros(0, np.int32), np.zeros(0, np.uint16), B, M, N, K, dev)
    assert np.array_equal(got, np.zeros((M, N), np.float32))
    # one block; interleaved empty rows; one dense block row; single block row M = bR
    A = np.zeros((M, K), np.float16)
    A[16:32, 32:48] = 1.5
    A[96:112, :] = np.arange(K, dtype=np.float16) / 64
    Ab = A.view(np.uint16)
    hdr, idx, data = oracle.bcsr(Ab, 16, 16)
    got = run_ref_shaped(16, hdr, idx, data, B, M, N, K, dev)
    assert float(np.max(np.abs(got - oracle.cpu_matmul_ref(Ab, B)))) <= 1e-2
    assert np.all(got[:16] == 0) and np.all(got[32:96] == 0)
    hdr1, idx1, data1 = oracle.bcsr(Ab[96:112], 16, 16)
    got = run_ref_shaped(16, hdr1, idx1, data1, B, 16, N, K, dev)
    assert float(np.max(np.abs(got - oracle.cpu_matmul_ref(Ab[96:112], B)))) <= 1e-2


def test_ldc_window_leaves_padding_untouched(dev):
    M, K, N = 128, 128, 48
    A, B, hdr, idx, data = make_problem(M, K, N, "blockrandom", 0.5, 16, 16)
    Abcsr = m.BCSR(M, K, 16, 16, to_dev(hdr, dev), to_dev(idx, dev), to_dev(data.view(np.float16), dev))
    Cbig = torch.full((M, 64), -7.0, dtype=torch.float32, device=dev)
    m.spmm(Abcsr, to_dev(B.view(np.float16), dev), N=N, C=Cbig)
    m.device_error_check()
    got = Cbig.cpu().numpy()
    assert np.all(got[:, N:] == -7.0)
    assert float(np.max(np.abs(got[:, :N] - oracle.cpu_matmul_ref(A, B)))) <= 1e-2


def test_variant_launchers_agree(dev):
    M, K, N = 256, 256, 96
    A, B, hdr, idx, data = make_problem(M, K, N, "blockrandom", 0.7, 16, 16)
    args = [to_dev(hdr, dev), to_dev(idx, dev), to_dev(data.view(np.float16), dev), to_dev(B.view(np.float16), dev)]
    C1 = torch.empty((M, N), device=dev)
    C2 = torch.empty((M, N), device=dev)
    m.sparseMatrixMulTensor(*args, C1, M, N, K)
    m.sparseMatrixMulTensorAdaptive(*args, C2, M, N, 3, K)
    torch.cuda.synchronize()
    assert torch.equal(C1, C2)


VARIANTS = {16: ["sparseMatrixMulTensor_v2_launch", "sparseMatrixMulTensor_v3_launch",
                 "sparseMatrixMulTensor_v1_improved_launch", "sparseMatrixMulTensor_option2_ldmatrix_sm80_launch"],
            32: ["sparseMatrixMulTensor32x16_v2_launch", "sparseMatrixMulTensor32x16_shared_launch",
                 "sparseMatrixMulTensor32x16_shared_vectorized_launch",
                 "sparseMatrixMulTensor32x16_v2_shared_vectorized_launch"],
            64: ["sparseMatrixMulTensor64x16_v2_launch"]}
PATTERN = {16: "blockrandom", 32: "pattern32by16", 64: "pattern64by16"}


@pytest.mark.parametrize("bR", [16, 32, 64])
def test_named_variant_launchers(dev, bR):
    """Every variant name the reference declares (src/cuda_kernels.cuh:47-99) has
    its own C-ABI launcher; each must give the base launcher's result bit for bit
    (the same pipeline runs), and that result must match the host multiply."""
    M, K, N = 256, 256, 96
    A, B, hdr, idx, data = make_problem(M, K, N, PATTERN[bR], 0.7, 16, bR)
    d = [to_dev(hdr, dev), to_dev(idx, dev), to_dev(data.view(np.float16), dev), to_dev(B.view(np.float16), dev)]
    base = torch.empty((M, N), device=dev)
    LAUNCH[bR](*d, base, M, N, K)
    m.device_error_check()
    assert float(np.max(np.abs(base.cpu().numpy() - oracle.cpu_matmul_ref(A, B)))) <= 1e-2
    L = m.lib()
    st = torch.cuda.current_stream().cuda_stream
    for name in VARIANTS[bR]:
        C = torch.full((M, N), float("nan"), device=dev)
        rc = getattr(L, name)(*[ctypes.c_void_p(x.data_ptr()) for x in d + [C]], M, N, K, ctypes.c_void_p(st))
        assert rc == 0, (name, m._lib.last_error())
        m.device_error_check()
        assert torch.equal(C, base), name


def test_square_launcher_tensor1(dev):
    """sparseMatrixMulTensor1 (src/cuda_kernels.cu:330-355) takes one size n for
    square matrices; its launcher gives the base 16x16 launcher's result."""
    n = 256
    A, B, hdr, idx, data = make_problem(n, n, n, "blockrandom", 0.7, 16, 16)
    d = [to_dev(hdr, dev), to_dev(idx, dev), to_dev(data.view(np.float16), dev), to_dev(B.view(np.float16), dev)]
    base = torch.empty((n, n), device=dev)
    LAUNCH[16](*d, base, n, n, n)
    C = torch.full((n, n), float("nan"), device=dev)
    st = torch.cuda.current_stream().cuda_stream
    rc = m.lib().sparseMatrixMulTensor1_launch(*[ctypes.c_void_p(x.data_ptr()) for x in d + [C]], n, ctypes.c_void_p(st))
    assert rc == 0, m._lib.last_error()
    m.device_error_check()
    assert torch.equal(C, base)
    assert float(np.max(np.abs(C.cpu().numpy() - oracle.cpu_matmul_ref(A, B)))) <= 1e-2


@pytest.mark.skipif(not oracle.ref_wmma_available(), reason="reference kernels not built")
@pytest.mark.parametrize("kernel,bR,pattern", [("sparseMatrixMulTensor", 16, "blockrandom"),
                                               ("sparseMatrixMulTensor_v2", 16, "blockrandom"),
                                               ("sparseMatrixMulTensor32x16", 32, "pattern32by16"),
                                               ("sparseMatrixMulTensor64x16", 64, "pattern64by16")])
def test_against_reference_wmma_kernels(dev, kernel, bR, pattern):
    """The reference's own WMMA kernels, built unmodified from its tree, run on the
    same device inputs; both results must agree within the harness tolerance."""
    M, K, N = 512, 512, 256
    A, B, hdr, idx, data = make_problem(M, K, N, pattern, 0.8, 16, bR)
    d = [to_dev(hdr, dev), to_dev(idx, dev), to_dev(data.view(np.float16), dev), to_dev(B.view(np.float16), dev)]
    Cref = torch.zeros((M, N), dtype=torch.float32, device=dev)
    oracle.ref_wmma_launch(kernel, d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(), d[3].data_ptr(),
                           Cref.data_ptr(), M, N, torch.cuda.current_stream().cuda_stream)
    Cnew = torch.empty((M, N), dtype=torch.float32, device=dev)
    LAUNCH[bR](*d, Cnew, M, N, K)
    m.device_error_check()
    diff = float((Cref - Cnew).abs().max())
    assert diff <= 1e-2


def test_validate_structure(dev):
    M, K = 128, 128
    A, B, hdr, idx, data = make_problem(M, K, 32, "blockrandom", 0.5, 16, 16)
    good = m.BCSR(M, K, 16, 16, to_dev(hdr, dev), to_dev(idx, dev), to_dev(data.view(np.float16), dev))
    m.validate(good)
    bad_hdr = hdr.copy()
    bad_hdr[3] = bad_hdr[4] + 1          # row 3 would end before it starts
    with pytest.raises(m.SpmmError) as e:
        m.validate(m.BCSR(M, K, 16, 16, to_dev(bad_hdr, dev), good.col_idx, good.vals))
    assert e.value.status == m.Status.BAD_STRUCTURE
    bad_idx = idx.copy()
    bad_idx[0] = K // 16
    with pytest.raises(m.SpmmError) as e:
        m.validate(m.BCSR(M, K, 16, 16, good.row_ptr, to_dev(bad_idx, dev), good.vals))
    assert e.value.status == m.Status.BAD_STRUCTURE


def test_bounded_wait_gives_up_and_context_survives(dev):
    assert m.debug_wait_timeout(20_000_000) == m.Status.TIMEOUT
    # the context is still usable afterwards
    A, B, hdr, idx, data = make_problem(64, 64, 16, "blockrandom", 0.5, 16, 16)
    got = run_ref_shaped(16, hdr, idx, data, B, 64, 16, 64, dev)
    assert float(np.max(np.abs(got - oracle.cpu_matmul_ref(A, B)))) <= 1e-2
