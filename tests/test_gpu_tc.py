"""The tcgen05 (UMMA + TMEM) pipeline against the FP64 oracle, every
instantiated (block height, column tile, precision), including empty block
rows, partial column tiles and poisoned outputs.

Bars: fp16 / bf16 inputs rounded first, so the FP64 product of the rounded
values is the reference and only fp32 accumulation order differs:
normwise error <= 1e-5. Split fp16 hi+lo against the fp32 values: <= 2e-6.
Rows of ~50 blocks (K = 4096 at 20 %) accumulate ~800 terms in fp32: <= 3e-5.
"""
import numpy as np
import pytest
import torch

import matrixmultiplicationcuda_gb300 as m
from oracle import oracle

pytestmark = pytest.mark.gpu

CASES = [(64, 128, "f16", 2), (64, 256, "f16", 2), (64, 512, "f16", 1), (64, 512, "f16", 2),
         (32, 256, "f16", 2), (32, 512, "f16", 1), (16, 256, "f16", 2), (16, 512, "f16", 1),
         (64, 128, "bf16", 2), (64, 256, "bf16", 2), (64, 512, "bf16", 1), (64, 512, "bf16", 2),
         (32, 256, "bf16", 2), (16, 512, "bf16", 1),
         (64, 256, "split", 2), (64, 128, "split", 2), (64, 512, "split", 1)]
DT = {"f16": m.DType.F16, "bf16": m.DType.BF16, "split": m.DType.F16_SPLIT}


def rounded(x, name):
    t = torch.from_numpy(x)
    if name == "f16":
        return t.half().double().numpy()
    if name == "bf16":
        return t.bfloat16().double().numpy()
    return x.astype(np.float64)


@pytest.mark.parametrize("bR,nt,name,acc", CASES)
@pytest.mark.parametrize("N,K,dens,queue", [(64, 1024, 0.06, 1), (200, 1024, 0.06, 1), (512, 1024, 0.06, 0),
                                            (512, 4096, 0.2, 1)])
def test_tc_matches_fp64(dev, bR, nt, name, acc, N, K, dens, queue):
    """K = 4096 at 20 % gives rows of ~50 blocks: index chunks of 32 and partial
    A groups at row ends; queue=1 takes items from the work queue."""
    N = N - N % 8
    M = 512
    rp, ci = m.gen_structure(M, K, bR, m.PATTERN_LOGNORMAL, dens, 1.5, seed=bR + N)
    vals = m.gen_values(len(ci), bR, 16, m.DIST_UNIFORM, seed=3)
    Bf = m.gen_dense(K, N, m.DIST_UNIFORM, seed=4)
    A = m.BCSR.from_host(M, K, bR, rp, ci, vals, DT[name], device=dev)
    Bq, Blo, _ = m.quantize(torch.from_numpy(Bf).to(dev).reshape(-1), DT[name])
    C = torch.full((M, N), float("nan"), dtype=torch.float32, device=dev)
    m.spmm(A, Bq.view(K, N), N=N, C=C, B_lo=Blo.view(K, N) if Blo is not None else None,
           cfg=m.Config(kernel=2, n_tile=nt, acc_buffers=acc, schedule=queue))
    m.device_error_check()
    got = C.cpu().numpy()
    ref = oracle.bcsr_matmul_f64(rp, ci, rounded(vals, name), bR, 16, rounded(Bf, name))
    assert np.isfinite(got).all()
    mx, fr = oracle.rel_errors(got, ref)
    # fp32 accumulation over ~16 x blocks-per-row terms sets the floor: the
    # K = 4096, 20 % rows sum ~800 products
    bar = (2e-6 if name == "split" else 1e-5) if K <= 1024 else 3e-5
    assert mx <= bar and fr <= bar, (mx, fr)
    empty = np.nonzero(np.diff(rp) == 0)[0]
    for br in empty[:4]:
        assert np.all(got[br * bR:(br + 1) * bR] == 0)


@pytest.mark.parametrize("queue", [0, 1])
def test_tc_short_rows_repeated(dev, queue):
    """Rows of zero to two blocks, launched back to back: most groups hold one
    block, so some B-panel issuers copy nothing for long stretches. Every launch
    must finish without a timed-out pipeline wait and match the FP64 oracle."""
    M, K, N, bR = 4096, 2048, 256, 16
    rp, ci = m.gen_structure(M, K, bR, m.PATTERN_RANDOM, 0.006, 0.0, seed=77)
    vals = m.gen_values(len(ci), bR, 16, m.DIST_UNIFORM, seed=78)
    Bf = m.gen_dense(K, N, m.DIST_UNIFORM, seed=79)
    A = m.BCSR.from_host(M, K, bR, rp, ci, vals, m.DType.F16, device=dev)
    B = torch.from_numpy(Bf).to(dev).half()
    C = torch.empty((M, N), dtype=torch.float32, device=dev)
    for _ in range(40):
        m.spmm(A, B, N=N, C=C, cfg=m.Config(kernel=2, n_tile=256, acc_buffers=2, schedule=queue))
    m.device_error_check()
    ref = oracle.bcsr_matmul_f64(rp, ci, rounded(vals, "f16"), bR, 16, rounded(Bf, "f16"))
    mx, fr = oracle.rel_errors(C.cpu().numpy(), ref)
    assert mx <= 1e-5 and fr <= 1e-5, (mx, fr)


@pytest.mark.parametrize("bR,nt,name,acc", [(64, 256, "f16", 2), (64, 512, "f16", 1), (32, 256, "bf16", 2),
                                            (16, 512, "f16", 1), (64, 256, "split", 2)])
@pytest.mark.parametrize("split,queue", [(2, 0), (3, 1), (8, 1), (16, 0)])
def test_tc_split_k(dev, bR, nt, name, acc, split, queue):
    """Split-K: each block row's blocks spread over `split` items whose partial
    products are added into a zeroed C. Rows of 0 to ~200 blocks, so some
    slices are empty and some end in a partial group."""
    M, K, N = 512, 8192, 256
    rp, ci = m.gen_structure(M, K, bR, m.PATTERN_LOGNORMAL, 0.2, 1.5, seed=bR + split)
    vals = m.gen_values(len(ci), bR, 16, m.DIST_UNIFORM, seed=5)
    Bf = m.gen_dense(K, N, m.DIST_UNIFORM, seed=6)
    A = m.BCSR.from_host(M, K, bR, rp, ci, vals, DT[name], device=dev)
    Bq, Blo, _ = m.quantize(torch.from_numpy(Bf).to(dev).reshape(-1), DT[name])
    C = torch.full((M, N), float("nan"), dtype=torch.float32, device=dev)
    m.spmm(A, Bq.view(K, N), N=N, C=C, B_lo=Blo.view(K, N) if Blo is not None else None,
           cfg=m.Config(kernel=2, n_tile=nt, acc_buffers=acc, schedule=queue, split_k=split))
    m.device_error_check()
    got = C.cpu().numpy()
    ref = oracle.bcsr_matmul_f64(rp, ci, rounded(vals, name), bR, 16, rounded(Bf, name))
    mx, fr = oracle.rel_errors(got, ref)
    assert np.isfinite(got).all()
    assert mx <= 3e-5 and fr <= 3e-5, (mx, fr)
    for br in np.nonzero(np.diff(rp) == 0)[0][:4]:
        assert np.all(got[br * bR:(br + 1) * bR] == 0)


TC64_CASES = [(256, "f16", 5), (256, "f16", 8), (512, "f16", 5), (512, "f16", 4), (256, "bf16", 5),
              (512, "bf16", 4), (256, "split", 5), (512, "split", 2)]


@pytest.mark.parametrize("nt,name,stages", TC64_CASES)
@pytest.mark.parametrize("N,K,dens,queue,split", [(64, 1024, 0.06, 1, 1), (200, 1024, 0.06, 0, 1),
                                                  (512, 1024, 0.06, 0, 1), (512, 4096, 0.2, 1, 1),
                                                  (512, 8192, 0.2, 1, 1)])
def test_tc64_matches_fp64(dev, nt, name, stages, N, K, dens, queue, split):
    """The 64-row pipeline with M = 64 UMMAs (kernel 3): partial column tiles,
    N not a multiple of 64 (2-D panel copies), rows of ~400 blocks, the work
    queue."""
    M, bR = 512, 64
    rp, ci = m.gen_structure(M, K, bR, m.PATTERN_LOGNORMAL, dens, 1.5, seed=N + K + nt)
    vals = m.gen_values(len(ci), bR, 16, m.DIST_UNIFORM, seed=3)
    Bf = m.gen_dense(K, N, m.DIST_UNIFORM, seed=4)
    A = m.BCSR.from_host(M, K, bR, rp, ci, vals, DT[name], device=dev)
    Bq, Blo, _ = m.quantize(torch.from_numpy(Bf).to(dev).reshape(-1), DT[name])
    C = torch.full((M, N), float("nan"), dtype=torch.float32, device=dev)
    m.spmm(A, Bq.view(K, N), N=N, C=C, B_lo=Blo.view(K, N) if Blo is not None else None,
           cfg=m.Config(kernel=3, n_tile=nt, stages=stages, schedule=queue, split_k=split))
    m.device_error_check()
    got = C.cpu().numpy()
    ref = oracle.bcsr_matmul_f64(rp, ci, rounded(vals, name), bR, 16, rounded(Bf, name))
    assert np.isfinite(got).all()
    mx, fr = oracle.rel_errors(got, ref)
    # split: fp32 accumulation over ~1000 products per output (sqrt(1000) x 2^-24
    # ~ 2e-6); the M = 64 instructions sum in another order than M = 128
    bar = (5e-6 if name == "split" else 1e-5) if K <= 1024 else 3e-5
    assert mx <= bar and fr <= bar, (mx, fr)
    for br in np.nonzero(np.diff(rp) == 0)[0][:4]:
        assert np.all(got[br * bR:(br + 1) * bR] == 0)
