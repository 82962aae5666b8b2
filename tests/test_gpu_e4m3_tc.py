"""The tcgen05 e4m3 kernels (block-scaled kind::mxf8f6f4 MMAs with one
power-of-two scale per block) against the FP64 oracle product.

Two references per product:
  * the FP64 product of the stored values (e4m3 bytes x block scale x B scale):
    e4m3 x e4m3 products are exact in fp32, so only the accumulation differs;
    normwise bar 1e-5;
  * the same product on the mma.sync e4m3 path (kernel 1), which converts e4m3
    to fp16 in registers and scales each block's partial sum: normwise 1e-5.
Covered: every tcgen05 e4m3 instantiation (block heights 16, 32, 64; column
tiles 128, 256, 512; one and two accumulators, one and two CTAs per SM),
partial groups (rows with an odd number of blocks), empty rows, N not a
multiple of 128 (2-D panel copies), split-K, per-matrix plans with split rows
and the inputs-ready chain, the headline size against the exact inputs at the
documented e4m3 bar, and a block scale that is not a power of two (reported
by spmm_device_error_check).
"""
import numpy as np
import pytest
import torch

import matrixmultiplicationcuda_gb300 as m
from oracle import oracle

pytestmark = pytest.mark.gpu


def e4m3_values(q_u8):
    """e4m3 bytes -> float64 (torch's float8_e4m3fn conversion is exact)."""
    return q_u8.view(torch.float8_e4m3fn).float().cpu().numpy().astype(np.float64)


def problem(M, K, N, bR, pattern, density, param, seed, dev, empty_rows=()):
    rp, ci = m.gen_structure(M, K, bR, pattern, density, param, seed=seed)
    if empty_rows:
        keep = np.ones(len(ci), bool)
        for r in empty_rows:
            keep[rp[r]:rp[r + 1]] = False
        counts = np.diff(rp)
        counts[list(empty_rows)] = 0
        rp = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
        ci = ci[keep]
    vals = m.gen_values(len(ci), bR, 16, m.DIST_SCALED_NORMAL, seed=seed + 1)
    Bf = m.gen_dense(K, N, m.DIST_NORMAL, seed=seed + 2)
    A = m.BCSR.from_host(M, K, bR, rp, ci, vals, m.DType.E4M3, device=dev)
    Bq, _, Bs = m.quantize(torch.from_numpy(Bf).to(dev).reshape(-1), m.DType.E4M3)
    Bq = Bq.view(K, N)
    bs = float(Bs[0])
    stored_A = e4m3_values(A.vals).reshape(-1, bR * 16) * A.scales.cpu().numpy()[:, None].astype(np.float64)
    stored = oracle.bcsr_matmul_f64(rp, ci, stored_A.reshape(-1), bR, 16, e4m3_values(Bq) * bs, threads=8)
    exact = oracle.bcsr_matmul_f64(rp, ci, vals.astype(np.float64), bR, 16, Bf.astype(np.float64), threads=8)
    return rp, ci, A, Bq, bs, stored, exact


def run(A, Bq, bs, N, cfg, dev):
    C = torch.full((A.M, N), float("nan"), dtype=torch.float32, device=dev)
    m.spmm(A, Bq, N=N, C=C, cfg=cfg, b_scale=bs)
    m.device_error_check()
    return C.cpu().numpy()


CFGS = [
    (64, m.Config(kernel=2, n_tile=256, acc_buffers=1)),       # two CTAs per SM
    (64, m.Config(kernel=2, n_tile=512, acc_buffers=1)),       # one CTA per SM
    (64, m.Config(kernel=2, n_tile=256, acc_buffers=2)),
    (64, m.Config(kernel=2, n_tile=128, acc_buffers=2)),
    (64, m.Config(kernel=2, n_tile=256, acc_buffers=1, schedule=1)),
    (64, m.Config(kernel=2, n_tile=256, acc_buffers=2, split_k=4)),
    (32, m.Config(kernel=2, n_tile=256)),
    (16, m.Config(kernel=2, n_tile=256)),
]


@pytest.mark.parametrize("bR,cfg", CFGS)
@pytest.mark.parametrize("N", [512, 272])
def test_tc_e4m3_matches_fp64_and_mma(dev, bR, cfg, N):
    M, K = 1024, 2048
    rp, ci, A, Bq, bs, stored, exact = problem(M, K, N, bR, m.PATTERN_LOGNORMAL, 0.05, 1.0, 40 + bR, dev,
                                               empty_rows=(1, 5))
    assert (np.diff(rp) % 2 == 1).any()                         # partial groups occur
    got = run(A, Bq, bs, N, cfg, dev)
    assert np.isfinite(got).all()
    assert np.all(got[bR:2 * bR] == 0) and np.all(got[5 * bR:6 * bR] == 0)
    mx, fr = oracle.rel_errors(got, stored)
    assert mx <= 1e-5 and fr <= 1e-5, (mx, fr)
    mma = run(A, Bq, bs, N, m.Config(kernel=1, n_tile=128, stages=4), dev)
    mx, fr = oracle.rel_errors(got, mma.astype(np.float64))
    assert mx <= 1e-5 and fr <= 1e-5, (mx, fr)
    mx, fr = oracle.rel_errors(got, exact)
    assert mx <= 8e-2 and fr <= 8e-2, (mx, fr)


@pytest.mark.parametrize("pattern,param,cfg", [
    (m.PATTERN_RANDOM, 0.0, m.Config(kernel=2, n_tile=512, acc_buffers=1)),
    (m.PATTERN_LOGNORMAL, 1.5, m.Config(kernel=2, n_tile=256, acc_buffers=1)),   # split rows
    (m.PATTERN_LOGNORMAL, 1.5, m.Config(kernel=2, n_tile=512, acc_buffers=1)),
])
def test_tc_e4m3_plan_chain(dev, pattern, param, cfg):
    M, K, N, bR = 4096, 4096, 512, 64
    rp, ci, A, Bq, bs, stored, exact = problem(M, K, N, bR, pattern, 0.03, param, 77, dev)
    plan = m.BcsrPlan(A, N, cfg)
    torch.cuda.synchronize()
    Cs = [torch.full((M, N), float("nan"), dtype=torch.float32, device=dev) for _ in range(2)]
    for i in range(4):
        plan.run(A, Bq, C=Cs[i % 2], b_scale=bs, inputs_ready=i > 0)
    m.device_error_check()
    plan.close()
    for C in Cs:
        got = C.cpu().numpy()
        mx, fr = oracle.rel_errors(got, stored)
        assert mx <= 1e-5 and fr <= 1e-5, (mx, fr)


def test_tc_e4m3_headline_size(dev):
    """A 16384^2, 64x16 blocks, 2 %, N 512: the stored-value product exactly
    (normwise 1e-5) and the exact inputs at the documented e4m3 bar."""
    M = K = 16384
    rp, ci, A, Bq, bs, stored, exact = problem(M, K, 512, 64, m.PATTERN_RANDOM, 0.02, 0, 20240, dev)
    for cfg in (m.Config(kernel=2, n_tile=256, acc_buffers=1), m.Config(kernel=2, n_tile=512, acc_buffers=1)):
        got = run(A, Bq, bs, 512, cfg, dev)
        mx, fr = oracle.rel_errors(got, stored)
        assert mx <= 1e-5 and fr <= 1e-5, (mx, fr)
        mx, fr = oracle.rel_errors(got, exact)
        assert mx <= 8e-2 and fr <= 8e-2, (mx, fr)


def test_non_power_of_two_scale_is_reported(dev):
    M, K, N, bR = 256, 512, 256, 64
    rp, ci, A, Bq, bs, stored, exact = problem(M, K, N, bR, m.PATTERN_RANDOM, 0.2, 0, 5, dev)
    A.scales[0] *= 1.5
    C = torch.empty((M, N), dtype=torch.float32, device=dev)
    m.spmm(A, Bq, N=N, C=C, cfg=m.Config(kernel=2, n_tile=256, acc_buffers=1), b_scale=bs)
    with pytest.raises(m.SpmmError) as e:
        m.device_error_check()
    assert e.value.status == m.Status.INVALID_ARG
    # the library default for e4m3 stays on mma.sync, which takes any scale
    A.scales[0] /= 1.5
    got = run(A, Bq, bs, N, None, dev)
    mx, fr = oracle.rel_errors(got, stored)
    assert mx <= 1e-5 and fr <= 1e-5
