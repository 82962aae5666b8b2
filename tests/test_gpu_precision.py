"""Mixed-precision products against the FP64 host product of the exact
(pre-rounding) values.

Workload: the mixed-precision configuration scaled down -- 64x16 blocks, 2-8 %
block density, block values N(0,1) x 10^u with u ~ U[-3, 3] per block, B N(0,1).
Bars (normwise, max|err|/max|ref| and Frobenius):
  fp16        <= 2e-3   (inputs rounded to 11 significant bits)
  bf16        <= 1e-2   (8 significant bits)
  fp16 hi+lo  <= 2e-6   (about 22 significant bits, fp32 accumulation)
  e4m3 + per-block scales <= 8e-2 (4 significant bits; recorded, above the 1e-2 target)
"""
import numpy as np
import pytest
import torch

import matrixmultiplicationcuda_gb300 as m
from oracle import oracle

pytestmark = pytest.mark.gpu

BARS = {m.DType.F16: 2e-3, m.DType.BF16: 1e-2, m.DType.F16_SPLIT: 2e-6, m.DType.E4M3: 8e-2}


def build(M, K, N, bR, density, seed, dev):
    rp, ci = m.gen_structure(M, K, bR, m.PATTERN_RANDOM, density, 0, seed=seed)
    vals = m.gen_values(len(ci), bR, 16, m.DIST_SCALED_NORMAL, seed=seed + 1)
    B = m.gen_dense(K, N, m.DIST_NORMAL, seed=seed + 2)
    ref = oracle.bcsr_matmul_f64(rp, ci, vals.astype(np.float64), bR, 16, B.astype(np.float64))
    return rp, ci, vals, B, ref


def run(dtype, rp, ci, vals, B, M, K, bR, dev, cfg=None):
    A = m.BCSR.from_host(M, K, bR, rp, ci, vals, dtype, device=dev)
    Bt = torch.from_numpy(B).to(dev)
    Bq, Blo, Bsc = m.quantize(Bt.reshape(-1), dtype)
    Bq = Bq.view(B.shape)
    Blo = Blo.view(B.shape) if Blo is not None else None
    bscale = float(Bsc[0]) if Bsc is not None else 1.0
    C = m.spmm(A, Bq, N=B.shape[1], B_lo=Blo, b_scale=bscale, cfg=cfg)
    m.device_error_check()
    return C.cpu().numpy()


@pytest.mark.parametrize("dtype", [m.DType.F16, m.DType.BF16, m.DType.F16_SPLIT, m.DType.E4M3])
@pytest.mark.parametrize("bR", [16, 32, 64])
def test_precision_bars(dev, dtype, bR):
    M, K, N = 1024, 2048, 256
    rp, ci, vals, B, ref = build(M, K, N, bR, 0.04, 100 + bR, dev)
    got = run(dtype, rp, ci, vals, B, M, K, bR, dev)
    mx, fr = oracle.rel_errors(got, ref)
    assert np.isfinite(got).all()
    assert mx <= BARS[dtype] and fr <= BARS[dtype], (dtype.name, mx, fr)


def test_precisions_order(dev):
    M, K, N = 1024, 4096, 128
    rp, ci, vals, B, ref = build(M, K, N, 64, 0.02, 7, dev)
    errs = {d: oracle.rel_errors(run(d, rp, ci, vals, B, M, K, 64, dev), ref)[1] for d in BARS}
    assert errs[m.DType.F16_SPLIT] < errs[m.DType.F16] < errs[m.DType.BF16] < errs[m.DType.E4M3]


def test_quantize_e4m3_scales(dev):
    x = torch.tensor([[0.0] * 16, [1.0] * 15 + [-448.0 * 3]], device=dev).reshape(-1)
    q, lo, sc = m.quantize(x, m.DType.E4M3, block_elems=16)
    torch.cuda.synchronize()
    # the smallest power of two >= max / 448: 1344 / 448 = 3 -> 4
    assert sc.cpu().tolist() == [1.0, 4.0]
    assert q.cpu().numpy()[31] == torch.tensor([-336.0]).to(torch.float8_e4m3fn).view(torch.uint8).item()
    y = torch.tensor([448.0, 0.5, -300.0, 1e-3, 448.0 * 2 ** 20, 3e-38, 2.0 ** -20 * 448, 7.0], device=dev)
    _, _, sc = m.quantize(y, m.DType.E4M3, block_elems=1)
    want = [1.0, 2.0 ** -9, 1.0, 2.0 ** -18, 2.0 ** 20, 2.0 ** -126, 2.0 ** -20, 2.0 ** -6]
    assert sc.cpu().tolist() == want


@pytest.mark.parametrize("count,offset", [(4096, 0), (4099, 0), (1003, 1), (257, 3), (3, 0)])
def test_quantize_matches_torch_rounding(dev, count, offset):
    """The conversions are round-to-nearest-even, element by element, whether
    they take the 16-byte path (aligned, four at a time) or the scalar one
    (misaligned source or the last count % 4 values)."""
    base = (torch.randn(count + offset + 8, device=dev) * 37.0)
    x = base[offset:offset + count]
    h, lo, _ = m.quantize(x, m.DType.F16_SPLIT)
    ref_h = x.half()
    assert torch.equal(h.view(torch.int16), ref_h.view(torch.int16))
    assert torch.equal(lo.view(torch.int16), (x - ref_h.float()).half().view(torch.int16))
    b, _, _ = m.quantize(x, m.DType.BF16)
    assert torch.equal(b.view(torch.int16), x.bfloat16().view(torch.int16))
    q, _, sc = m.quantize(x, m.DType.E4M3, block_elems=64)
    scales = sc.repeat_interleave(64)[:count]
    ref_q = (x / scales).to(torch.float8_e4m3fn).view(torch.uint8)
    assert torch.equal(q, ref_q)


def test_quantize_single_large_scale_block(dev):
    """One scale over many elements (how B is scaled for e4m3): the chunked
    reduction finds the exact maximum."""
    x = torch.randn(3_000_001, device=dev)
    x[1_234_567] = -99.5
    _, _, sc = m.quantize(x, m.DType.E4M3, block_elems=x.numel())
    assert sc.numel() == 1 and float(sc[0]) == 0.25     # 99.5 / 448 = 0.222 -> 2^-2
