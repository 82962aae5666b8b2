"""Elementwise parity at full benchmark sizes against the FP64 oracle product.

* The headline product (A 16384^2, 64x16 blocks, random 2 %, values
  N(0,1) x 10^U[-3,3] per block, B 16384 x 512 N(0,1)) in fp16 and bf16, run
  the way the benchmark runs it: on a per-matrix plan with a 512-column tile
  and one accumulator, as a chain of launches over two problem copies with
  SPMM_RUN_INPUTS_READY (each launch starting under the previous one). Every
  element of C is compared with oracle.bcsr_matmul_f64:
    - of the stored (rounded) values: normwise max and Frobenius relative
      error <= 1e-5 (only the fp32 accumulation order differs);
    - of the exact fp32 inputs: the documented per-type bars (fp16 2e-3,
      bf16 1e-2), which include the storage rounding.
* One 8192^2 product per structure of the sweep (random, band of half-width 8
  block columns, 256 x 256 block-diagonal tiles, log-normal rows with CV 1.5),
  16x16 blocks at 5 %, N 1024, fp16, by the library default and on a plan
  (which stacks the band and block-diagonal rows into 64-row blocks), compared
  with the FP64 product of the stored values on 48 sampled block rows at
  1e-5.
"""
import os

import numpy as np
import pytest

import matrixmultiplicationcuda_gb300 as m
from oracle import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu
THREADS = max(1, min(16, os.cpu_count() or 1))


def _stored(t):
    return t.float().cpu().numpy().astype(np.float64)


@pytest.fixture(scope="module")
def headline():
    M = K = 16384
    N, bR = 512, 64
    rp, ci = m.gen_structure(M, K, bR, m.PATTERN_RANDOM, 0.02, 0, seed=20240)
    vals = m.gen_values(len(ci), bR, 16, m.DIST_SCALED_NORMAL, seed=20241)
    Bf = m.gen_dense(K, N, m.DIST_NORMAL, seed=20242)
    exact = oracle.bcsr_matmul_f64(rp, ci, vals.astype(np.float64), bR, 16, Bf.astype(np.float64), threads=THREADS)
    return M, K, N, bR, rp, ci, vals, Bf, exact


@pytest.mark.parametrize("dtype,bar", [(m.DType.F16, 2e-3), (m.DType.BF16, 1e-2)])
def test_headline_plan_chain_elementwise(dev, headline, dtype, bar):
    M, K, N, bR, rp, ci, vals, Bf, exact = headline
    tdt = torch.float16 if dtype == m.DType.F16 else torch.bfloat16
    copies = []
    for _ in range(2):
        A = m.BCSR.from_host(M, K, bR, rp, ci, vals, dtype, device=dev)
        B = torch.from_numpy(Bf).to(dev).to(tdt)
        copies.append((A, B, torch.full((M, N), float("nan"), dtype=torch.float32, device=dev)))
    plan = m.BcsrPlan(copies[0][0], N, m.Config(kernel=2, n_tile=512, acc_buffers=1))
    torch.cuda.synchronize()          # every input is written before the chain starts
    for i in range(4):                # a chain of flagged launches, alternating copies
        A, B, C = copies[i % 2]
        plan.run(A, B, C=C, inputs_ready=True)
    m.device_error_check()
    plan.close()
    A0 = copies[0][0]
    stored = oracle.bcsr_matmul_f64(rp, ci, _stored(A0.vals), bR, 16, _stored(copies[0][1]), threads=THREADS)
    for A, B, C in copies:
        got = C.cpu().numpy()
        assert np.isfinite(got).all()
        mx, fr = oracle.rel_errors(got, stored)
        assert mx <= 1e-5 and fr <= 1e-5, (mx, fr)
        mx, fr = oracle.rel_errors(got, exact)
        assert mx <= bar and fr <= bar, (mx, fr)


@pytest.mark.parametrize("pattern,param", [(m.PATTERN_RANDOM, 0.0), (m.PATTERN_BAND, 8.0),
                                           (m.PATTERN_BLOCKDIAG, 256.0), (m.PATTERN_LOGNORMAL, 1.5)])
@pytest.mark.parametrize("planned", [False, True])
def test_sweep_structures_at_8192(dev, pattern, param, planned):
    M = K = 8192
    N, bR = 1024, 16
    rp, ci = m.gen_structure(M, K, bR, pattern, 0.05, param, seed=31)
    vals = m.gen_values(len(ci), bR, 16, m.DIST_UNIFORM, seed=32)
    Bf = m.gen_dense(K, N, m.DIST_UNIFORM, seed=33)
    A = m.BCSR.from_host(M, K, bR, rp, ci, vals, m.DType.F16, device=dev)
    B = torch.from_numpy(Bf).to(dev).half()
    C = torch.full((M, N), float("nan"), dtype=torch.float32, device=dev)
    if planned:
        plan = m.BcsrPlan(A, N)
        plan.run(A, B, C=C)
    else:
        m.spmm(A, B, N=N, C=C)
    m.device_error_check()
    if planned:
        plan.close()
    got = C.cpu().numpy()
    assert np.isfinite(got).all()
    MB = M // bR
    rows = np.unique(np.concatenate([np.linspace(0, MB - 1, 40).astype(int),
                                     np.argsort(np.diff(rp))[-8:]]))          # spread + the longest rows
    assert len(rows) >= 32
    sv, sB = _stored(A.vals), _stored(B)
    for r in rows:
        ref = oracle.bcsr_matmul_f64(rp, ci, sv, bR, 16, sB, br0=int(r), br1=int(r) + 1)
        g = got[r * bR:(r + 1) * bR]
        if not ref.any():
            assert not g.any(), r
            continue
        mx, fr = oracle.rel_errors(g, ref)
        assert mx <= 1e-5 and fr <= 1e-5, (r, mx, fr)
