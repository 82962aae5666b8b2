"""Products at full benchmark sizes, checked through properties that do not
need the oracle's dense multiply: with integer-valued A and B in [-2, 2] every
product and partial sum is exact in fp32 (|C| <= 36 blocks x 16 x 4 << 2^24),
whatever the summation order, so
  * the row sums of C equal A (B 1)   and   * the column sums equal (1^T A) B
exactly. Both right-hand sides are computed in int64 on the host from the BCSR
arrays in a fraction of a second. Every kernel family, schedule and split-K
runs at the headline size (A 16384^2, 64x16 blocks, 2 %, N 512) and at an
8192^2, 16x16, 5 %, N 1024 size."""
import numpy as np
import pytest

import matrixmultiplicationcuda_gb300 as m

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def problem(M, K, bR, density, N, seed):
    rp, ci = m.gen_structure(M, K, bR, m.PATTERN_RANDOM, density, 0, seed=seed)
    rng = np.random.default_rng(seed)
    vals = rng.integers(-2, 3, len(ci) * bR * 16).astype(np.float32)
    B = rng.integers(-2, 3, (K, N)).astype(np.int64)
    return rp, ci, vals, B


def checksums(rp, ci, vals, B, bR):
    """(A (B 1), (1^T A) B) in int64 from the BCSR arrays."""
    blocks = vals.reshape(-1, bR, 16).astype(np.int64)
    MB = len(rp) - 1
    K, N = B.shape
    bsum = B.sum(axis=1).reshape(K // 16, 16)                  # B 1, in 16-row slabs
    per_block = np.einsum("brc,bc->br", blocks, bsum[ci])      # each block's share of its rows' sums
    rows = np.zeros((MB, bR), np.int64)
    np.add.at(rows, np.repeat(np.arange(MB), np.diff(rp)), per_block)
    colA = np.zeros((K // 16, 16), np.int64)
    np.add.at(colA, ci, blocks.sum(axis=1))                    # 1^T A, in 16-column slabs
    return rows.reshape(-1), colA.reshape(-1) @ B


CASES = {
    "headline": (16384, 16384, 64, 0.02, 512, 20240),
    "c2_16x16": (8192, 8192, 16, 0.05, 1024, 77),
}
_cache = {}


def get_case(name):
    if name not in _cache:
        M, K, bR, dens, N, seed = CASES[name]
        rp, ci, vals, B = problem(M, K, bR, dens, N, seed)
        _cache[name] = (rp, ci, vals, B, checksums(rp, ci, vals, B, bR))
    return _cache[name]


@pytest.mark.parametrize("name,cfg", [
    ("headline", None),
    ("headline", m.Config(kernel=2, n_tile=512, acc_buffers=1)),
    ("headline", m.Config(kernel=2, n_tile=256, schedule=1)),
    ("headline", m.Config(kernel=2, n_tile=256, split_k=4)),
    ("headline", m.Config(kernel=3, n_tile=256)),
    ("headline", m.Config(kernel=3, n_tile=512, schedule=1)),
    ("headline", m.Config(kernel=1, n_tile=128, stages=4)),
    ("c2_16x16", None),
    ("c2_16x16", m.Config(kernel=2, n_tile=256, split_k=2)),
    ("c2_16x16", m.Config(kernel=1, n_tile=256, stages=4)),
])
@pytest.mark.parametrize("dtype", ["f16", "bf16"])
def test_full_size_checksums(dev, name, cfg, dtype):
    M, K, bR, dens, N, seed = CASES[name]
    rp, ci, vals, B, (row_sums, col_sums) = get_case(name)
    dt = m.DType.F16 if dtype == "f16" else m.DType.BF16
    tdt = torch.float16 if dtype == "f16" else torch.bfloat16
    A = m.BCSR.from_host(M, K, bR, rp, ci, vals, dt, device=dev)
    Bd = torch.from_numpy(B.astype(np.float32)).to(dev).to(tdt)
    C = torch.full((M, N), float("nan"), dtype=torch.float32, device=dev)
    m.spmm(A, Bd, N=N, C=C, cfg=cfg)
    m.device_error_check()
    Ch = C.cpu().double().numpy()
    assert np.isfinite(Ch).all()
    assert np.array_equal(Ch.sum(axis=1), row_sums.astype(np.float64))
    assert np.array_equal(Ch.sum(axis=0), col_sums.astype(np.float64))
    assert np.array_equal(Ch, np.rint(Ch))                     # every entry an exact integer


def test_full_size_hybrid_plan_checksums(dev):
    """The planned hybrid product at 8192^2 (16x16 blocks at 5 % stored,
    plus about 1 % of scattered entries as CSR), checked the same way."""
    M = K = 8192
    N = 512
    rp, ci, vals, B, _ = get_case("c2_16x16")[:5]
    B = B[:, :N]
    rng = np.random.default_rng(9)
    nnz_rows = rng.binomial(K, 0.01, M)
    crp = np.concatenate([[0], np.cumsum(nnz_rows)]).astype(np.int32)
    ccol = np.concatenate([np.sort(rng.choice(K, n, replace=False)) for n in nnz_rows]).astype(np.int32)
    cval = rng.integers(1, 3, len(ccol)) * rng.choice([-1, 1], len(ccol))
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    A = m.BCSR.from_host(M, K, 16, rp, ci, vals, m.DType.F16, device=dev)
    plan = m.HcsrPlan(A, t(crp), t(ccol), t(cval.astype(np.float16)))
    Bd = t(B.astype(np.float32)).half()
    C = torch.full((M, N), float("nan"), dtype=torch.float32, device=dev)
    plan.run(Bd, N=N, C=C)
    m.device_error_check()
    plan.close()
    rows_b, cols_b = checksums(rp, ci, vals, B, 16)
    bsum = B.sum(axis=1)
    rows_c = np.zeros(M, np.int64)
    np.add.at(rows_c, np.repeat(np.arange(M), nnz_rows), cval * bsum[ccol])
    colA = np.zeros(K, np.int64)
    np.add.at(colA, ccol, cval)
    Ch = C.cpu().double().numpy()
    assert np.array_equal(Ch.sum(axis=1), (rows_b + rows_c).astype(np.float64))
    assert np.array_equal(Ch.sum(axis=0), (cols_b + colA @ B).astype(np.float64))
