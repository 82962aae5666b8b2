"""Batched uneven products (spmm_batch_plan_create / spmm_batch_run) against
the FP64 oracle, CUDA-graph replay, and the 64-problem workload against 64
sequential single-product launches."""
import numpy as np
import pytest

import matrixmultiplicationcuda_gb300 as m
from oracle import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def rounded(x, name):
    t = torch.from_numpy(np.ascontiguousarray(x))
    return (t.half() if name == "f16" else t.bfloat16()).double().numpy()


def upload(M, K, bR, rp, ci, vals, Bf, dtype, dev):
    A = m.BCSR.from_host(M, K, bR, rp, ci, vals, dtype, device=dev)
    tdt = torch.float16 if dtype == m.DType.F16 else torch.bfloat16
    B = torch.from_numpy(Bf).to(dev).to(tdt).contiguous()
    C = torch.full((M, Bf.shape[1]), float("nan"), dtype=torch.float32, device=dev)
    return A, B, C


# (M, K, bR, pattern, density, param, N): every block height, column counts
# that are and are not multiples of 64 / 128 / 256, rows with no blocks
# (log-normal counts with CV 2), rows longer than one 32-index chunk.
SMALL = [
    (512, 1024, 64, m.PATTERN_RANDOM, 0.06, 0.0, 512),
    (256, 512, 32, m.PATTERN_LOGNORMAL, 0.1, 2.0, 128),
    (1024, 2048, 16, m.PATTERN_BAND, 0.05, 8.0, 256),
    (768, 768, 64, m.PATTERN_BLOCKDIAG, 0.0, 128.0, 200),
    (640, 4096, 32, m.PATTERN_RANDOM, 0.2, 0.0, 64),
    (128, 256, 16, m.PATTERN_RANDOM, 0.3, 0.0, 384),
    (512, 512, 64, m.PATTERN_LOGNORMAL, 0.05, 2.0, 136),
    (320, 1024, 16, m.PATTERN_LOGNORMAL, 0.02, 2.0, 512),
]


def build_small(dev, name, specs=SMALL, seed=0):
    dtype = m.DType.F16 if name == "f16" else m.DType.BF16
    probs, host = [], []
    for i, (M, K, bR, pat, dens, param, N) in enumerate(specs):
        rp, ci = m.gen_structure(M, K, bR, pat, dens, param, seed=seed + 11 * i + 1)
        vals = m.gen_values(len(ci), bR, 16, m.DIST_UNIFORM, seed=seed + 11 * i + 2)
        Bf = m.gen_dense(K, N, m.DIST_UNIFORM, seed=seed + 11 * i + 3)
        probs.append(upload(M, K, bR, rp, ci, vals, Bf, dtype, dev))
        host.append((rp, ci, vals, Bf, bR))
    return probs, host


def check_fp64(probs, host, name, bar=3e-5):
    for i, ((A, B, C), (rp, ci, vals, Bf, bR)) in enumerate(zip(probs, host)):
        got = C.cpu().numpy()
        assert np.isfinite(got).all(), i
        ref = oracle.bcsr_matmul_f64(rp, ci, rounded(vals, name), bR, 16, rounded(Bf, name))
        mx, fr = oracle.rel_errors(got, ref)
        assert mx <= bar and fr <= bar, (i, mx, fr)
        for br in np.nonzero(np.diff(rp) == 0)[0][:4]:
            assert np.all(got[br * bR:(br + 1) * bR] == 0), (i, br)


@pytest.mark.parametrize("name", ["f16", "bf16"])
@pytest.mark.parametrize("stages,n_tile", [(0, 0), (4, 0), (8, 0), (0, 128), (0, 256)])
def test_batch_matches_fp64(dev, name, stages, n_tile):
    probs, host = build_small(dev, name)
    plan = m.BatchPlan(probs, cfg=m.Config(stages=stages, n_tile=n_tile))
    plan.run()
    m.device_error_check()
    check_fp64(probs, host, name)
    plan.close()


def test_batch_graph_replay(dev):
    """The launch replays from a CUDA graph: the queue is reset by the launch
    itself, and results are bitwise those of the eager launch (each item is
    reduced by one CTA in a fixed order)."""
    probs, host = build_small(dev, "f16", seed=5)
    plan = m.BatchPlan(probs)
    plan.run()
    torch.cuda.synchronize()
    eager = [C.clone() for _, _, C in probs]
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        plan.run()
    for _ in range(3):
        for _, _, C in probs:
            C.fill_(float("nan"))
        g.replay()
        torch.cuda.synchronize()
        m.device_error_check()
        for (_, _, C), e in zip(probs, eager):
            assert torch.equal(C, e)
    check_fp64(probs, host, "f16")
    plan.close()


def test_batch_empty_and_degenerate(dev):
    """Problems with no stored blocks, no rows or no columns: C rows are
    written as zeros where they exist, and nothing else is touched."""
    specs = [(256, 512, 64, m.PATTERN_RANDOM, 0.0, 0.0, 128),
             (512, 1024, 16, m.PATTERN_RANDOM, 0.05, 0.0, 256)]
    probs, host = build_small(dev, "f16", specs=specs, seed=9)
    A0 = m.BCSR(0, 64, 16, 16, torch.zeros(1, dtype=torch.int32, device=dev),
                torch.zeros(0, dtype=torch.int32, device=dev),
                torch.zeros(0, dtype=torch.float16, device=dev))
    B0 = torch.zeros((64, 128), dtype=torch.float16, device=dev)
    C0 = torch.zeros((0, 128), dtype=torch.float32, device=dev)
    plan = m.BatchPlan(probs + [(A0, B0, C0)])
    plan.run()
    m.device_error_check()
    check_fp64(probs, host, "f16")
    assert torch.all(probs[0][2] == 0)
    plan.close()


def test_batch_rejects_bad_problems(dev):
    probs, _ = build_small(dev, "f16", specs=SMALL[:2])
    A, B, C = probs[1]
    A_b = m.BCSR(A.M, A.K, A.bR, A.bC, A.row_ptr, A.col_idx, A.vals.view(torch.bfloat16), m.DType.BF16)
    with pytest.raises(m.SpmmError) as e:
        m.BatchPlan([probs[0], (A_b, B, C)])
    assert e.value.status == m.Status.INVALID_ARG
    with pytest.raises(m.SpmmError) as e:
        m.BatchPlan(probs, cfg=m.Config(n_tile=512))
    assert e.value.status == m.Status.UNSUPPORTED
    bad_rp = A.row_ptr.clone()
    bad_rp[1] = bad_rp[2] + 1     # not monotone
    A_bad = m.BCSR(A.M, A.K, A.bR, A.bC, bad_rp, A.col_idx, A.vals)
    with pytest.raises(m.SpmmError) as e:
        m.BatchPlan([(A_bad, B, C)])
    assert e.value.status == m.Status.BAD_STRUCTURE


def test_uneven_64_matches_sequential(dev):
    """The 64-problem uneven workload in one launch equals 64 sequential
    single-product launches (same fp32 accumulation, possibly another order),
    and a slice of every problem matches the FP64 oracle."""
    specs = m.uneven_batch_specs(64, seed=2024)
    probs, host = [], []
    for sp in specs:
        rp, ci, vals, Bf = m.make_problem(sp)
        probs.append(upload(sp["M"], sp["K"], sp["bR"], rp, ci, vals, Bf, m.DType.F16, dev))
        host.append((rp, ci, vals, Bf, sp["bR"]))
    plan = m.BatchPlan(probs)
    plan.run()
    m.device_error_check()
    seq = []
    for A, B, _ in probs:
        seq.append(m.spmm(A, B))
    torch.cuda.synchronize()
    m.device_error_check()
    for i, ((A, B, C), S) in enumerate(zip(probs, seq)):
        assert torch.isfinite(C).all(), i
        scale = max(float(S.abs().max()), 1e-30)
        assert float((C - S).abs().max()) / scale <= 3e-5, i
    for i, ((A, B, C), (rp, ci, vals, Bf, bR)) in enumerate(zip(probs, host)):
        br1 = min(len(rp) - 1, 8)
        ref = oracle.bcsr_matmul_f64(rp, ci, rounded(vals, "f16"), bR, 16, rounded(Bf, "f16"), 0, br1)
        got = C[:br1 * bR].cpu().numpy()
        mx, fr = oracle.rel_errors(got, ref)
        assert mx <= 5e-5 and fr <= 5e-5, (i, mx, fr)
    plan.close()


def test_batch_short_rows_repeated(dev):
    """Mostly one-block rows (B-panel issuers idle for long stretches), replayed
    many times: no pipeline wait may time out."""
    specs = [(4096, 2048, 16, m.PATTERN_RANDOM, 0.006, 0.0, 256),
             (2048, 2048, 32, m.PATTERN_RANDOM, 0.01, 0.0, 128)]
    probs, host = build_small(dev, "f16", specs=specs, seed=21)
    plan = m.BatchPlan(probs)
    for _ in range(40):
        plan.run()
    m.device_error_check()
    check_fp64(probs, host, "f16", bar=1e-5)
    plan.close()


@pytest.mark.parametrize("seed", [3, 5, 9])
def test_batch_random_mixes(dev, seed):
    """Seeded random batches: 1-24 products of random block height, shape,
    structure, density and N (a multiple of 8), in fp16 or bf16, on a random
    ring depth and column tile; two runs of one plan, each against FP64."""
    rng = np.random.default_rng(seed)
    name = ["f16", "bf16"][seed % 2]
    pats = [(m.PATTERN_RANDOM, 0.0), (m.PATTERN_BAND, 4.0), (m.PATTERN_LOGNORMAL, 1.5), (m.PATTERN_BLOCKDIAG, 64.0)]
    specs = []
    for _ in range(int(rng.integers(1, 25))):
        bR = int(rng.choice([16, 32, 64]))
        pat, param = pats[int(rng.integers(len(pats)))]
        M = int(rng.integers(1, 24)) * 64
        K = int(rng.integers(1, 40)) * 64
        specs.append((M, K, bR, pat, float(rng.choice([0.02, 0.1, 0.4])), param, int(rng.integers(1, 64)) * 8))
    probs, host = build_small(dev, name, specs=specs, seed=100 * seed)
    cfg = m.Config(stages=int(rng.choice([0, 4, 8])), n_tile=int(rng.choice([0, 128, 256])))
    plan = m.BatchPlan(probs, cfg=cfg)
    for _ in range(2):
        for (_, _, C) in probs:
            C.fill_(float("nan"))
        plan.run()
        m.device_error_check()
        check_fp64(probs, host, name)
    plan.close()


def test_batch_stacks_shared_column_problems(dev):
    """16- and 32-row band and block-diagonal problems run stacked into 64-row
    blocks over the union of their rows' columns; random ones and 64-row ones
    run as they are. Every product matches FP64 over two runs, and after new
    values are written into the stacked problems' A (every run reads the
    member blocks from A's own values)."""
    specs = [
        (1024, 1024, 16, m.PATTERN_BAND, 0.1, 6.0, 256),       # stacks
        (1024, 1024, 32, m.PATTERN_BLOCKDIAG, 0.0, 128.0, 128),  # stacks
        (1024, 2048, 16, m.PATTERN_RANDOM, 0.05, 0.0, 512),     # union ~ all blocks: does not
        (512, 512, 64, m.PATTERN_BAND, 0.1, 4.0, 256),         # 64-row: as it is
        (960, 1024, 16, m.PATTERN_BLOCKDIAG, 0.0, 64.0, 200),   # stacks, ragged N
    ]
    probs, host = build_small(dev, "f16", specs=specs, seed=77)
    plan = m.BatchPlan(probs)
    assert plan.info()[1] == 3
    for _ in range(2):
        for (_, _, C) in probs:
            C.fill_(float("nan"))
        plan.run()
        m.device_error_check()
        check_fp64(probs, host, "f16")
    # new values in place (same structure): the next run multiplies them
    for k, ((A, B, C), (rp, ci, vals, Bf, bR)) in enumerate(zip(probs, host)):
        v2 = m.gen_values(len(ci), bR, 16, m.DIST_UNIFORM, seed=900 + k)
        A.vals.copy_(torch.from_numpy(v2).to(dev).half())
        host[k] = (rp, ci, v2, Bf, bR)
    plan.run()
    m.device_error_check()
    check_fp64(probs, host, "f16")
    plan.close()
