"""The per-matrix plan (spmm_bcsr_plan_*): heaviest-first items, with rows far
longer than the average load per CTA split into parts that add into a C tile
their part 0 zeroed. Checked exactly at the headline size with integer inputs
(row / column checksums, three runs in a row so the counters reset), against
the unplanned product and FP64 with random values, with and without split
rows, at ragged N, for every block height, and the argument checks."""
import numpy as np
import pytest

import matrixmultiplicationcuda_gb300 as m
from oracle import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("pattern,param,cfg", [
    (m.PATTERN_RANDOM, 0.0, m.Config(kernel=2, n_tile=512, acc_buffers=1)),      # rows of similar length: no split
    (m.PATTERN_LOGNORMAL, 1.5, m.Config(kernel=2, n_tile=512, acc_buffers=1)),   # rows up to ~13x the mean: split
    (m.PATTERN_LOGNORMAL, 1.5, m.Config(kernel=2, n_tile=256, acc_buffers=2)),
])
def test_plan_headline_size_exact_checksums(dev, pattern, param, cfg):
    M = K = 16384
    N, bR = 512, 64
    rp, ci = m.gen_structure(M, K, bR, pattern, 0.02, param, seed=20240)
    rng = np.random.default_rng(1)
    vals = rng.integers(-2, 3, len(ci) * bR * 16).astype(np.float32)
    B = rng.integers(-2, 3, (K, N)).astype(np.int64)
    A = m.BCSR.from_host(M, K, bR, rp, ci, vals, m.DType.BF16, device=dev)
    Bd = torch.from_numpy(B.astype(np.float32)).to(dev).bfloat16()
    plan = m.BcsrPlan(A, N, cfg)
    items, groups, pcfg = plan.info()
    ntiles = -(-N // pcfg.n_tile)
    if pattern == m.PATTERN_RANDOM:
        assert groups == 0 and items == (M // bR) * ntiles
    else:
        assert groups > 0 and items > (M // bR) * ntiles
    blocks = vals.reshape(-1, bR, 16).astype(np.int64)
    bsum = B.sum(axis=1).reshape(K // 16, 16)
    rows = np.zeros((M // bR, bR), np.int64)
    np.add.at(rows, np.repeat(np.arange(M // bR), np.diff(rp)), np.einsum("brc,bc->br", blocks, bsum[ci]))
    colA = np.zeros((K // 16, 16), np.int64)
    np.add.at(colA, ci, blocks.sum(axis=1))
    cols = colA.reshape(-1) @ B
    first = None
    for run in range(3):   # the split rows' counters reset between launches
        C = torch.full((M, N), float("nan"), dtype=torch.float32, device=dev)
        plan.run(A, Bd, C=C)
        m.device_error_check()
        Ch = C.cpu().double().numpy()
        assert np.array_equal(Ch.sum(axis=1), rows.reshape(-1).astype(np.float64)), run
        assert np.array_equal(Ch.sum(axis=0), cols.astype(np.float64)), run
        if first is None:
            first = Ch
        assert np.array_equal(Ch, first)
    plan.close()


@pytest.mark.parametrize("bR,M,K,N,cfg", [
    (64, 4096, 8192, 264, m.Config(kernel=2, n_tile=256)),          # 2 column tiles, ragged N, spare slots
    (64, 16384, 4096, 512, m.Config(kernel=2, n_tile=512, acc_buffers=2)),   # one CTA per SM: no spare slots
    (64, 16384, 4096, 512, m.Config(kernel=2, n_tile=256, acc_buffers=2)),   # 512 items: no spare slots
    (32, 2048, 4096, 256, None),
    (16, 1024, 4096, 256, None),
])
def test_plan_matches_unplanned_and_fp64(dev, bR, M, K, N, cfg):
    rp, ci = m.gen_structure(M, K, bR, m.PATTERN_LOGNORMAL, 0.05, 1.5, seed=M + bR)
    vals = m.gen_values(len(ci), bR, 16, m.DIST_UNIFORM, seed=3)
    A = m.BCSR.from_host(M, K, bR, rp, ci, vals, m.DType.F16, device=dev)
    Bd = torch.from_numpy(m.gen_dense(K, N, m.DIST_UNIFORM, seed=4)).to(dev).half()
    plan = m.BcsrPlan(A, N, cfg)
    items, split_rows, pcfg = plan.info()
    C1 = torch.full((M, N), float("nan"), dtype=torch.float32, device=dev)
    for _ in range(2):
        plan.run(A, Bd, C=C1)
    C0 = m.spmm(A, Bd, N=N, cfg=pcfg)
    m.device_error_check()
    plan.close()
    got, base = C1.cpu().numpy(), C0.cpu().numpy()
    assert np.isfinite(got).all()
    mx, fr = oracle.rel_errors(got, base.astype(np.float64))
    assert mx <= 1e-5 and fr <= 1e-5, (split_rows, mx, fr)
    vh = vals.astype(np.float16).astype(np.float64)
    ref = oracle.bcsr_matmul_f64(rp, ci, vh, bR, 16, Bd.cpu().double().numpy())
    mx, fr = oracle.rel_errors(got, ref)
    assert mx <= 2e-5 and fr <= 2e-5


def test_plan_rejects(dev):
    M = K = 1024
    rp, ci = m.gen_structure(M, K, 64, m.PATTERN_RANDOM, 0.1, 0, seed=1)
    vals = m.gen_values(len(ci), 64, 16, m.DIST_UNIFORM, seed=2)
    A = m.BCSR.from_host(M, K, 64, rp, ci, vals, m.DType.F16, device=dev)
    for cfg in (m.Config(kernel=1), m.Config(kernel=2, split_k=2), m.Config(kernel=2, schedule=3)):
        with pytest.raises(m.SpmmError) as e:
            m.BcsrPlan(A, 256, cfg)
        assert e.value.status == m.Status.UNSUPPORTED
    # schedule 2 (the tuner table's mark for a plan entry) builds the plan too
    p2 = m.BcsrPlan(A, 256, m.Config(kernel=2, schedule=2))
    assert p2.info()[2].schedule == 1
    p2.close()
    plan = m.BcsrPlan(A, 256)
    assert plan.info()[2].schedule == 1                    # the plan's own work queue
    m.BcsrPlan(A, 256, plan.info()[2]).close()             # what it reports builds another plan
    rp2, ci2 = m.gen_structure(2 * M, K, 64, m.PATTERN_RANDOM, 0.1, 0, seed=1)
    A2 = m.BCSR.from_host(2 * M, K, 64, rp2, ci2, m.gen_values(len(ci2), 64, 16, m.DIST_UNIFORM, seed=2),
                          m.DType.F16, device=dev)
    B = torch.zeros((K, 256), dtype=torch.float16, device=dev)
    with pytest.raises(m.SpmmError) as e:
        plan.run(A2, B, C=torch.empty((2 * M, 256), dtype=torch.float32, device=dev))   # not the plan's M
    assert e.value.status == m.Status.INVALID_ARG
    plan.close()


def test_plan_in_cuda_graph(dev):
    """plan.run is one launch with no allocation or synchronisation, so it
    captures into a CUDA graph; replays (split rows included) match eager runs
    and leave the counters reset."""
    M = K = 8192
    N, bR = 512, 64
    rp, ci = m.gen_structure(M, K, bR, m.PATTERN_LOGNORMAL, 0.05, 1.5, seed=77)
    rng = np.random.default_rng(3)
    vals = rng.integers(-2, 3, len(ci) * bR * 16).astype(np.float32)
    A = m.BCSR.from_host(M, K, bR, rp, ci, vals, m.DType.F16, device=dev)
    B = torch.from_numpy(rng.integers(-2, 3, (K, N)).astype(np.float32)).to(dev).half()
    plan = m.BcsrPlan(A, N, m.Config(kernel=2, n_tile=256, acc_buffers=2))
    assert plan.info()[1] > 0
    eager = plan.run(A, B).clone()
    C = torch.empty((M, N), dtype=torch.float32, device=dev)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        plan.run(A, B, C=C, stream=s)      # warm-up on the capture stream
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        plan.run(A, B, C=C, stream=torch.cuda.current_stream())
    for _ in range(3):
        C.fill_(float("nan"))
        g.replay()
        torch.cuda.synchronize()
        m.device_error_check()
        assert torch.equal(C, eager)       # integer inputs: exact whatever the order of the adds
    plan.close()


def test_plan_unequal_parts_more_items_than_ctas(dev):
    """A few rows of 301 blocks among rows of 5, four column tiles: more items
    than CTAs, and each long row cut into parts of unequal length (23 and 24
    blocks). Part 0 of a row must come before its siblings in the item list,
    or a CTA could wait for a zeroing it does itself later. Exact checksums,
    three launches, no wait gives up."""
    M = K = 8192
    N, bR = 1024, 64
    MB, KB = M // bR, K // 16
    lens = np.full(MB, 5)
    lens[[0, 40, 77, 127]] = 301
    rp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    rng = np.random.default_rng(8)
    ci = np.concatenate([np.sort(rng.choice(KB, n, replace=False)) for n in lens]).astype(np.int32)
    vals = rng.integers(-2, 3, len(ci) * bR * 16).astype(np.float32)
    B = rng.integers(-2, 3, (K, N)).astype(np.int64)
    A = m.BCSR.from_host(M, K, bR, rp, ci, vals, m.DType.F16, device=dev)
    Bd = torch.from_numpy(B.astype(np.float32)).to(dev).half()
    plan = m.BcsrPlan(A, N, m.Config(kernel=2, n_tile=256, acc_buffers=2))
    items, groups, _ = plan.info()
    assert groups == 4 * 4 and items > 304
    blocks = vals.reshape(-1, bR, 16).astype(np.int64)
    bsum = B.sum(axis=1).reshape(K // 16, 16)
    rows = np.zeros((MB, bR), np.int64)
    np.add.at(rows, np.repeat(np.arange(MB), lens), np.einsum("brc,bc->br", blocks, bsum[ci]))
    colA = np.zeros((K // 16, 16), np.int64)
    np.add.at(colA, ci, blocks.sum(axis=1))
    cols = colA.reshape(-1) @ B
    for run in range(3):
        C = torch.full((M, N), float("nan"), dtype=torch.float32, device=dev)
        plan.run(A, Bd, C=C)
        m.device_error_check()
        Ch = C.cpu().double().numpy()
        assert np.array_equal(Ch.sum(axis=1), rows.reshape(-1).astype(np.float64)), run
        assert np.array_equal(Ch.sum(axis=0), cols.astype(np.float64)), run
    plan.close()


def _int_problem(M, K, N, bR, pattern, density, seed, dev, dtype=m.DType.BF16):
    rp, ci = m.gen_structure(M, K, bR, pattern, density, 1.5, seed=seed)
    rng = np.random.default_rng(seed)
    vals = rng.integers(-2, 3, len(ci) * bR * 16).astype(np.float32)
    B = rng.integers(-2, 3, (K, N)).astype(np.float32)
    A = m.BCSR.from_host(M, K, bR, rp, ci, vals, dtype, device=dev)
    tdt = torch.bfloat16 if dtype == m.DType.BF16 else torch.float16
    return A, torch.from_numpy(B).to(dev).to(tdt)


@pytest.mark.parametrize("pattern,density", [(m.PATTERN_RANDOM, 0.02), (m.PATTERN_LOGNORMAL, 0.05)])
def test_plan_inputs_ready_back_to_back(dev, pattern, density):
    """SPMM_RUN_INPUTS_READY over a stream of independent products (four
    problems with the same structure, different values, round-robin): each
    launch overlaps the tail of the one before it, claims its queued items and
    writes C only after that launch has finished. Integer inputs make every
    product exact, so each C must equal the same product run without the flag,
    split rows included, over many launches of one plan."""
    M = K = 16384 if pattern == m.PATTERN_RANDOM else 8192
    N = 512
    probs = []
    for s in range(4):
        A, B = _int_problem(M, K, N, 64, pattern, density, 31, dev)
        if s:   # same structure, different values: scale B
            B = (B * (s + 1)).contiguous()
        probs.append((A, B))
    plan = m.BcsrPlan(probs[0][0], N)
    assert (plan.info()[1] > 0) == (pattern == m.PATTERN_LOGNORMAL)
    refs = []
    for A, B in probs:
        refs.append(plan.run(A, B).clone())
    Cs = [torch.full((M, N), float("nan"), dtype=torch.float32, device=dev) for _ in probs]
    torch.cuda.synchronize()   # the flag's promise: no kernel since then writes A or B
    for i in range(40):
        A, B = probs[i % 4]
        plan.run(A, B, C=Cs[i % 4], inputs_ready=True)
    torch.cuda.synchronize()
    m.device_error_check()
    for C, ref in zip(Cs, refs):
        assert torch.equal(C, ref)
    plan.close()


@pytest.mark.parametrize("seed", [1, 2, 3, 4])
def test_plan_inputs_ready_random_chains(dev, seed):
    """Seeded random products on a random plan entry of the tuner table (every
    block height, random shape and N, random or log-normal rows, fp16 or bf16):
    three problems of one structure with different B, twelve launches chained
    with SPMM_RUN_INPUTS_READY round-robin, each C equal to the same product run
    without the flag (integer inputs: every product exact)."""
    from matrixmultiplicationcuda_gb300 import tuner
    rng = np.random.default_rng(seed)
    for _ in range(3):
        bR = int(rng.choice([16, 32, 64]))
        M = int(rng.integers(2, 40)) * 64
        K = int(rng.integers(2, 40)) * 64
        N = int(rng.integers(1, 96)) * 8
        pattern = [m.PATTERN_RANDOM, m.PATTERN_LOGNORMAL][int(rng.integers(2))]
        dtype = [m.DType.F16, m.DType.BF16][int(rng.integers(2))]
        density = float(rng.choice([0.02, 0.08, 0.3]))
        A, B0 = _int_problem(M, K, N, bR, pattern, density, int(rng.integers(1 << 20)), dev, dtype)
        mask = tuner.supported_mask(bR, dtype, N)
        cand = [c for ok, c in zip(mask, tuner.configs()) if ok and tuner.is_plan(c)]
        if not cand:
            continue
        cfg = cand[int(rng.integers(len(cand)))]
        plan = m.BcsrPlan(A, N, cfg)
        Bs = [B0] + [(B0 * (s + 2)).contiguous() for s in range(2)]
        refs = [plan.run(A, B).clone() for B in Bs]
        Cs = [torch.full((M, N), float("nan"), dtype=torch.float32, device=dev) for _ in Bs]
        torch.cuda.synchronize()
        for i in range(12):
            plan.run(A, Bs[i % 3], C=Cs[i % 3], inputs_ready=True)
        torch.cuda.synchronize()
        m.device_error_check()
        for C, ref in zip(Cs, refs):
            assert torch.equal(C, ref), (bR, M, K, N, pattern, dtype.name, density, tuner.config_name(cfg))
        plan.close()


def test_plan_inputs_ready_keeps_c_order(dev):
    """Two launches write the same C: the second (with the flag) starts its
    copies and MMAs while the first runs, but stores C only after the first has
    finished, so C holds the second product."""
    M = K = 16384
    N = 512
    A1, B1 = _int_problem(M, K, N, 64, m.PATTERN_RANDOM, 0.02, 5, dev)
    B2 = (B1 * -3).contiguous()
    plan = m.BcsrPlan(A1, N)
    ref2 = plan.run(A1, B2).clone()
    C = torch.empty((M, N), dtype=torch.float32, device=dev)
    torch.cuda.synchronize()   # the flag's promise: no kernel since then writes A or B
    for _ in range(5):
        plan.run(A1, B1, C=C)
        plan.run(A1, B2, C=C, inputs_ready=True)
        torch.cuda.synchronize()
        m.device_error_check()
        assert torch.equal(C, ref2)
    plan.close()


def test_plan_run_rejects_unknown_flags(dev):
    import ctypes
    from matrixmultiplicationcuda_gb300._lib import lib, stream_handle
    from matrixmultiplicationcuda_gb300.bcsr import _dense_desc
    A, B = _int_problem(1024, 1024, 256, 64, m.PATTERN_RANDOM, 0.1, 2, dev)
    plan = m.BcsrPlan(A, 256)
    C = torch.empty((1024, 256), dtype=torch.float32, device=dev)
    a, b = A.desc(), _dense_desc(B, ldb=B.stride(0))
    st = lib().spmm_bcsr_plan_run_ex(plan._h, ctypes.byref(a), ctypes.byref(b), 256, ctypes.c_void_p(C.data_ptr()),
                                     256, 2, stream_handle(None))
    assert st == int(m.Status.INVALID_ARG)
    plan.close()


def test_plan_inputs_ready_in_cuda_graph(dev):
    """A chain of flagged plan runs over four independent products, captured in
    one CUDA graph (consecutive launches keep their programmatic dependency)
    and replayed: every C matches the eager product bit for bit."""
    M = K = 8192
    N = 512
    probs = []
    for s in range(4):
        A, B = _int_problem(M, K, N, 64, m.PATTERN_LOGNORMAL, 0.05, 40 + s, dev)
        probs.append((A, B))
    plans = [m.BcsrPlan(A, N, m.Config(kernel=2, n_tile=512, acc_buffers=1)) for A, _ in probs]
    refs = [p.run(A, B).clone() for p, (A, B) in zip(plans, probs)]
    Cs = [torch.empty((M, N), dtype=torch.float32, device=dev) for _ in probs]
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        for p, (A, B), C in zip(plans, probs, Cs):
            p.run(A, B, C=C, stream=s, inputs_ready=True)   # warm-up on the capture stream
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        st = torch.cuda.current_stream()
        for p, (A, B), C in zip(plans, probs, Cs):
            p.run(A, B, C=C, stream=st, inputs_ready=True)
    for _ in range(3):
        for C in Cs:
            C.fill_(float("nan"))
        torch.cuda.synchronize()
        g.replay()
        torch.cuda.synchronize()
        m.device_error_check()
        for C, ref in zip(Cs, refs):
            assert torch.equal(C, ref)
    for p in plans:
        p.close()


def _int_bcsr(M, K, bR, pattern, density, param, seed, dev, dtype=m.DType.F16):
    rp, ci = m.gen_structure(M, K, bR, pattern, density, param, seed=seed)
    rng = np.random.default_rng(seed)
    vals = rng.integers(-2, 3, len(ci) * bR * 16).astype(np.float32)
    return rp, ci, vals, m.BCSR.from_host(M, K, bR, rp, ci, vals, dtype, device=dev)


@pytest.mark.parametrize("bR", [16, 32])
@pytest.mark.parametrize("pattern,param", [(m.PATTERN_BAND, 8), (m.PATTERN_BLOCKDIAG, 256)])
@pytest.mark.parametrize("N,cfg", [(1024, None), (520, m.Config(kernel=2, n_tile=512, acc_buffers=1))])
def test_plan_stacks_short_blocks(dev, bR, pattern, param, N, cfg):
    """16- and 32-row blocks whose block rows share their columns (band,
    block-diagonal) run stacked as 64-row blocks: the same product as the
    unplanned one, exactly (integer inputs), and new values on the same
    structure are picked up by the next run."""
    M = K = 4096
    rp, ci, vals, A = _int_bcsr(M, K, bR, pattern, 0.2, param, 11, dev)
    B = torch.from_numpy(np.random.default_rng(12).integers(-2, 3, (K, N)).astype(np.float32)).to(dev).half()
    plan = m.BcsrPlan(A, N, cfg)
    st, nb = plan.stacking()
    assert st == 64 // bR and 0 < nb * 100 <= len(ci) * 60
    ref = m.spmm(A, B, N=N)
    C = torch.full((M, N), float("nan"), dtype=torch.float32, device=dev)
    plan.run(A, B, C=C)
    m.device_error_check()
    assert torch.equal(C, ref)
    A2 = m.BCSR.from_host(M, K, bR, rp, ci, -2 * vals, m.DType.F16, device=dev)   # same structure
    torch.cuda.synchronize()
    plan.run(A2, B, C=C, inputs_ready=True)   # the early start reads the new values too
    m.device_error_check()
    assert torch.equal(C, -2 * ref)
    plan.close()


@pytest.mark.parametrize("M,pattern,density,N", [(4096, m.PATTERN_RANDOM, 0.05, 1024),     # columns rarely shared
                                                 (4096 + 16, m.PATTERN_BAND, 0.2, 1024),  # M not a multiple of 64
                                                 (4096, m.PATTERN_BAND, 0.2, 256)])       # N too small to pay
def test_plan_does_not_stack(dev, M, pattern, density, N):
    K = 4096
    rp, ci, vals, A = _int_bcsr(M, K, 16, pattern, density, 8, 13, dev)
    B = torch.from_numpy(np.random.default_rng(14).integers(-2, 3, (K, N)).astype(np.float32)).to(dev).half()
    plan = m.BcsrPlan(A, N)
    assert plan.stacking() == (1, 0)
    assert torch.equal(plan.run(A, B), m.spmm(A, B, N=N))
    m.device_error_check()
    plan.close()


def test_plan_stacked_bf16_in_cuda_graph(dev):
    """A stacked run (one launch that assembles the 64-row blocks from A's own
    values) captured in a graph and replayed matches the eager product."""
    M = K = 8192
    N = 1024
    rp, ci, vals, A = _int_bcsr(M, K, 16, m.PATTERN_BAND, 0.2, 8, 15, dev, m.DType.BF16)
    B = torch.from_numpy(np.random.default_rng(16).integers(-2, 3, (K, N)).astype(np.float32)).to(dev).bfloat16()
    plan = m.BcsrPlan(A, N)
    assert plan.stacking()[0] == 4
    eager = m.spmm(A, B, N=N)
    C = torch.empty((M, N), dtype=torch.float32, device=dev)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        plan.run(A, B, C=C, stream=s)
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        plan.run(A, B, C=C, stream=torch.cuda.current_stream())
    for _ in range(3):
        C.fill_(float("nan"))
        g.replay()
        torch.cuda.synchronize()
        m.device_error_check()
        assert torch.equal(C, eager)
    plan.close()


@pytest.mark.parametrize("bR,dtype,N", [(16, m.DType.F16, 1024), (32, m.DType.BF16, 1000), (16, m.DType.BF16, 776)])
def test_plan_stacked_every_entry_inputs_ready_chain(dev, bR, dtype, N):
    """Every plan entry of the tuner table that stacks this product (band
    rows sharing their columns): the stacked run equals the unplanned product
    exactly, and so do twelve launches chained with SPMM_RUN_INPUTS_READY
    round-robin over three B (integer inputs). N = 1000 and 776 take the
    2-D panel path."""
    from matrixmultiplicationcuda_gb300 import tuner
    M, K = 2048, 3072
    rp, ci, vals, A = _int_bcsr(M, K, bR, m.PATTERN_BAND, 0.2, 8, 21 + bR, dev, dtype)
    tdt = torch.float16 if dtype == m.DType.F16 else torch.bfloat16
    B0 = torch.from_numpy(np.random.default_rng(22).integers(-2, 3, (K, N)).astype(np.float32)).to(dev).to(tdt)
    Bs = [B0] + [(B0 * (s + 2)).contiguous() for s in range(2)]
    refs = [m.spmm(A, B, N=N) for B in Bs]
    stacked = 0
    for cfg in [c for c in tuner.configs() if tuner.is_plan(c)]:
        try:
            plan = m.BcsrPlan(A, N, cfg)
        except m.SpmmError:
            continue   # no 64-row kernel for this entry's tile at this N, and none at bR either
        if plan.stacking()[0] == 1:
            plan.close()
            continue
        stacked += 1
        C0 = torch.full((M, N), float("nan"), dtype=torch.float32, device=dev)
        plan.run(A, Bs[0], C=C0)
        m.device_error_check()
        assert torch.equal(C0, refs[0]), tuner.config_name(cfg)
        Cs = [torch.full((M, N), float("nan"), dtype=torch.float32, device=dev) for _ in Bs]
        torch.cuda.synchronize()
        for i in range(12):
            plan.run(A, Bs[i % 3], C=Cs[i % 3], inputs_ready=True)
        torch.cuda.synchronize()
        m.device_error_check()
        for C, ref in zip(Cs, refs):
            assert torch.equal(C, ref), tuner.config_name(cfg)
        plan.close()
    assert stacked >= 3
