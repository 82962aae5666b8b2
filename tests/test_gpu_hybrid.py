"""The hybrid BCSR + CSR product (spmm_hcsr_mm): the CSR part is added by the
tcgen05 pipeline's epilogue in the same launch. Checked against an FP64
product of the whole matrix for thresholds that send everything to BCSR,
split the blocks, and send everything to CSR."""
import numpy as np
import pytest

import matrixmultiplicationcuda_gb300 as m
from oracle import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def mixed_matrix(M, K, seed):
    """fp16 bits of an M x K matrix whose 16x16 blocks have densities spread
    over [0, 1] (and a fifth of the blocks empty)."""
    rng = np.random.default_rng(seed)
    dens = rng.uniform(0, 1, (M // 16, K // 16)) * (rng.uniform(size=(M // 16, K // 16)) > 0.2)
    mask = rng.uniform(size=(M, K)) < np.repeat(np.repeat(dens, 16, 0), 16, 1)
    vals = rng.uniform(-1, 1, (M, K)).astype(np.float32) * mask
    return oracle.f32_to_f16(vals).view(np.uint16).reshape(M, K)


def run_hybrid(dev, A_bits, th, N, seed=1, cfg=None):
    M, K = A_bits.shape
    (bh, bi, bd), (ch, cx, cd) = m.host_dense_to_hcsr(A_bits, th)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    Ab = m.BCSR(M, K, 16, 16, t(bh), t(bi), t(bd.view(np.float16)))
    Bf = np.random.default_rng(seed).uniform(-1, 1, (K, N)).astype(np.float32)
    B = t(Bf).half()
    C = torch.full((M, N), float("nan"), dtype=torch.float32, device=dev)
    m.hcsr_mm(Ab, t(ch), t(cx), t(cd.view(np.float16)), B, N=N, C=C, cfg=cfg)
    m.device_error_check()
    Ad = oracle.f16_to_f32(A_bits).astype(np.float64)
    ref = Ad @ B.cpu().double().numpy()
    return C.cpu().numpy(), ref, len(bi), len(cx)


@pytest.mark.parametrize("th", [0.0, 0.3, 0.6, 0.9, 1.1])
@pytest.mark.parametrize("N", [64, 200, 512])
def test_hybrid_matches_fp64(dev, th, N):
    A = mixed_matrix(512, 768, seed=int(th * 10) + N)
    got, ref, nnzb, nnz = run_hybrid(dev, A, th, N)
    assert np.isfinite(got).all()
    mx, fr = oracle.rel_errors(got, ref)
    assert mx <= 2e-5 and fr <= 2e-5, (th, nnzb, nnz, mx, fr)
    if th == 0.0:
        assert nnz == 0
    if th > 1.0:
        assert nnzb == 0


@pytest.mark.parametrize("nt,queue", [(256, 0), (512, 1)])
def test_hybrid_configurations(dev, nt, queue):
    A = mixed_matrix(1024, 1024, seed=5)
    got, ref, nnzb, nnz = run_hybrid(dev, A, 0.5, 512, cfg=m.Config(kernel=2, n_tile=nt, schedule=queue))
    assert nnzb > 0 and nnz > 0
    mx, fr = oracle.rel_errors(got, ref)
    assert mx <= 2e-5 and fr <= 2e-5


def test_hybrid_rejects_unsupported(dev):
    A = mixed_matrix(128, 128, seed=3)
    with pytest.raises(m.SpmmError) as e:
        run_hybrid(dev, A, 0.5, 128, cfg=m.Config(kernel=2, split_k=2))
    assert e.value.status == m.Status.UNSUPPORTED
    with pytest.raises(m.SpmmError) as e:
        run_hybrid(dev, A, 0.5, 128, cfg=m.Config(kernel=1))
    assert e.value.status == m.Status.UNSUPPORTED


@pytest.mark.parametrize("N", [8, 64, 264, 1024])
def test_csr_comparator_matches_fp64(dev, N):
    """The native CSR product on the CSR part of a hybrid split (all entries
    when the threshold is above 1)."""
    A = mixed_matrix(384, 512, seed=N)
    (_, _, _), (ch, cx, cd) = m.host_dense_to_hcsr(A, 1.1)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    B = t(np.random.default_rng(N).uniform(-1, 1, (512, N)).astype(np.float32)).half()
    C = torch.full((384, N), float("nan"), dtype=torch.float32, device=dev)
    m.csr_mm(t(ch), t(cx), t(cd.view(np.float16)), 512, B, C=C)
    m.device_error_check()
    ref = oracle.f16_to_f32(A).astype(np.float64) @ B.cpu().double().numpy()
    mx, fr = oracle.rel_errors(C.cpu().numpy(), ref)
    assert mx <= 1e-5 and fr <= 1e-5


def test_csr_comparator_ragged_rows_and_checks(dev):
    """M not a multiple of the kernel's 8 rows per CTA, empty rows (every row
    of C is written, zeros there), a leading dimension above N, and the
    argument checks (N % 8, unaligned B)."""
    M, K, N = 101, 96, 40
    rng = np.random.default_rng(5)
    A = (rng.uniform(-1, 1, (M, K)) * (rng.uniform(size=(M, K)) < 0.1)).astype(np.float32)
    A[3] = 0
    A[50:60] = 0
    bits = oracle.f32_to_f16(A).view(np.uint16).reshape(M, K)
    ch, cx, cd = m.host_dense_to_csr(bits)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    B = t(rng.uniform(-1, 1, (K, N)).astype(np.float32)).half()
    Cbig = torch.full((M, 48), float("nan"), dtype=torch.float32, device=dev)
    m.csr_mm(t(ch), t(cx), t(cd.view(np.float16)), K, B, C=Cbig, ldc=48)
    m.device_error_check()
    got = Cbig[:, :N].cpu().numpy()
    ref = oracle.f16_to_f32(bits).astype(np.float64) @ B.cpu().double().numpy()
    assert (got[3] == 0).all() and (got[50:60] == 0).all()
    assert np.isnan(Cbig[:, N:].cpu().numpy()).all()     # columns past N untouched
    mx, fr = oracle.rel_errors(got, ref)
    assert mx <= 1e-5 and fr <= 1e-5
    with pytest.raises(m.SpmmError) as e:
        m.csr_mm(t(ch), t(cx), t(cd.view(np.float16)), K, B[:, :36], N=36)
    assert e.value.status == m.Status.UNSUPPORTED
    Bbuf = torch.zeros(K * N + 8, dtype=torch.float16, device=dev)
    Bmis = Bbuf[4:4 + K * N].view(K, N)                   # 8 bytes off a 16-byte boundary
    with pytest.raises(m.SpmmError) as e:
        m.csr_mm(t(ch), t(cx), t(cd.view(np.float16)), K, Bmis)
    assert e.value.status == m.Status.MISALIGNED


def run_plan(dev, A_bits, th, N, seed=1, cfg=None, Bf=None):
    """The planned hybrid product (gather blocks) on the same split."""
    M, K = A_bits.shape
    (bh, bi, bd), (ch, cx, cd) = m.host_dense_to_hcsr(A_bits, th)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    Ab = m.BCSR(M, K, 16, 16, t(bh), t(bi), t(bd.view(np.float16)))
    if Bf is None:
        Bf = np.random.default_rng(seed).uniform(-1, 1, (K, N)).astype(np.float32)
    B = t(Bf).half()
    plan = m.HcsrPlan(Ab, t(ch), t(cx), t(cd.view(np.float16)))
    C = torch.full((M, N), float("nan"), dtype=torch.float32, device=dev)
    plan.run(B, N=N, C=C, cfg=cfg)
    m.device_error_check()
    info = plan.info()
    plan.close()
    # the packed matrix: every stored block plus ceil(entries / 16) gather blocks per block row
    ent = np.diff(ch)[: M].reshape(M // 16, 16).sum(1)
    assert info == (len(bi) + int(((ent + 15) // 16).sum()), int(((ent + 15) // 16).sum()))
    Ad = oracle.f16_to_f32(A_bits).astype(np.float64)
    Bn = B.cpu().double().numpy()
    # the product over A's entries: a B row that only meets zero columns of A
    # takes no part (the FP64 product would form 0 * inf there)
    unused = ~Ad.any(axis=0)
    Bn[unused] = np.where(np.isfinite(Bn[unused]), Bn[unused], 0.0)
    ref = Ad @ Bn
    return C.cpu().numpy(), ref, len(bi), len(cx)


@pytest.mark.parametrize("th", [0.0, 0.3, 0.6, 1.1])
@pytest.mark.parametrize("N", [64, 200, 512])
def test_hybrid_plan_matches_fp64(dev, th, N):
    A = mixed_matrix(512, 768, seed=int(th * 10) + N + 7)
    got, ref, nnzb, nnz = run_plan(dev, A, th, N)
    assert np.isfinite(got).all()
    mx, fr = oracle.rel_errors(got, ref)
    assert mx <= 2e-5 and fr <= 2e-5, (th, nnzb, nnz, mx, fr)


@pytest.mark.parametrize("cfg", [dict(n_tile=256, schedule=1), dict(n_tile=512), dict(n_tile=256, split_k=2)])
def test_hybrid_plan_configurations(dev, cfg):
    A = mixed_matrix(1024, 1024, seed=11)
    got, ref, nnzb, nnz = run_plan(dev, A, 0.5, 512, cfg=m.Config(kernel=2, **cfg))
    assert nnzb > 0 and nnz > 0
    mx, fr = oracle.rel_errors(got, ref)
    assert mx <= 2e-5 and fr <= 2e-5


def test_hybrid_plan_long_rows_and_empty_parts(dev):
    """Rows of 1000+ CSR entries (many gather blocks per block row), and the
    all-zero matrix (no blocks of either kind)."""
    M, K, N = 64, 4096, 256
    rng = np.random.default_rng(3)
    A = np.zeros((M, K), np.float32)
    A[::16] = rng.uniform(-1, 1, (M // 16, K))          # one full row per block row: density 1/16
    A[5, ::3] = rng.uniform(-1, 1, len(range(0, K, 3)))
    bits = oracle.f32_to_f16(A).view(np.uint16).reshape(M, K)
    got, ref, nnzb, nnz = run_plan(dev, bits, 0.5, N)
    assert nnzb == 0 and nnz > 4000
    mx, fr = oracle.rel_errors(got, ref)
    assert mx <= 2e-5 and fr <= 2e-5
    zero = np.zeros((M, K), np.uint16)
    got, ref, nnzb, nnz = run_plan(dev, zero, 0.5, N)
    assert nnzb == 0 and nnz == 0 and (got == 0).all()


def test_hybrid_plan_padding_reads_zeros(dev):
    """Unused slots of a gather block index row K (past B) and must add exact
    zeros: B's row 0 is +inf and no entry or stored block of A touches column
    0, so a slot that read a real row of B would turn C into NaN."""
    M, K, N = 256, 512, 128
    A = mixed_matrix(M, K, seed=21).copy()
    A[:, 0] = 0
    A[:, :16] &= np.where(np.random.default_rng(2).uniform(size=(M, 16)) < 0.1, 0xFFFF, 0).astype(np.uint16)
    Bf = np.random.default_rng(4).uniform(-1, 1, (K, N)).astype(np.float32)
    Bf[0] = np.inf
    got, ref, nnzb, nnz = run_plan(dev, A, 0.5, N, Bf=Bf)
    assert nnz > 0 and np.isfinite(got).all()
    mx, fr = oracle.rel_errors(got, ref)
    assert mx <= 2e-5 and fr <= 2e-5


def test_hybrid_plan_rejects_unsupported(dev):
    A = mixed_matrix(128, 128, seed=3)
    with pytest.raises(m.SpmmError) as e:
        run_plan(dev, A, 0.5, 128, cfg=m.Config(kernel=1))
    assert e.value.status == m.Status.UNSUPPORTED
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    rp, ci = m.gen_structure(128, 128, 32, m.PATTERN_RANDOM, 0.2, 0, seed=1)
    vals = m.gen_values(len(ci), 32, 16, m.DIST_UNIFORM, seed=2)
    A32 = m.BCSR.from_host(128, 128, 32, rp, ci, vals, m.DType.F16, device=dev)
    z = torch.zeros(129, dtype=torch.int32, device=dev)
    with pytest.raises(m.SpmmError) as e:
        m.HcsrPlan(A32, z, z[:0], z[:0].half())
    assert e.value.status == m.Status.UNSUPPORTED
