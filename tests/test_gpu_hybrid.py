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
