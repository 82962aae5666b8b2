"""The native dense comparator (spmm_dense_mm, tcgen05): fp16 and bf16 products
against an FP64 product of the same stored values, at tile-aligned and ragged
shapes (M, N, K off the 128 x 256 x 64 tile), a leading dimension above N, and
the argument checks."""
import numpy as np
import pytest

import matrixmultiplicationcuda_gb300 as m
from oracle import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def check(dev, M, K, N, dtype=torch.float16, seed=0, ldc=None):
    g = torch.Generator().manual_seed(seed)
    A = (torch.rand((M, K), generator=g) * 2 - 1).to(dtype).to(dev)
    B = (torch.rand((K, N), generator=g) * 2 - 1).to(dtype).to(dev)
    ldc = N if ldc is None else ldc
    Cbuf = torch.full((M, ldc), float("nan"), dtype=torch.float32, device=dev)
    C = Cbuf[:, :N]
    m.dense_mm(A, B, C=C)
    m.device_error_check()
    ref = A.cpu().double().numpy() @ B.cpu().double().numpy()
    got = C.cpu().numpy()
    assert np.isfinite(got).all()
    if ldc > N:
        assert np.isnan(Cbuf[:, N:].cpu().numpy()).all()   # columns past N untouched
    mx, fr = oracle.rel_errors(got, ref)
    assert mx <= 2e-5 and fr <= 2e-5, (M, K, N, mx, fr)


@pytest.mark.parametrize("M,K,N", [(128, 64, 256), (256, 512, 512), (1024, 1024, 1024), (384, 2048, 768)])
def test_dense_tile_aligned(dev, M, K, N):
    check(dev, M, K, N)


@pytest.mark.parametrize("M,K,N", [(1, 16, 8), (100, 40, 200), (300, 200, 264), (129, 72, 520), (640, 1000, 24)])
def test_dense_ragged(dev, M, K, N):
    check(dev, M, K, N, seed=M + K + N)


def test_dense_bf16_and_ldc(dev):
    check(dev, 512, 768, 512, dtype=torch.bfloat16, seed=3)
    check(dev, 200, 128, 264, seed=4, ldc=272)


def test_dense_many_tiles_per_cta(dev):
    """More tiles than SMs: each CTA runs several tiles through both accumulators."""
    check(dev, 4096, 256, 2048, seed=5)


def test_dense_rejects(dev):
    A = torch.zeros((64, 64), dtype=torch.float16, device=dev)
    B = torch.zeros((64, 36), dtype=torch.float16, device=dev)
    with pytest.raises(m.SpmmError) as e:
        m.dense_mm(A, B)
    assert e.value.status == m.Status.UNSUPPORTED
    with pytest.raises(m.SpmmError) as e:
        m.dense_mm(A, B.float())
    assert e.value.status == m.Status.UNSUPPORTED
    Abuf = torch.zeros(64 * 64 + 8, dtype=torch.float16, device=dev)
    with pytest.raises(m.SpmmError) as e:
        m.dense_mm(Abuf[4:4 + 64 * 64].view(64, 64), torch.zeros((64, 64), dtype=torch.float16, device=dev))
    assert e.value.status == m.Status.MISALIGNED
