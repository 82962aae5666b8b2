"""Every supported entry of the tuner table (kernel configurations and
per-matrix plans) on seeded random products: block heights 16 / 32 / 64;
fp16, bf16, e4m3 with per-block scales and split fp16; random, band and
log-normal structures from 1 % to 60 % block density; M, K and N drawn at
random (N a multiple of 8, or 16 for e4m3). Each product is checked against
the FP64 oracle product of the values the library stores (so input rounding
is out of the comparison and only the fp32 accumulation remains, <= 2e-5
normwise), twice in a row per entry (work queues and plan counters reset)."""
import numpy as np
import pytest

import matrixmultiplicationcuda_gb300 as m
from matrixmultiplicationcuda_gb300 import DType, tuner
from oracle import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

BAR = 2e-5
PATTERNS = {m.PATTERN_RANDOM: 0.0, m.PATTERN_BAND: 4.0, m.PATTERN_LOGNORMAL: 1.5}


def _stored_f64(t, lo=None, scales=None, per=None):
    """The values a quantized array stores, in double (hi + lo, times its
    per-block scale for e4m3)."""
    if t.dtype == torch.uint8:
        t = t.view(torch.float8_e4m3fn)
    y = t.float().cpu().numpy().astype(np.float64)
    if lo is not None:
        y = y + lo.float().cpu().numpy().astype(np.float64)
    if scales is not None:
        y = (y.reshape(-1, per) * scales.cpu().numpy().astype(np.float64)[:, None]).reshape(-1)
    return y


@pytest.mark.parametrize("seed", [7, 11])
def test_every_table_entry_on_random_products(dev, seed):
    rng = np.random.default_rng(seed)
    table = tuner.configs()
    checked = 0
    for _ in range(40):
        bR = int(rng.choice([16, 32, 64]))
        dt = [DType.F16, DType.BF16, DType.E4M3, DType.F16_SPLIT][int(rng.integers(4))]
        M = int(rng.integers(1, 40)) * 64
        K = int(rng.integers(1, 40)) * 16 * (2 if dt == DType.E4M3 else 1)
        N = int(rng.integers(1, 80)) * (16 if dt == DType.E4M3 else 8)
        pat = int(rng.choice(list(PATTERNS)))
        dens = float(rng.choice([0.01, 0.05, 0.2, 0.6]))
        s = int(rng.integers(1 << 30))
        rp, ci = m.gen_structure(M, K, bR, pat, dens, PATTERNS[pat], seed=s)
        if len(ci) == 0:
            continue
        vals = m.gen_values(len(ci), bR, 16, m.DIST_SCALED_NORMAL if dt == DType.E4M3 else m.DIST_UNIFORM,
                            seed=s + 1)
        qv, qlo, qs = m.quantize(torch.from_numpy(vals).to(dev), dt, block_elems=bR * 16)
        A = m.BCSR(M, K, bR, 16, torch.from_numpy(rp).to(dev), torch.from_numpy(ci).to(dev), qv, dt, qlo, qs)
        Bq, Blo, Bs = m.quantize(torch.from_numpy(m.gen_dense(K, N, m.DIST_UNIFORM, seed=s + 2)).to(dev).reshape(-1),
                                 dt)
        Bq = Bq.view(K, N)
        Blo = Blo.view(K, N) if Blo is not None else None
        bs = float(Bs[0]) if Bs is not None else 1.0
        ref = oracle.bcsr_matmul_f64(rp, ci, _stored_f64(qv, qlo, qs if dt == DType.E4M3 else None, bR * 16), bR, 16,
                                     _stored_f64(Bq, Blo).reshape(K, N) * bs, threads=8)
        for ok, c in zip(tuner.supported_mask(bR, dt, N), table):
            if not ok:
                continue
            plan = m.BcsrPlan(A, N, c) if tuner.is_plan(c) else None
            for run in range(2):
                C = torch.full((M, N), float("nan"), device=dev)
                if plan is not None:
                    plan.run(A, Bq, C=C, B_lo=Blo, b_scale=bs)
                else:
                    m.spmm(A, Bq, N=N, C=C, cfg=c, B_lo=Blo, b_scale=bs)
                m.device_error_check()
                got = C.cpu().numpy()
                case = (bR, dt.name, M, K, N, pat, dens, tuner.config_name(c), run)
                assert np.isfinite(got).all(), case
                mx, fr = oracle.rel_errors(got, ref)
                assert mx <= BAR and fr <= BAR, (case, mx, fr)
                checked += 1
            if plan is not None:
                plan.close()
    assert checked > 500
