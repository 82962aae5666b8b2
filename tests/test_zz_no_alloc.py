"""The allocation-free entry point, spmm_bcsr_mm_noalloc.

It exists for callers that cannot call cudaMalloc: an application or
allocator that owns every device allocation, a memory budget that forbids the
CUDA allocator, or code that must not allocate while a stream is captured. Its
scratch (the error word and the work-queue counters) lives in a fixed array
compiled into the library, so these tests check, through the C ABI, that on
two calls in a row it returns what spmm_bcsr_mm returns on the same tcgen05
pipeline and what the FP64 oracle product gives, that it rejects what it
cannot hold, and that it leaves the device's free memory unchanged.
Tolerances: normwise relative difference <= 1e-6 against spmm_bcsr_mm run on
the same pipeline (kernel 2; only the item-to-CTA assignment differs, fp32
accumulation in the same block order), and the documented per-type bars
against the FP64 product of the stored values (fp16 2e-3, bf16 1e-2, split
fp16 2e-6).

This file is collected last on purpose, so that a run stopping at the first
failure has already run every other test.
"""
import ctypes
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest
import torch

import matrixmultiplicationcuda_gb300 as m
from matrixmultiplicationcuda_gb300._lib import BcsrDesc, Config, DenseDesc, Status, stream_handle
from oracle import oracle

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _descs(A, Bq, Blo=None):
    a = A.desc()
    b = DenseDesc()
    b.data = Bq.data_ptr()
    b.data_lo = Blo.data_ptr() if Blo is not None else None
    b.scale = 1.0
    b.ldb = Bq.shape[1]
    return a, b


def _call(fn, A, Bq, C, Blo=None, cfg=None):
    a, b = _descs(A, Bq, Blo)
    st = fn(ctypes.byref(a), ctypes.byref(b), Bq.shape[1], ctypes.c_void_p(C.data_ptr()), C.shape[1],
            ctypes.byref(cfg if cfg is not None else Config()), stream_handle())
    return Status(st)


BAR = {m.DType.F16: 2e-3, m.DType.BF16: 1e-2, m.DType.F16_SPLIT: 2e-6}


def _stored_f64(t, lo=None):
    """The values a quantized array stores, in double (hi + lo for split)."""
    x = t.float().cpu().numpy().astype(np.float64)
    return x + lo.float().cpu().numpy().astype(np.float64) if lo is not None else x


@pytest.mark.parametrize("bR,dtype", [(64, m.DType.F16), (32, m.DType.BF16), (64, m.DType.F16_SPLIT)])
def test_matches_regular_entry_point_on_two_calls(dev, bR, dtype):
    M, K, N = 1024, 2048, 512
    rp, ci = m.gen_structure(M, K, bR, m.PATTERN_LOGNORMAL, 0.05, 1.5, seed=21)
    vals = m.gen_values(len(ci), bR, 16, m.DIST_UNIFORM, seed=22)
    A = m.BCSR.from_host(M, K, bR, rp, ci, vals, dtype, device=dev)
    Bq, Blo, _ = m.quantize(torch.from_numpy(m.gen_dense(K, N, m.DIST_UNIFORM, seed=23)).to(dev).reshape(-1), dtype)
    Bq = Bq.view(K, N)
    Blo = Blo.view(K, N) if Blo is not None else None
    L = m.lib()
    ref = torch.full((M, N), float("nan"), device=dev)
    same_pipeline = Config()
    same_pipeline.kernel = 2       # the tcgen05 pipeline the allocation-free entry runs
    assert _call(L.spmm_bcsr_mm, A, Bq, ref, Blo, same_pipeline) == Status.OK
    m.device_error_check()
    ref_np = ref.cpu().numpy()
    f64 = oracle.bcsr_matmul_f64(rp, ci, _stored_f64(A.vals, A.vals_lo), bR, 16,
                                 _stored_f64(Bq, Blo), threads=8)
    for _ in range(2):
        out = torch.full((M, N), float("nan"), device=dev)
        assert _call(L.spmm_bcsr_mm_noalloc, A, Bq, out, Blo) == Status.OK
        assert Status(L.spmm_noalloc_error_check(stream_handle())) == Status.OK
        got = out.cpu().numpy()
        assert np.isfinite(got).all()
        mx, fr = oracle.rel_errors(got, ref_np.astype(np.float64))
        assert mx <= 1e-6 and fr <= 1e-6, (mx, fr)
        mx, fr = oracle.rel_errors(got, f64)
        assert mx <= BAR[dtype] and fr <= BAR[dtype], (mx, fr)


def test_k_zero_clears_the_window(dev):
    """K == 0 (no block columns) zeroes the C window and leaves the padding."""
    M, N = 128, 64
    rp = torch.zeros(M // 64 + 1, dtype=torch.int32, device=dev)
    A = m.BCSR(M, 0, 64, 16, rp, torch.zeros(0, dtype=torch.int32, device=dev),
               torch.zeros(0, dtype=torch.float16, device=dev))
    Bq = torch.zeros((1, N), dtype=torch.float16, device=dev)
    C = torch.full((M, N + 16), 5.0, device=dev)
    a, b = _descs(A, Bq)
    st = m.lib().spmm_bcsr_mm_noalloc(ctypes.byref(a), ctypes.byref(b), N, ctypes.c_void_p(C.data_ptr()), N + 16,
                                      None, stream_handle())
    assert Status(st) == Status.OK, m._lib.last_error()
    torch.cuda.synchronize()
    assert torch.all(C[:, :N] == 0) and torch.all(C[:, N:] == 5.0)


def test_rejects_what_it_cannot_hold():
    L = m.lib()
    a = BcsrDesc()
    a.M, a.K, a.bR, a.bC = 64 * (1 << 24), 4096, 64, 16     # 2^24 block rows
    a.row_ptr = a.col_idx = a.vals = 256
    a.dtype = int(m.DType.F16)
    b = DenseDesc()
    b.data = 256
    b.scale = 1.0
    b.ldb = 128 * 128
    st = L.spmm_bcsr_mm_noalloc(ctypes.byref(a), ctypes.byref(b), 128 * 128, ctypes.c_void_p(256), 128 * 128,
                                None, None)
    assert Status(st) == Status.SCRATCH_TOO_SMALL
    assert "2^30" in m._lib.last_error()
    # exactly 2^30 items (2^22 block rows x 256 column tiles of 256 columns) is already too many
    a.M = 64 * (1 << 22)
    b.ldb = 128 * 512
    st = L.spmm_bcsr_mm_noalloc(ctypes.byref(a), ctypes.byref(b), 128 * 512, ctypes.c_void_p(256), 128 * 512,
                                None, None)
    assert Status(st) == Status.SCRATCH_TOO_SMALL
    # split-K multiplies the items: 2^21 block rows x 64 tiles fit, x 8 slices do not
    a.M = 64 * (1 << 21)
    cfg = Config()
    cfg.split_k = 8
    b.ldb = 256 * 64
    st = L.spmm_bcsr_mm_noalloc(ctypes.byref(a), ctypes.byref(b), 256 * 64, ctypes.c_void_p(256), 256 * 64,
                                ctypes.byref(cfg), None)
    assert Status(st) == Status.SCRATCH_TOO_SMALL, m._lib.last_error()
    a.M = 1024
    a.dtype = int(m.DType.E4M3)
    st = L.spmm_bcsr_mm_noalloc(ctypes.byref(a), ctypes.byref(b), 128, ctypes.c_void_p(256), 128, None, None)
    assert Status(st) == Status.UNSUPPORTED


def test_leaves_device_memory_untouched_in_a_fresh_process(dev):
    """In a process that never calls the regular entry point, two calls after a
    warm-up call do not change the device's free memory."""
    script = textwrap.dedent('''
        import ctypes, sys, torch
        sys.path.insert(0, %r)
        import matrixmultiplicationcuda_gb300 as m
        from matrixmultiplicationcuda_gb300._lib import Config, DenseDesc, stream_handle
        dev = torch.device("cuda", 0)
        M, K, N = 512, 1024, 256
        rp, ci = m.gen_structure(M, K, 64, m.PATTERN_RANDOM, 0.1, 0, seed=5)
        A = m.BCSR.from_host(M, K, 64, rp, ci, m.gen_values(len(ci), 64, 16, m.DIST_UNIFORM, seed=6), m.DType.F16, device=dev)
        B = torch.randn(K, N, device=dev).half()
        C = torch.empty(M, N, device=dev)
        a = A.desc(); b = DenseDesc(); b.data = B.data_ptr(); b.scale = 1.0; b.ldb = N
        L = m.lib()
        def call():
            assert L.spmm_bcsr_mm_noalloc(ctypes.byref(a), ctypes.byref(b), N, ctypes.c_void_p(C.data_ptr()), N,
                                          ctypes.byref(Config()), stream_handle()) == 0, m._lib.last_error()
        call(); torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        call(); call(); torch.cuda.synchronize()
        free1 = torch.cuda.mem_get_info()[0]
        assert L.spmm_noalloc_error_check(stream_handle()) == 0
        assert torch.isfinite(C).all()
        print("free", free0, free1)
        sys.exit(0 if free0 == free1 else 3)
    ''' % ROOT)
    r = subprocess.run([sys.executable, "-c", script], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
