"""Device-side API: BCSR operands held in torch device tensors, and the calls
into the library's kernels."""
import ctypes
from dataclasses import dataclass
from typing import Optional

import numpy as np

from ._lib import (BcsrDesc, Config, DenseDesc, DType, SpmmError, Status, check, lib,
                   stream_handle)

_TORCH_DT = None


def _torch():
    import torch
    return torch


def _ptr(t):
    return ctypes.c_void_p(0 if t is None else t.data_ptr())


def storage_dtype(dtype):
    torch = _torch()
    return {DType.F16: torch.float16, DType.BF16: torch.bfloat16, DType.E4M3: torch.uint8,
            DType.F16_SPLIT: torch.float16}[DType(dtype)]


@dataclass
class BCSR:
    """A on the device in the reference's BCSR layout (formats/BCSRMatrix.cuh:9-26).

    row_ptr: int32 [M/bR + 1]; col_idx: int32 [nnzb] in units of 16 columns;
    vals: [nnzb * bR * bC] blocks row-major (fp16 / bf16 / e4m3 bytes);
    vals_lo: F16_SPLIT low halves; scales: E4M3 per-block fp32 scales.
    """
    M: int
    K: int
    bR: int
    bC: int
    row_ptr: object
    col_idx: object
    vals: object
    dtype: DType = DType.F16
    vals_lo: object = None
    scales: object = None

    @property
    def nnzb(self):
        return int(self.col_idx.numel())

    def desc(self):
        d = BcsrDesc()
        d.M, d.K, d.bR, d.bC = self.M, self.K, self.bR, self.bC
        d.row_ptr = self.row_ptr.data_ptr()
        d.col_idx = self.col_idx.data_ptr() if self.col_idx.numel() else None
        d.vals = self.vals.data_ptr() if self.vals.numel() else None
        d.vals_lo = self.vals_lo.data_ptr() if self.vals_lo is not None else None
        d.scales = self.scales.data_ptr() if self.scales is not None else None
        d.dtype = int(self.dtype)
        return d

    @staticmethod
    def from_host(M, K, bR, row_ptr, col_idx, vals_f32, dtype=DType.F16, device="cuda"):
        """Upload a host BCSR (fp32 block values) and convert the values to `dtype`
        on the device with the library's conversion kernels."""
        torch = _torch()
        rp = torch.as_tensor(np.ascontiguousarray(row_ptr, np.int32)).to(device)
        ci = torch.as_tensor(np.ascontiguousarray(col_idx, np.int32)).to(device)
        v32 = torch.as_tensor(np.ascontiguousarray(vals_f32, np.float32).reshape(-1)).to(device)
        vals, lo, sc = quantize(v32, dtype, block_elems=bR * 16)
        return BCSR(M, K, bR, 16, rp, ci, vals, DType(dtype), lo, sc)


def _dense_desc(B, B_lo=None, scale=1.0, ldb=None):
    d = DenseDesc()
    d.data = B.data_ptr()
    d.data_lo = B_lo.data_ptr() if B_lo is not None else None
    d.scale = float(scale)
    d.ldb = int(ldb if ldb is not None else B.shape[-1])
    return d


def spmm(A: BCSR, B, N=None, C=None, cfg: Optional[Config] = None, stream=None, B_lo=None,
         b_scale=1.0, ldc=None):
    """C = A @ B on the device (fp32 C, allocated if not given). Asynchronous."""
    torch = _torch()
    N = int(B.shape[1]) if N is None else int(N)
    if C is None:
        C = torch.empty((A.M, N), dtype=torch.float32, device=B.device)
    ldc = int(C.stride(0)) if ldc is None else int(ldc)
    a = A.desc()
    b = _dense_desc(B, B_lo, b_scale, ldb=B.stride(0))
    st = lib().spmm_bcsr_mm(ctypes.byref(a), ctypes.byref(b), N, ctypes.c_void_p(C.data_ptr()),
                            ldc, ctypes.byref(cfg) if cfg is not None else None,
                            stream_handle(stream))
    check(st)
    return C


def hcsr_mm(A_blocks: BCSR, csr_row_ptr, csr_col_idx, csr_vals, B, N=None, C=None,
            cfg: Optional[Config] = None, stream=None, ldc=None):
    """Hybrid product C = A_blocks @ B + A_rest @ B in one launch (fp16): the
    BCSR part on the tensor cores, the CSR part (row_ptr [M+1], col_idx, fp16
    vals, device tensors) added in the same kernel's epilogue."""
    from ._lib import CsrDesc
    torch = _torch()
    N = int(B.shape[1]) if N is None else int(N)
    if C is None:
        C = torch.empty((A_blocks.M, N), dtype=torch.float32, device=B.device)
    ldc = int(C.stride(0)) if ldc is None else int(ldc)
    a = A_blocks.desc()
    r = CsrDesc()
    r.M, r.K = A_blocks.M, A_blocks.K
    r.row_ptr = csr_row_ptr.data_ptr()
    r.col_idx = csr_col_idx.data_ptr() if csr_col_idx.numel() else None
    r.vals = csr_vals.data_ptr() if csr_vals.numel() else None
    b = _dense_desc(B, None, 1.0, ldb=B.stride(0))
    check(lib().spmm_hcsr_mm(ctypes.byref(a), ctypes.byref(r), ctypes.byref(b), N, ctypes.c_void_p(C.data_ptr()),
                             ldc, ctypes.byref(cfg) if cfg is not None else None, stream_handle(stream)))
    return C


RUN_INPUTS_READY = 1   # SPMM_RUN_INPUTS_READY


class BcsrPlan:
    """A per-matrix plan for the tcgen05 pipeline (spmm_bcsr_plan_*): the item
    list ordered heaviest first, with the longest block rows split across the
    CTA slots the rows leave spare, taken by the CTAs from the plan's own work
    queue. Built once from A's row_ptr; run() is one launch on any A with the
    same structure. One plan runs one launch at a time: use one plan per
    stream for concurrent launches."""

    def __init__(self, A: BCSR, N, cfg: Optional[Config] = None, stream=None):
        a = A.desc()
        h = ctypes.c_void_p()
        check(lib().spmm_bcsr_plan_create(ctypes.byref(a), int(N), ctypes.byref(cfg) if cfg is not None else None,
                                          stream_handle(stream), ctypes.byref(h)))
        self._h = h
        self.M, self.N = A.M, int(N)

    def info(self):
        """(items, split rows, the configuration it runs)."""
        n, sp, c = ctypes.c_int(), ctypes.c_int(), Config()
        check(lib().spmm_bcsr_plan_info(self._h, ctypes.byref(n), ctypes.byref(sp), ctypes.byref(c)))
        return n.value, sp.value, c

    def stacking(self):
        """(block rows per stacked 64-row row, stacked blocks); (1, 0) when the
        plan runs the blocks as they are."""
        st, nb = ctypes.c_int(), ctypes.c_longlong()
        check(lib().spmm_bcsr_plan_stacking(self._h, ctypes.byref(st), ctypes.byref(nb)))
        return st.value, nb.value

    def run(self, A: BCSR, B, C=None, stream=None, B_lo=None, b_scale=1.0, ldc=None, inputs_ready=False):
        """One launch. inputs_ready=True (SPMM_RUN_INPUTS_READY) promises that no
        kernel launched on the stream since its last host synchronisation writes A
        or B: the launch then copies and multiplies its first items while the kernel
        before it is still running, and waits for that kernel only before it claims
        queued work or writes C."""
        torch = _torch()
        if C is None:
            C = torch.empty((self.M, self.N), dtype=torch.float32, device=B.device)
        ldc = int(C.stride(0)) if ldc is None else int(ldc)
        a = A.desc()
        b = _dense_desc(B, B_lo, b_scale, ldb=B.stride(0))
        check(lib().spmm_bcsr_plan_run_ex(self._h, ctypes.byref(a), ctypes.byref(b), self.N,
                                          ctypes.c_void_p(C.data_ptr()), ldc, RUN_INPUTS_READY if inputs_ready else 0,
                                          stream_handle(stream)))
        return C

    def close(self):
        if self._h:
            lib().spmm_bcsr_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class HcsrPlan:
    """The planned hybrid product (fp16, 16x16 blocks): the CSR part packed once
    into gather blocks that the tcgen05 pipeline runs beside the stored blocks.
    The plan copies both parts; run() is one launch."""

    def __init__(self, A_blocks: BCSR, csr_row_ptr, csr_col_idx, csr_vals, stream=None):
        from ._lib import CsrDesc
        a = A_blocks.desc()
        r = CsrDesc()
        r.M, r.K = A_blocks.M, A_blocks.K
        r.row_ptr = csr_row_ptr.data_ptr()
        r.col_idx = csr_col_idx.data_ptr() if csr_col_idx.numel() else None
        r.vals = csr_vals.data_ptr() if csr_vals.numel() else None
        self.M, self.K = A_blocks.M, A_blocks.K
        h = ctypes.c_void_p()
        check(lib().spmm_hcsr_plan_create(ctypes.byref(a), ctypes.byref(r), stream_handle(stream), ctypes.byref(h)))
        self._h = h

    def info(self):
        """(blocks, gather_blocks) of the packed matrix."""
        nb, ng = ctypes.c_longlong(), ctypes.c_longlong()
        check(lib().spmm_hcsr_plan_info(self._h, ctypes.byref(nb), ctypes.byref(ng)))
        return nb.value, ng.value

    def run(self, B, N=None, C=None, cfg: Optional[Config] = None, stream=None, ldc=None):
        torch = _torch()
        N = int(B.shape[1]) if N is None else int(N)
        if C is None:
            C = torch.empty((self.M, N), dtype=torch.float32, device=B.device)
        ldc = int(C.stride(0)) if ldc is None else int(ldc)
        b = _dense_desc(B, None, 1.0, ldb=B.stride(0))
        check(lib().spmm_hcsr_plan_run(self._h, ctypes.byref(b), N, ctypes.c_void_p(C.data_ptr()), ldc,
                                       ctypes.byref(cfg) if cfg is not None else None, stream_handle(stream)))
        return C

    def close(self):
        if self._h:
            lib().spmm_hcsr_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def dense_mm(A, B, C=None, stream=None):
    """Dense A (M x K) @ B (K x N), fp16 or bf16 device tensors (row-major, rows
    16-byte aligned), fp32 C, on the tcgen05 tensor cores: the native dense
    comparator."""
    torch = _torch()
    M, K = int(A.shape[0]), int(A.shape[1])
    N = int(B.shape[1])
    if A.dtype != B.dtype or A.dtype not in (torch.float16, torch.bfloat16):
        raise SpmmError(Status.UNSUPPORTED, "A and B must both be fp16 or both bf16")
    dt = DType.BF16 if A.dtype == torch.bfloat16 else DType.F16
    if C is None:
        C = torch.empty((M, N), dtype=torch.float32, device=B.device)
    b = _dense_desc(B, None, 1.0, ldb=B.stride(0))
    check(lib().spmm_dense_mm(ctypes.c_void_p(A.data_ptr()), int(A.stride(0)), ctypes.byref(b), M, K, N, int(dt),
                              ctypes.c_void_p(C.data_ptr()), int(C.stride(0)), stream_handle(stream)))
    return C


def csr_mm(row_ptr, col_idx, vals, K, B, N=None, C=None, stream=None, ldc=None):
    """CSR x dense (fp16, device tensors), C fp32: the native comparator."""
    from ._lib import CsrDesc
    torch = _torch()
    N = int(B.shape[1]) if N is None else int(N)
    M = row_ptr.numel() - 1
    if C is None:
        C = torch.empty((M, N), dtype=torch.float32, device=B.device)
    r = CsrDesc()
    r.M, r.K = M, int(K)
    r.row_ptr = row_ptr.data_ptr()
    r.col_idx = col_idx.data_ptr() if col_idx.numel() else None
    r.vals = vals.data_ptr() if vals.numel() else None
    b = _dense_desc(B, None, 1.0, ldb=B.stride(0))
    check(lib().spmm_csr_mm(ctypes.byref(r), ctypes.byref(b), N, ctypes.c_void_p(C.data_ptr()),
                            int(C.stride(0)) if ldc is None else int(ldc), stream_handle(stream)))
    return C


def _ref_launch(fn, hdr, idx, data, B, C, M, N, K, stream, extra=()):
    st = fn(_ptr(hdr), _ptr(idx), _ptr(data), _ptr(B), _ptr(C), int(M), int(N), *extra, int(K),
            stream_handle(stream))
    check(st)
    return C


# Reference-shaped launchers (src/cuda_kernels.cuh:39-114 argument order, + K, + stream).
def sparseMatrixMulTensor(hdr, idx, data, B, C, M, N, K, stream=None):
    return _ref_launch(lib().sparseMatrixMulTensor_launch, hdr, idx, data, B, C, M, N, K, stream)


def sparseMatrixMulTensor32x16(hdr, idx, data, B, C, M, N, K, stream=None):
    return _ref_launch(lib().sparseMatrixMulTensor32x16_launch, hdr, idx, data, B, C, M, N, K, stream)


def sparseMatrixMulTensor64x16(hdr, idx, data, B, C, M, N, K, stream=None):
    return _ref_launch(lib().sparseMatrixMulTensor64x16_launch, hdr, idx, data, B, C, M, N, K, stream)


def sparseMatrixMulTensorAdaptive(hdr, idx, data, B, C, M, N, colBlocksPerRow, K, stream=None):
    return _ref_launch(lib().sparseMatrixMulTensorAdaptive_launch, hdr, idx, data, B, C, M, N, K,
                       stream, (int(colBlocksPerRow),))


def sparseMatrixMulTensorAdaptive32x16(hdr, idx, data, B, C, M, N, colBlocksPerRow, K, stream=None):
    return _ref_launch(lib().sparseMatrixMulTensorAdaptive32x16_launch, hdr, idx, data, B, C, M, N,
                       K, stream, (int(colBlocksPerRow),))


def sparseMatrixMulTensorAdaptive64x16(hdr, idx, data, B, C, M, N, colBlocksPerRow, K, stream=None):
    return _ref_launch(lib().sparseMatrixMulTensorAdaptive64x16_launch, hdr, idx, data, B, C, M, N,
                       K, stream, (int(colBlocksPerRow),))


def dense_to_bcsr(A_half, bR=16, bC=16, stream=None):
    """GPU BCSRMatrix constructor: (row_ptr, col_idx, vals) device tensors, bit-exact
    to formats/BCSRMatrix.cu:22-74. Synchronises once (to size the outputs)."""
    torch = _torch()
    M, K = A_half.shape
    lda = A_half.stride(0)
    MB = M // bR
    rp = torch.empty(MB + 1, dtype=torch.int32, device=A_half.device)
    nnzb = ctypes.c_longlong(0)
    s = stream_handle(stream)
    check(lib().spmm_dense_to_bcsr_count(_ptr(A_half), M, K, lda, bR, bC, _ptr(rp),
                                         ctypes.byref(nnzb), s))
    ci = torch.empty(max(nnzb.value, 0), dtype=torch.int32, device=A_half.device)
    vals = torch.empty(max(nnzb.value, 0) * bR * bC, dtype=torch.float16, device=A_half.device)
    if nnzb.value:
        check(lib().spmm_dense_to_bcsr_fill(_ptr(A_half), M, K, lda, bR, bC, _ptr(rp), _ptr(ci),
                                            _ptr(vals), s))
    return rp, ci, vals


def gpu_gen_structure(M, K, bR, pattern, density, param=0.0, seed=1, device="cuda", stream=None):
    """BCSR structure generated on the GPU: (row_ptr, col_idx) device tensors
    (the host gen_structure's streams; see spmm_gpu_gen_structure)."""
    torch = _torch()
    rp = torch.empty(M // bR + 1, dtype=torch.int32, device=device)
    n = ctypes.c_longlong(0)
    s = stream_handle(stream)
    check(lib().spmm_gpu_gen_structure(M, K, bR, pattern, float(density), float(param), seed, _ptr(rp), None, 0,
                                       ctypes.byref(n), s))
    ci = torch.empty(max(n.value, 1), dtype=torch.int32, device=device)
    check(lib().spmm_gpu_gen_structure(M, K, bR, pattern, float(density), float(param), seed, _ptr(rp), _ptr(ci),
                                       n.value, ctypes.byref(n), s))
    return rp, ci[:n.value]


def gpu_gen_values(nnzb, bR, bC=16, dist=0, seed=2, device="cuda", stream=None):
    torch = _torch()
    out = torch.empty(nnzb * bR * bC, dtype=torch.float32, device=device)
    check(lib().spmm_gpu_gen_values(nnzb, bR, bC, dist, seed, _ptr(out), stream_handle(stream)))
    return out


def gpu_gen_dense(rows, cols, dist=0, seed=3, device="cuda", stream=None):
    torch = _torch()
    out = torch.empty((rows, cols), dtype=torch.float32, device=device)
    check(lib().spmm_gpu_gen_dense(rows * cols, dist, seed, _ptr(out), stream_handle(stream)))
    return out


def gpu_generate_matrix(rows, cols, sparsity=0.7, pattern="random", blocksize=16, seed=123, device="cuda",
                        stream=None):
    """A dense fp16 matrix in one of the reference generator's patterns, made on the GPU."""
    torch = _torch()
    out = torch.empty((rows, cols), dtype=torch.float16, device=device)
    check(lib().spmm_gpu_generate_matrix(rows, cols, float(sparsity), pattern.encode(), blocksize, seed, _ptr(out),
                                         stream_handle(stream)))
    return out


def validate(A: BCSR, stream=None):
    check(lib().spmm_bcsr_validate(_ptr(A.row_ptr), _ptr(A.col_idx) if A.nnzb else None, A.M, A.K,
                                   A.bR, A.nnzb, stream_handle(stream)))


def quantize(src_f32, dtype, block_elems=None, stream=None):
    """fp32 device tensor -> (values, low halves or None, scales or None) in `dtype`."""
    torch = _torch()
    dtype = DType(dtype)
    n = src_f32.numel()
    dev = src_f32.device
    dst = torch.empty(n, dtype=storage_dtype(dtype), device=dev)
    lo = torch.empty(n, dtype=torch.float16, device=dev) if dtype == DType.F16_SPLIT else None
    sc = None
    be = 0
    if dtype == DType.E4M3:
        be = int(block_elems if block_elems else n)
        sc = torch.empty((n + be - 1) // be if n else 0, dtype=torch.float32, device=dev)
    if n:
        check(lib().spmm_quantize(_ptr(src_f32), n, int(dtype), be, _ptr(dst), _ptr(lo), _ptr(sc),
                                  stream_handle(stream)))
    return dst, lo, sc


def device_error_check(stream=None):
    check(lib().spmm_device_error_check(stream_handle(stream)))


def debug_wait_timeout(timeout_ns, stream=None):
    """Returns the Status of the bounded-wait diagnostic (TIMEOUT expected)."""
    return Status(lib().spmm_debug_wait_timeout(int(timeout_ns), stream_handle(stream)))


class BatchPlan:
    """Many independent products C_i = A_i @ B_i in one persistent launch
    (spmm_batch_plan_create / spmm_batch_run). The plan reads each A_i's row
    pointers once, orders the (problem, block row, column tile) items heaviest
    first and keeps them on the device; run() only launches, so it can be
    captured in a CUDA graph and replayed. The tensors are referenced by the
    plan and must stay alive and in place while it is used."""

    def __init__(self, problems, cfg: Optional[Config] = None):
        """problems: list of (A: BCSR, B [K, N] tensor, C [M, N] fp32 tensor)."""
        from ._lib import Problem
        self._keep = list(problems)
        arr = (Problem * max(len(problems), 1))()
        for i, (A, B, C) in enumerate(problems):
            arr[i].A = A.desc()
            arr[i].B = _dense_desc(B, ldb=B.stride(0))
            arr[i].N = int(B.shape[1])
            arr[i].C = C.data_ptr()
            arr[i].ldc = int(C.stride(0))
        self._arr = arr
        h = ctypes.c_void_p()
        check(lib().spmm_batch_plan_create(arr, len(problems),
                                           ctypes.byref(cfg) if cfg is not None else None,
                                           ctypes.byref(h)))
        self._h = h

    def run(self, stream=None):
        check(lib().spmm_batch_run(self._h, stream_handle(stream)))

    def info(self):
        """(items of the launch, problems run stacked into 64-row blocks)."""
        n, st = ctypes.c_int(), ctypes.c_int()
        check(lib().spmm_batch_plan_info(self._h, ctypes.byref(n), ctypes.byref(st)))
        return n.value, st.value

    def close(self):
        if self._h:
            lib().spmm_batch_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
