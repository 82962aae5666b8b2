"""GB300 (sm_103a) BCSR sparse x dense matrix multiply.

Python access to libbcsr_spmm.so, the C ABI declared in include/bcsr_spmm.h.
Device memory and streams come from PyTorch; all arithmetic happens in the
library's own CUDA kernels. There is no CPU fallback: if the shared library is
missing, importing the compute entry points raises.

The reference-shaped launchers keep the argument lists of the reference's
kernels (src/cuda_kernels.cuh:39-114): ``sparseMatrixMulTensor(hdr, idx,
data, B, C, M, N, K)`` and the 32x16 / 64x16 / Adaptive variants.
"""
import ctypes
import os

from ._lib import (  # noqa: F401
    SpmmError,
    Status,
    DType,
    Config,
    lib,
    lib_path,
    check,
    stream_handle,
)
from .bcsr import (  # noqa: F401
    BCSR,
    spmm,
    sparseMatrixMulTensor,
    sparseMatrixMulTensor32x16,
    sparseMatrixMulTensor64x16,
    sparseMatrixMulTensorAdaptive,
    sparseMatrixMulTensorAdaptive32x16,
    sparseMatrixMulTensorAdaptive64x16,
    dense_to_bcsr,
    validate,
    quantize,
    device_error_check,
    debug_wait_timeout,
    BatchPlan,
    hcsr_mm,
    HcsrPlan,
    BcsrPlan,
    csr_mm,
    dense_mm,
    gpu_gen_structure,
    gpu_gen_values,
    gpu_gen_dense,
    gpu_generate_matrix,
)
from .host import (  # noqa: F401
    generate_matrix,
    gen_structure,
    plan_items,
    stack_structure,
    gen_values,
    gen_dense,
    host_dense_to_bcsr,
    host_dense_to_csr,
    host_dense_to_hcsr,
    mtx_load,
    mtx_load_bcsr,
    mtx_save,
    bcsr_save,
    bcsr_load,
    mat_load,
    mat_save,
    PATTERN_RANDOM,
    PATTERN_BAND,
    PATTERN_BLOCKDIAG,
    PATTERN_LOGNORMAL,
    DIST_UNIFORM,
    DIST_SCALED_NORMAL,
    DIST_NORMAL,
)

from .workloads import uneven_batch_specs, make_problem  # noqa: F401,E402

__all__ = [n for n in dir() if not n.startswith("_")]
