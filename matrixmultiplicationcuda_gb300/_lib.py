"""Loads libbcsr_spmm.so and declares the C signatures of include/bcsr_spmm.h."""
import ctypes
import enum
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
lib_path = os.path.join(_HERE, "lib", "libbcsr_spmm.so")

c_int, c_uint, c_ll, c_ull, c_size, c_float, c_double, c_vp, c_char_p = (
    ctypes.c_int, ctypes.c_uint, ctypes.c_longlong, ctypes.c_ulonglong, ctypes.c_size_t,
    ctypes.c_float, ctypes.c_double, ctypes.c_void_p, ctypes.c_char_p)


class Status(enum.IntEnum):
    OK = 0
    INVALID_ARG = 1
    UNSUPPORTED = 2
    MISALIGNED = 3
    CUDA = 4
    TIMEOUT = 5
    BAD_STRUCTURE = 6
    SCRATCH_TOO_SMALL = 7


class DType(enum.IntEnum):
    F16 = 0
    BF16 = 1
    E4M3 = 2
    F16_SPLIT = 3


class Config(ctypes.Structure):
    _fields_ = [("kernel", c_int), ("n_tile", c_int), ("stages", c_int), ("ctas_per_sm", c_int),
                ("acc_buffers", c_int), ("schedule", c_int), ("split_k", c_int)]


class BcsrDesc(ctypes.Structure):
    _fields_ = [("M", c_int), ("K", c_int), ("bR", c_int), ("bC", c_int),
                ("row_ptr", c_vp), ("col_idx", c_vp), ("vals", c_vp), ("vals_lo", c_vp),
                ("scales", c_vp), ("dtype", c_int)]


class DenseDesc(ctypes.Structure):
    _fields_ = [("data", c_vp), ("data_lo", c_vp), ("scale", c_float), ("ldb", c_int)]


class CsrDesc(ctypes.Structure):
    _fields_ = [("M", c_int), ("K", c_int), ("row_ptr", c_vp), ("col_idx", c_vp), ("vals", c_vp)]


class Problem(ctypes.Structure):
    _fields_ = [("A", BcsrDesc), ("B", DenseDesc), ("N", c_int), ("C", c_vp), ("ldc", c_int)]


class MlpShape(ctypes.Structure):
    _fields_ = [("in_", c_int), ("hidden", c_int), ("layers", c_int), ("out", c_int)]


class SpmmError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (Status(status).name, msg))
        self.status = Status(status)


# name -> (restype, argtypes)
_SIGS = {
    "spmm_abi_version": (c_int, []),
    "spmm_last_error": (c_char_p, []),
    "spmm_device_sm_count": (c_int, []),
    "spmm_device_error_check": (c_int, [c_vp]),
    "spmm_bcsr_mm": (c_int, [ctypes.POINTER(BcsrDesc), ctypes.POINTER(DenseDesc), c_int, c_vp,
                             c_int, ctypes.POINTER(Config), c_vp]),
    "spmm_bcsr_validate": (c_int, [c_vp, c_vp, c_int, c_int, c_int, c_ll, c_vp]),
    "spmm_gpu_gen_structure": (c_int, [c_int, c_int, c_int, c_int, c_double, c_double, c_ull, c_vp, c_vp, c_ll,
                                       ctypes.POINTER(c_ll), c_vp]),
    "spmm_gpu_gen_values": (c_int, [c_ll, c_int, c_int, c_int, c_ull, c_vp, c_vp]),
    "spmm_gpu_gen_dense": (c_int, [c_ll, c_int, c_ull, c_vp, c_vp]),
    "spmm_gpu_generate_matrix": (c_int, [c_int, c_int, c_double, c_char_p, c_int, c_ull, c_vp, c_vp]),
    "spmm_csr_mm": (c_int, [ctypes.POINTER(CsrDesc), ctypes.POINTER(DenseDesc), c_int, c_vp, c_int, c_vp]),
    "spmm_hcsr_plan_create": (c_int, [ctypes.POINTER(BcsrDesc), ctypes.POINTER(CsrDesc), c_vp,
                                      ctypes.POINTER(c_vp)]),
    "spmm_hcsr_plan_info": (c_int, [c_vp, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)]),
    "spmm_hcsr_plan_run": (c_int, [c_vp, ctypes.POINTER(DenseDesc), c_int, c_vp, c_int, ctypes.POINTER(Config),
                                   c_vp]),
    "spmm_hcsr_plan_destroy": (c_int, [c_vp]),
    "spmm_bcsr_plan_create": (c_int, [ctypes.POINTER(BcsrDesc), c_int, ctypes.POINTER(Config), c_vp,
                                      ctypes.POINTER(c_vp)]),
    "spmm_bcsr_plan_info": (c_int, [c_vp, ctypes.POINTER(c_int), ctypes.POINTER(c_int), ctypes.POINTER(Config)]),
    "spmm_bcsr_plan_run": (c_int, [c_vp, ctypes.POINTER(BcsrDesc), ctypes.POINTER(DenseDesc), c_int, c_vp, c_int,
                                   c_vp]),
    "spmm_bcsr_plan_run_ex": (c_int, [c_vp, ctypes.POINTER(BcsrDesc), ctypes.POINTER(DenseDesc), c_int, c_vp, c_int,
                                      ctypes.c_uint, c_vp]),
    "spmm_bcsr_plan_stacking": (c_int, [c_vp, ctypes.POINTER(c_int), ctypes.POINTER(c_ll)]),
    "spmm_bcsr_plan_destroy": (c_int, [c_vp]),
    "spmm_dense_mm": (c_int, [c_vp, c_int, ctypes.POINTER(DenseDesc), c_int, c_int, c_int, c_int, c_vp, c_int,
                              c_vp]),
    "spmm_hcsr_mm": (c_int, [ctypes.POINTER(BcsrDesc), ctypes.POINTER(CsrDesc), ctypes.POINTER(DenseDesc), c_int,
                             c_vp, c_int, ctypes.POINTER(Config), c_vp]),
    "sparseMatrixMulTensor_launch": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_uint, c_uint, c_uint, c_vp]),
    "sparseMatrixMulTensor32x16_launch": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_uint, c_uint, c_uint, c_vp]),
    "sparseMatrixMulTensor64x16_launch": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_uint, c_uint, c_uint, c_vp]),
    "sparseMatrixMulTensor_v2_launch": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_uint, c_uint, c_uint, c_vp]),
    "sparseMatrixMulTensor_option2_ldmatrix_sm80_launch": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_uint, c_uint,
                                                                   c_uint, c_vp]),
    "sparseMatrixMulTensor1_launch": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_uint, c_vp]),
    "sparseMatrixMulTensor_v3_launch": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_uint, c_uint, c_uint, c_vp]),
    "sparseMatrixMulTensor_v1_improved_launch": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_uint, c_uint, c_uint, c_vp]),
    "sparseMatrixMulTensor32x16_v2_launch": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_uint, c_uint, c_uint, c_vp]),
    "sparseMatrixMulTensor32x16_shared_launch": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_uint, c_uint, c_uint, c_vp]),
    "sparseMatrixMulTensor32x16_shared_vectorized_launch": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_uint, c_uint,
                                                                    c_uint, c_vp]),
    "sparseMatrixMulTensor32x16_v2_shared_vectorized_launch": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_uint,
                                                                       c_uint, c_uint, c_vp]),
    "sparseMatrixMulTensor64x16_v2_launch": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_uint, c_uint, c_uint, c_vp]),
    "sparseMatrixMulTensorAdaptive_launch": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_uint, c_uint, c_uint, c_uint, c_vp]),
    "sparseMatrixMulTensorAdaptive32x16_launch": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_uint, c_uint, c_uint, c_uint, c_vp]),
    "sparseMatrixMulTensorAdaptive64x16_launch": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_uint, c_uint, c_uint, c_uint, c_vp]),
    "spmm_dense_to_bcsr_count": (c_int, [c_vp, c_int, c_int, c_int, c_int, c_int, c_vp, ctypes.POINTER(c_ll), c_vp]),
    "spmm_dense_to_bcsr_fill": (c_int, [c_vp, c_int, c_int, c_int, c_int, c_int, c_vp, c_vp, c_vp, c_vp]),
    "spmm_quantize": (c_int, [c_vp, c_size, c_int, c_int, c_vp, c_vp, c_vp, c_vp]),
    "spmm_batch_plan_create": (c_int, [ctypes.POINTER(Problem), c_int, ctypes.POINTER(Config), ctypes.POINTER(c_vp)]),
    "spmm_batch_run": (c_int, [c_vp, c_vp]),
    "spmm_batch_plan_info": (c_int, [c_vp, ctypes.POINTER(c_int), ctypes.POINTER(c_int)]),
    "spmm_batch_plan_destroy": (c_int, [c_vp]),
    "spmm_debug_wait_timeout": (c_int, [c_ull, c_vp]),
    "spmm_bcsr_mm_noalloc": (c_int, [ctypes.POINTER(BcsrDesc), ctypes.POINTER(DenseDesc), c_int, c_vp,
                                     c_int, ctypes.POINTER(Config), c_vp]),
    "spmm_noalloc_error_check": (c_int, [c_vp]),
    "spmm_tune_config_count": (c_int, []),
    "spmm_tune_config": (c_int, [c_int, ctypes.POINTER(Config)]),
    "spmm_default_config": (c_int, [c_int, c_int, c_int, ctypes.POINTER(Config)]),
    "spmm_config_supported": (c_int, [c_int, c_int, c_int, ctypes.POINTER(Config)]),
    "spmm_tune_sweep": (c_int, [ctypes.POINTER(BcsrDesc), ctypes.POINTER(DenseDesc), c_int, c_vp, c_int, c_int,
                                c_int, c_vp, c_size, c_vp, c_vp]),
    "spmm_tune_sweep_b2b": (c_int, [c_vp, c_int, c_int, c_int, c_vp, c_vp]),
    "spmm_structure_features": (c_int, [ctypes.POINTER(BcsrDesc), c_int, c_vp, c_vp]),
    "spmm_mlp_param_count": (c_ll, [ctypes.POINTER(MlpShape)]),
    "spmm_mlp_workspace_floats": (c_ll, [ctypes.POINTER(MlpShape), c_int]),
    "spmm_mlp_forward": (c_int, [ctypes.POINTER(MlpShape), c_vp, c_vp, c_int, c_vp, c_vp, c_vp]),
    "spmm_mlp_backward": (c_int, [ctypes.POINTER(MlpShape), c_vp, c_vp, c_vp, c_vp, c_int, c_vp, c_vp, c_vp,
                                  c_vp]),
    "spmm_mlp_adam": (c_int, [c_vp, c_vp, c_vp, c_vp, c_ll, c_ll, c_float, c_float, c_float, c_float, c_float,
                              c_int, c_vp]),
    "spmm_cost_model_create": (c_int, [ctypes.POINTER(MlpShape), c_vp, ctypes.POINTER(c_vp)]),
    "spmm_cost_model_destroy": (c_int, [c_vp]),
    "spmm_cost_model_load": (c_int, [c_char_p, ctypes.POINTER(c_vp)]),
    "spmm_cost_model_select": (c_int, [c_vp, ctypes.POINTER(BcsrDesc), c_int, ctypes.POINTER(Config), c_vp,
                                       c_vp]),
    # host side (csrc/host)
    "spmm_structure_features_host": (c_int, [c_vp, c_vp, c_int, c_int, c_int, c_int, c_int, c_vp]),
    "spmm_generate_matrix": (c_int, [c_int, c_int, c_double, c_char_p, c_int, c_uint, c_vp]),
    "spmm_gen_structure": (c_ll, [c_int, c_int, c_int, c_int, c_double, c_double, c_ull, c_vp, c_vp]),
    "spmm_bcsr_stack_structure": (c_int, [c_vp, c_vp, c_int, c_int, ctypes.POINTER(c_ll), c_vp, c_vp, c_vp]),
    "spmm_bcsr_plan_items": (c_int, [c_vp, c_int, c_int, c_ll, ctypes.POINTER(c_int), ctypes.POINTER(c_int), c_vp,
                                     c_vp, c_vp]),
    "spmm_gen_values": (None, [c_ll, c_int, c_int, c_int, c_ull, c_vp]),
    "spmm_gen_dense": (None, [c_ll, c_int, c_ull, c_vp]),
    "spmm_mat_read_header": (c_int, [c_char_p, ctypes.POINTER(c_int), ctypes.POINTER(c_int)]),
    "spmm_mat_load": (c_int, [c_char_p, c_vp, c_size, ctypes.POINTER(c_int), ctypes.POINTER(c_int), ctypes.POINTER(c_int)]),
    "spmm_mat_save": (c_int, [c_char_p, c_vp, c_int, c_int]),
    "spmm_host_dense_to_bcsr": (c_ll, [c_vp, c_int, c_int, c_int, c_int, c_vp, c_vp, c_vp]),
    "spmm_host_dense_to_csr": (c_ll, [c_vp, c_int, c_int, c_vp, c_vp, c_vp]),
    "spmm_mtx_read_header": (c_int, [c_char_p, ctypes.POINTER(c_int), ctypes.POINTER(c_int), ctypes.POINTER(c_ll)]),
    "spmm_mtx_load": (c_int, [c_char_p, c_vp, c_size, ctypes.POINTER(c_int), ctypes.POINTER(c_int),
                              ctypes.POINTER(c_int)]),
    "spmm_mtx_load_bcsr": (c_int, [c_char_p, c_int, c_int, ctypes.POINTER(c_int), ctypes.POINTER(c_int), c_vp,
                                   ctypes.POINTER(c_ll), c_vp, c_vp, c_ll]),
    "spmm_mtx_save": (c_int, [c_char_p, c_vp, c_int, c_int]),
    "spmm_bcsr_save": (c_int, [c_char_p, c_int, c_int, c_int, c_int, c_int, c_ll, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "spmm_bcsr_load": (c_int, [c_char_p] + [ctypes.POINTER(c_int)] * 5 + [ctypes.POINTER(c_ll), c_vp, c_vp, c_vp,
                                                                          c_vp, c_vp, c_ll]),
    "spmm_host_dense_to_hcsr": (c_int, [c_vp, c_int, c_int, c_float, ctypes.POINTER(c_ll), ctypes.POINTER(c_ll),
                                        c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
}

_lib = None


def lib():
    """The loaded library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(lib_path):
            raise ImportError(
                "libbcsr_spmm.so is not built (%s); run "
                "`python -m matrixmultiplicationcuda_gb300.build` or __graft_entry__.build()" % lib_path)
        L = ctypes.CDLL(lib_path)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def last_error():
    return (lib().spmm_last_error() or b"").decode(errors="replace")


def check(status):
    if status != 0:
        raise SpmmError(status, last_error())
    return status


def stream_handle(stream=None):
    """cudaStream_t of a torch stream (default: the current stream) as c_void_p."""
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return c_vp(s.cuda_stream)
