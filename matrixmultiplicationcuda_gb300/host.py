"""Host-side API: generators, the .mat text format, host BCSR/CSR construction.
All of it runs the library's C++ host code (csrc/host)."""
import ctypes

import numpy as np

from ._lib import SpmmError, Status, check, last_error, lib

PATTERN_RANDOM, PATTERN_BAND, PATTERN_BLOCKDIAG, PATTERN_LOGNORMAL = 0, 1, 2, 3
DIST_UNIFORM, DIST_SCALED_NORMAL, DIST_NORMAL = 0, 1, 2


def _vp(a):
    return ctypes.c_void_p(a.ctypes.data)


def generate_matrix(rows, cols, sparsity=0.7, pattern="random", blocksize=16, seed=123):
    """mg::generate_matrix<float> (matrix_generator.cpp:28-140): float32 [rows, cols]."""
    out = np.empty((rows, cols), np.float32)
    if lib().spmm_generate_matrix(rows, cols, float(sparsity), pattern.encode(), blocksize,
                                  seed, _vp(out)) != 0:
        raise SpmmError(Status.INVALID_ARG, last_error())
    return out


def gen_structure(M, K, bR, pattern, density, param=0.0, seed=1):
    """BCSR structure (row_ptr, col_idx) of an M x K matrix with bR x 16 blocks."""
    MB, KB = M // bR, K // 16
    rp = np.empty(MB + 1, np.int32)
    ci = np.empty(max(MB * KB, 1), np.int32)
    n = lib().spmm_gen_structure(M, K, bR, pattern, float(density), float(param), seed, _vp(rp),
                                 _vp(ci))
    if n < 0:
        raise SpmmError(Status.INVALID_ARG, last_error())
    return rp, ci[:n].copy()


def gen_values(nnzb, bR, bC=16, dist=DIST_UNIFORM, seed=2):
    out = np.empty(nnzb * bR * bC, np.float32)
    lib().spmm_gen_values(nnzb, bR, bC, dist, seed, _vp(out))
    return out


def gen_dense(rows, cols, dist=DIST_UNIFORM, seed=3):
    out = np.empty((rows, cols), np.float32)
    lib().spmm_gen_dense(rows * cols, dist, seed, _vp(out))
    return out


def host_dense_to_bcsr(A_half_bits, bR=16, bC=16):
    """BCSRMatrix(matrix, bR, bC) on the host: (hdr, idx, data as uint16 bits)."""
    A = np.ascontiguousarray(A_half_bits).view(np.uint16)
    rows, cols = A.shape
    n = lib().spmm_host_dense_to_bcsr(_vp(A), rows, cols, bR, bC, None, None, None)
    if n < 0:
        raise SpmmError(Status.INVALID_ARG, last_error())
    hdr = np.empty(rows // bR + 1, np.int32)
    idx = np.empty(max(n, 1), np.int32)
    data = np.empty(max(n * bR * bC, 1), np.uint16)
    lib().spmm_host_dense_to_bcsr(_vp(A), rows, cols, bR, bC, _vp(hdr), _vp(idx), _vp(data))
    return hdr, idx[:n], data[:n * bR * bC]


def host_dense_to_hcsr(A_half_bits, threshold):
    """HCSRMatrix(matrix, threshold) (formats/HCSRMatrix.cpp:10-36) on the host:
    ((hdr, idx, data bits) of the 16x16 BCSR part, (row_ptr, col_idx, vals bits)
    of the CSR part)."""
    A = np.ascontiguousarray(A_half_bits).view(np.uint16)
    rows, cols = A.shape
    nnzb, nnz = ctypes.c_longlong(0), ctypes.c_longlong(0)
    if lib().spmm_host_dense_to_hcsr(_vp(A), rows, cols, float(threshold), ctypes.byref(nnzb), ctypes.byref(nnz),
                                     None, None, None, None, None, None) != 0:
        raise SpmmError(Status.INVALID_ARG, last_error())
    bh = np.empty(rows // 16 + 1, np.int32)
    bi = np.empty(max(nnzb.value, 1), np.int32)
    bd = np.empty(max(nnzb.value * 256, 1), np.uint16)
    ch = np.empty(rows + 1, np.int32)
    cx = np.empty(max(nnz.value, 1), np.int32)
    cd = np.empty(max(nnz.value, 1), np.uint16)
    lib().spmm_host_dense_to_hcsr(_vp(A), rows, cols, float(threshold), ctypes.byref(nnzb), ctypes.byref(nnz),
                                  _vp(bh), _vp(bi), _vp(bd), _vp(ch), _vp(cx), _vp(cd))
    return (bh, bi[:nnzb.value], bd[:nnzb.value * 256]), (ch, cx[:nnz.value], cd[:nnz.value])


def host_dense_to_csr(A_half_bits):
    A = np.ascontiguousarray(A_half_bits).view(np.uint16)
    rows, cols = A.shape
    n = lib().spmm_host_dense_to_csr(_vp(A), rows, cols, None, None, None)
    hdr = np.empty(rows + 1, np.int32)
    idx = np.empty(max(n, 1), np.int32)
    data = np.empty(max(n, 1), np.uint16)
    lib().spmm_host_dense_to_csr(_vp(A), rows, cols, _vp(hdr), _vp(idx), _vp(data))
    return hdr, idx[:n], data[:n]


def mat_load(path):
    """Matrix(path) (Matrix.cu:14-32): (half bits [rows, cols] as uint16, nonZeros)."""
    r, c = ctypes.c_int(0), ctypes.c_int(0)
    check(lib().spmm_mat_read_header(str(path).encode(), ctypes.byref(r), ctypes.byref(c)))
    out = np.empty((r.value, c.value), np.uint16)
    nz = ctypes.c_int(0)
    check(lib().spmm_mat_load(str(path).encode(), _vp(out), out.size, ctypes.byref(r),
                              ctypes.byref(c), ctypes.byref(nz)))
    return out, nz.value


def mat_save(path, vals_f32):
    v = np.ascontiguousarray(vals_f32, np.float32)
    check(lib().spmm_mat_save(str(path).encode(), _vp(v), v.shape[0], v.shape[1]))
