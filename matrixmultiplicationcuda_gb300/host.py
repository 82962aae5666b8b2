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


def plan_items(row_ptr, ntiles, slots):
    """The per-matrix plan's item list on the host (spmm_bcsr_plan_items):
    (items [n, 4] = {block row, column tile, first block, end block} heaviest
    first, pair [n] = -1 or 128 * group + part, parts [groups])."""
    rp = np.ascontiguousarray(row_ptr, np.int32)
    n, g = ctypes.c_int(), ctypes.c_int()
    check(lib().spmm_bcsr_plan_items(_vp(rp), len(rp) - 1, int(ntiles), int(slots), ctypes.byref(n), ctypes.byref(g),
                                     None, None, None))
    items = np.empty((max(n.value, 1), 4), np.int32)
    pair = np.empty(max(n.value, 1), np.int32)
    parts = np.empty(max(g.value, 1), np.int32)
    check(lib().spmm_bcsr_plan_items(_vp(rp), len(rp) - 1, int(ntiles), int(slots), ctypes.byref(n), ctypes.byref(g),
                                     _vp(items), _vp(pair), _vp(parts)))
    return items[:n.value], pair[:n.value], parts[:g.value]


def stack_structure(row_ptr, col_idx, rows_per_stack):
    """The stacked structure a plan builds for 16- or 32-row blocks
    (spmm_bcsr_stack_structure): (row_ptr, col_idx, map [blocks, rows_per_stack]
    of source block indices or -1)."""
    rp = np.ascontiguousarray(row_ptr, np.int32)
    ci = np.ascontiguousarray(col_idx, np.int32)
    if ci.size == 0:
        ci = np.zeros(1, np.int32)
    MB = len(rp) - 1
    n = ctypes.c_longlong()
    check(lib().spmm_bcsr_stack_structure(_vp(rp), _vp(ci), MB, int(rows_per_stack), ctypes.byref(n), None, None,
                                          None))
    srp = np.empty(MB // rows_per_stack + 1, np.int32)
    sci = np.empty(max(n.value, 1), np.int32)
    smap = np.empty(max(n.value, 1) * rows_per_stack, np.int32)
    check(lib().spmm_bcsr_stack_structure(_vp(rp), _vp(ci), MB, int(rows_per_stack), ctypes.byref(n), _vp(srp),
                                          _vp(sci), _vp(smap)))
    return srp, sci[:n.value], smap[:n.value * rows_per_stack].reshape(-1, rows_per_stack)


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


def mtx_load(path):
    """A Matrix Market file as a dense fp16 matrix: (half bits [rows, cols], nonZeros)."""
    r, c, n = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_longlong(0)
    check(lib().spmm_mtx_read_header(str(path).encode(), ctypes.byref(r), ctypes.byref(c), ctypes.byref(n)))
    out = np.empty((r.value, c.value), np.uint16)
    nz = ctypes.c_int(0)
    check(lib().spmm_mtx_load(str(path).encode(), _vp(out), out.size, ctypes.byref(r), ctypes.byref(c),
                              ctypes.byref(nz)))
    return out, nz.value


def mtx_load_bcsr(path, bR=16, bC=16):
    """A Matrix Market file straight into BCSR: (rows, cols, row_ptr, col_idx, fp16 value bits)."""
    r, c, n = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_longlong(0)
    check(lib().spmm_mtx_read_header(str(path).encode(), ctypes.byref(r), ctypes.byref(c), ctypes.byref(n)))
    rp = np.empty(r.value // bR + 1, np.int32)
    nnzb = ctypes.c_longlong(0)
    check(lib().spmm_mtx_load_bcsr(str(path).encode(), bR, bC, ctypes.byref(r), ctypes.byref(c), _vp(rp),
                                   ctypes.byref(nnzb), None, None, 0))
    ci = np.empty(max(nnzb.value, 1), np.int32)
    vals = np.empty(max(nnzb.value * bR * bC, 1), np.uint16)
    check(lib().spmm_mtx_load_bcsr(str(path).encode(), bR, bC, ctypes.byref(r), ctypes.byref(c), _vp(rp),
                                   ctypes.byref(nnzb), _vp(ci), _vp(vals), nnzb.value))
    return r.value, c.value, rp, ci[:nnzb.value], vals[:nnzb.value * bR * bC]


def mtx_save(path, vals_f32):
    v = np.ascontiguousarray(vals_f32, np.float32)
    check(lib().spmm_mtx_save(str(path).encode(), _vp(v), v.shape[0], v.shape[1]))


def bcsr_save(path, M, K, bR, bC, row_ptr, col_idx, vals, dtype=0, vals_lo=None, scales=None):
    """The binary BCSR file (host arrays; vals as raw element bits)."""
    arrs = [np.ascontiguousarray(a) for a in (row_ptr, col_idx, vals)]
    lo = np.ascontiguousarray(vals_lo) if vals_lo is not None else None
    sc = np.ascontiguousarray(scales, np.float32) if scales is not None else None
    check(lib().spmm_bcsr_save(str(path).encode(), M, K, bR, bC, int(dtype), len(arrs[1]), _vp(arrs[0]),
                               _vp(arrs[1]) if len(arrs[1]) else None, _vp(arrs[2]) if arrs[2].size else None,
                               _vp(lo) if lo is not None else None, _vp(sc) if sc is not None else None))


def bcsr_load(path):
    """(M, K, bR, bC, dtype, row_ptr, col_idx, vals bits, vals_lo bits or None, scales or None)."""
    h = [ctypes.c_int(0) for _ in range(5)]
    n = ctypes.c_longlong(0)
    check(lib().spmm_bcsr_load(str(path).encode(), *[ctypes.byref(x) for x in h], ctypes.byref(n),
                               None, None, None, None, None, 0))
    M, K, bR, bC, dt = (x.value for x in h)
    esz = np.uint8 if dt == 2 else np.uint16
    rp = np.empty(M // bR + 1, np.int32)
    ci = np.empty(max(n.value, 1), np.int32)
    vals = np.empty(max(n.value * bR * bC, 1), esz)
    lo = np.empty(max(n.value * bR * bC, 1), np.uint16) if dt == 3 else None
    sc = np.empty(max(n.value, 1), np.float32) if dt == 2 else None
    check(lib().spmm_bcsr_load(str(path).encode(), *[ctypes.byref(x) for x in h], ctypes.byref(n), _vp(rp), _vp(ci),
                               _vp(vals), _vp(lo) if lo is not None else None, _vp(sc) if sc is not None else None,
                               n.value))
    k = n.value
    return (M, K, bR, bC, dt, rp, ci[:k], vals[:k * bR * bC], lo[:k * bR * bC] if lo is not None else None,
            sc[:k] if sc is not None else None)
