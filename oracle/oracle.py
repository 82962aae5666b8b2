"""ctypes access to the CPU oracle (liboracle.so) and, where it was built, to the
reference's own host code (_ref/libref.so).

Test infrastructure only: imported by tests/, the smoke check and the CPU
baseline of bench.py, never by the library.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libref.so")
REF_CUBIN = os.path.join(HERE, "_ref", "ref_kernels.cubin")
REF_RUNNER = os.path.join(HERE, "libref_wmma.so")
P = ctypes.c_void_p


def reference_tree():
    """Where the reference's sources are: $MMC_REFERENCE_TREE, else the default
    that oracle/Makefile holds (the one place that names it)."""
    env = os.environ.get("MMC_REFERENCE_TREE")
    if env:
        return env
    r = subprocess.run(["make", "-s", "-C", HERE, "--no-print-directory", "print-ref"], capture_output=True,
                       text=True)
    return r.stdout.strip() or None


def build(ref_tree=None):
    """make liboracle.so (and the WMMA runner); where the reference tree is present
    (ref_tree, else reference_tree()) also the _ref build from its sources."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    ref_tree = ref_tree or reference_tree()
    if ref_tree and os.path.isdir(ref_tree):
        subprocess.run(["make", "-s", "-C", HERE, "ref", "REF=" + ref_tree], check=True)
    if os.path.exists(REF_CUBIN):
        subprocess.run(["make", "-s", "-C", HERE, "libref_wmma.so"], check=True)


_o = None


def lib():
    global _o
    if _o is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        L.oracle_generate_matrix.restype = ctypes.c_int
        L.oracle_generate_matrix.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                             ctypes.c_char_p, ctypes.c_int, ctypes.c_uint, P]
        L.oracle_f32_to_f16.argtypes = [P, P, ctypes.c_size_t]
        L.oracle_f16_to_f32.argtypes = [P, P, ctypes.c_size_t]
        L.oracle_bcsr_count.restype = ctypes.c_longlong
        L.oracle_bcsr_count.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, P]
        L.oracle_bcsr_fill.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P]
        L.oracle_cpu_matmul_ref_rows.argtypes = [P, P] + [ctypes.c_int] * 5 + [P]
        L.oracle_cpu_matmul_ref_rows_mt.argtypes = [P, P] + [ctypes.c_int] * 5 + [P, ctypes.c_int]
        L.oracle_bcsr_matmul_f32_mt.argtypes = [P, P, P, ctypes.c_int, P, ctypes.c_int, ctypes.c_int,
                                                ctypes.c_int, ctypes.c_int, P, ctypes.c_int]
        L.oracle_bcsr_matmul_f64.argtypes = [P, P, P, ctypes.c_int, ctypes.c_int, P, ctypes.c_int,
                                             ctypes.c_int, ctypes.c_int, P]
        L.oracle_bcsr_matmul_f64_mt.argtypes = [P, P, P, ctypes.c_int, ctypes.c_int, P, ctypes.c_int,
                                                ctypes.c_int, ctypes.c_int, P, ctypes.c_int]
        L.oracle_gen_structure.restype = ctypes.c_longlong
        L.oracle_gen_structure.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_double, ctypes.c_double, ctypes.c_ulonglong, P, P]
        L.oracle_gen_values.argtypes = [ctypes.c_longlong, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_ulonglong, P]
        L.oracle_gen_dense.argtypes = [ctypes.c_longlong, ctypes.c_int, ctypes.c_ulonglong, P]
        L.oracle_maxdiff.restype = ctypes.c_float
        L.oracle_maxdiff.argtypes = [P, P, ctypes.c_size_t]
        L.oracle_avgrelerr.restype = ctypes.c_float
        L.oracle_avgrelerr.argtypes = [P, P, ctypes.c_size_t]
        L.oracle_rmse.restype = ctypes.c_double
        L.oracle_rmse.argtypes = [P, P, ctypes.c_size_t]
        L.oracle_rel_errors.argtypes = [P, P, ctypes.c_size_t, P]
        _o = L
    return _o


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def generate_matrix(rows, cols, sparsity, pattern, blocksize, seed):
    out = np.empty((rows, cols), np.float32)
    rc = lib().oracle_generate_matrix(rows, cols, sparsity, pattern.encode(), blocksize, seed, _p(out))
    if rc != 0:
        raise ValueError("Unknown pattern: " + pattern)
    return out


def f32_to_f16(x):
    x = np.ascontiguousarray(x, np.float32)
    out = np.empty(x.shape, np.uint16)
    lib().oracle_f32_to_f16(_p(x), _p(out), x.size)
    return out


def f16_to_f32(h):
    h = np.ascontiguousarray(h, np.uint16)
    out = np.empty(h.shape, np.float32)
    lib().oracle_f16_to_f32(_p(h), _p(out), h.size)
    return out


def bcsr(A_half_bits, bR=16, bC=16):
    """BCSRMatrix ctor restated: (hdr, idx, data bits) or None for rejected block sizes."""
    A = np.ascontiguousarray(A_half_bits, np.uint16)
    rows, cols = A.shape
    hdr = np.empty(rows // bR + 1, np.int32)
    n = lib().oracle_bcsr_count(_p(A), rows, cols, bR, bC, _p(hdr))
    if n < 0:
        return None
    idx = np.empty(max(n, 1), np.int32)
    data = np.empty(max(n * bR * bC, 1), np.uint16)
    lib().oracle_bcsr_fill(_p(A), rows, cols, bR, bC, _p(idx), _p(data))
    return hdr, idx[:n], data[:n * bR * bC]


def hcsr(A_half_bits, threshold):
    """HCSRMatrix(matrix, threshold) restated (formats/HCSRMatrix.cpp:10-36):
    16x16 blocks whose density -- nonzero elements / 256 as a float, the
    reference's blockDensity (miscutil.cpp:76-87) -- is >= threshold go to a
    16x16 BCSR part, every other element to a CSR part (formats/CSRMatrix.cu:
    13-37, with the column index of element i taken as i % cols). Returns
    ((hdr, idx, data bits), (row_ptr, col_idx, vals bits))."""
    A = np.ascontiguousarray(A_half_bits, np.uint16)
    rows, cols = A.shape
    nz = (A & 0x7FFF) != 0
    cnt = nz.reshape(rows // 16, 16, cols // 16, 16).sum(axis=(1, 3))
    dense_blk = (cnt.astype(np.float32) / np.float32(256.0)) >= np.float32(threshold)
    mask = np.repeat(np.repeat(dense_blk, 16, axis=0), 16, axis=1)
    A1 = np.where(mask, A, np.uint16(0)).astype(np.uint16)
    A2 = np.where(mask, np.uint16(0), A).astype(np.uint16)
    part_b = bcsr(A1, 16, 16)
    nz2 = (A2 & 0x7FFF) != 0
    rp = np.concatenate([[0], np.cumsum(nz2.sum(axis=1))]).astype(np.int32)
    r, c = np.nonzero(nz2)
    return part_b, (rp, c.astype(np.int32), A2[r, c].astype(np.uint16))


def cpu_matmul_ref(A_bits, B_bits, row0=0, row1=None, threads=1):
    """cpu_matmul_ref (nvbench_main.cu:78-91) for rows [row0, row1)."""
    A = np.ascontiguousarray(A_bits, np.uint16)
    B = np.ascontiguousarray(B_bits, np.uint16)
    M, K = A.shape
    N = B.shape[1]
    row1 = M if row1 is None else row1
    C = np.empty((row1 - row0, N), np.float32)
    lib().oracle_cpu_matmul_ref_rows_mt(_p(A), _p(B), M, K, N, row0, row1, _p(C), int(threads))
    return C


def bcsr_matmul_f32_mt(row_ptr, col_idx, vals_bits, bR, B_f32, br0=0, br1=None, threads=1):
    """Block-sparse host multiply in fp32 (a CPU baseline, not a reference
    algorithm): block rows [br0, br1) of A (BCSR, fp16 bits) times B (fp32)."""
    rp = np.ascontiguousarray(row_ptr, np.int32)
    ci = np.ascontiguousarray(col_idx, np.int32)
    v = np.ascontiguousarray(vals_bits, np.uint16)
    B = np.ascontiguousarray(B_f32, np.float32)
    K, N = B.shape
    br1 = len(rp) - 1 if br1 is None else br1
    C = np.empty(((br1 - br0) * bR, N), np.float32)
    lib().oracle_bcsr_matmul_f32_mt(_p(rp), _p(ci), _p(v), bR, _p(B), K, N, br0, br1, _p(C), int(threads))
    return C


def bcsr_matmul_f64(row_ptr, col_idx, vals, bR, bC, B, br0=0, br1=None, threads=1):
    """FP64 product of a BCSR A (block values in double) and a dense B (double),
    block rows [br0, br1), split by block rows over `threads` host threads."""
    rp = np.ascontiguousarray(row_ptr, np.int32)
    ci = np.ascontiguousarray(col_idx, np.int32)
    v = np.ascontiguousarray(vals, np.float64)
    Bd = np.ascontiguousarray(B, np.float64)
    N = Bd.shape[1]
    br1 = len(rp) - 1 if br1 is None else br1
    C = np.empty(((br1 - br0) * bR, N), np.float64)
    lib().oracle_bcsr_matmul_f64_mt(_p(rp), _p(ci), _p(v), bR, bC, _p(Bd), N, br0, br1, _p(C), int(threads))
    return C


PATTERN_RANDOM, PATTERN_BAND, PATTERN_BLOCKDIAG, PATTERN_LOGNORMAL = 0, 1, 2, 3
DIST_UNIFORM, DIST_SCALED_NORMAL, DIST_NORMAL = 0, 1, 2


def gen_structure(M, K, bR, pattern, density, param=0.0, seed=0):
    """The synthetic workloads' block structure (row_ptr, col_idx), restated
    from the library's counter-based generator definition."""
    rp = np.empty(M // bR + 1, np.int32)
    ci = np.empty(max((M // bR) * (K // 16), 1), np.int32)
    n = lib().oracle_gen_structure(M, K, bR, pattern, float(density), float(param), seed, _p(rp), _p(ci))
    if n < 0:
        raise ValueError("bad generator arguments")
    return rp, ci[:n].copy()


def gen_values(nnzb, bR, bC, dist, seed):
    """nnzb blocks of bR*bC fp32 values (flat), restated generator."""
    out = np.empty(max(nnzb * bR * bC, 1), np.float32)
    lib().oracle_gen_values(nnzb, bR, bC, dist, seed, _p(out))
    return out[:nnzb * bR * bC]


def gen_dense(rows, cols, dist, seed):
    """rows x cols fp32 values, restated generator."""
    out = np.empty((rows, cols), np.float32)
    lib().oracle_gen_dense(rows * cols, dist, seed, _p(out))
    return out


def maxdiff(A, B):
    A = np.ascontiguousarray(A, np.float32); B = np.ascontiguousarray(B, np.float32)
    return float(lib().oracle_maxdiff(_p(A), _p(B), A.size))


def avgrelerr(A, B):
    A = np.ascontiguousarray(A, np.float32); B = np.ascontiguousarray(B, np.float32)
    return float(lib().oracle_avgrelerr(_p(A), _p(B), A.size))


def rmse(A, B):
    A = np.ascontiguousarray(A, np.float32); B = np.ascontiguousarray(B, np.float32)
    return float(lib().oracle_rmse(_p(A), _p(B), A.size))


def rel_errors(C, R):
    """(max|C-R| / max|R|, ||C-R||_F / ||R||_F) against an FP64 reference R."""
    C = np.ascontiguousarray(C, np.float32)
    R = np.ascontiguousarray(R, np.float64)
    out = np.zeros(2, np.float64)
    lib().oracle_rel_errors(_p(C), _p(R), C.size, _p(out))
    return float(out[0]), float(out[1])


# ---- the reference's own host code (only where it was built from the tree) --------
_r = None


def ref_lib():
    global _r
    if _r is None:
        if not os.path.exists(REF_LIB):
            return None
        L = ctypes.CDLL(REF_LIB)
        L.ref_generate_matrix.restype = ctypes.c_int
        L.ref_generate_matrix.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                          ctypes.c_char_p, ctypes.c_int, ctypes.c_uint, P]
        L.ref_f32_to_f16.argtypes = [P, P, ctypes.c_size_t]
        L.ref_bcsr.restype = ctypes.c_longlong
        L.ref_bcsr.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P, P, P]
        L.ref_block_density.restype = ctypes.c_float
        L.ref_block_density.argtypes = [P] + [ctypes.c_int] * 6
        L.ref_load_mat.restype = ctypes.c_int
        L.ref_load_mat.argtypes = [ctypes.c_char_p, P, P, P, P, ctypes.c_size_t]
        L.ref_maxdiff.restype = ctypes.c_float
        L.ref_maxdiff.argtypes = [P, P, ctypes.c_uint]
        L.ref_avgrelerr.restype = ctypes.c_float
        L.ref_avgrelerr.argtypes = [P, P, ctypes.c_uint]
        L.ref_rmse.restype = ctypes.c_double
        L.ref_rmse.argtypes = [P, P, ctypes.c_uint]
        _r = L
    return _r


# ---- the reference's WMMA kernels (cubin built from the reference tree) -------------
_w = None


def ref_wmma_available():
    return os.path.exists(REF_CUBIN) and os.path.exists(REF_RUNNER)


def ref_wmma_launch(kernel, hdr, idx, data, B, C, M, N, stream=0):
    """Launch the reference kernel `kernel` (e.g. "sparseMatrixMulTensor") with the
    reference harness's grid. Pointers are device addresses (ints)."""
    global _w
    if _w is None:
        _w = ctypes.CDLL(REF_RUNNER)
        _w.ref_wmma_launch.restype = ctypes.c_int
        _w.ref_wmma_launch.argtypes = [ctypes.c_char_p, ctypes.c_char_p, P, P, P, P, P,
                                       ctypes.c_uint, ctypes.c_uint, P]
    rc = _w.ref_wmma_launch(REF_CUBIN.encode(), kernel.encode(), P(hdr), P(idx), P(data), P(B),
                            P(C), M, N, P(stream))
    if rc != 0:
        raise RuntimeError("reference kernel %s launch failed: %d" % (kernel, rc))
