"""Writes tests/golden/reference_golden.npz from the reference's OWN host code.

Run in a checkout that has the reference tree (it builds oracle/_ref/libref.so
from it first):

    python tests/golden/make_golden.py /path/to/MatrixMultiplicationCUDA

What is stored (all produced by the reference's sources, not by the oracle):
  * mg::generate_matrix<float> outputs for every pattern on small shapes
    (matrix_generator.cpp:28-140), as float32 bits;
  * __float2half outputs for edge-case and random floats;
  * BCSRMatrix(matrix, bR, bC) arrays (formats/BCSRMatrix.cu:22-74) for
    generated matrices and for hand-made blocks holding only -0 / only NaN;
  * the 1024 x 1024 blockrandom workload (16x16 blocks, 10% kept, seed 123):
    row_ptr, col_idx and a SHA-256 of the stored fp16 block values;
  * Matrix(".mat path") of a small text file (rows, cols, nonZeros, half bits);
  * maxdiff / avgrelerr / rmse (miscutil.cpp:35-74) on a 16 x 16 pair;
  * HCSRMatrix(matrix, threshold) (formats/HCSRMatrix.cpp:10-36) of a 128 x 128
    matrix with mixed block densities, at six thresholds: both parts' arrays.
"""
import ctypes
import hashlib
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import oracle  # noqa: E402

PATTERNS = ["random", "checkerboard", "diagonal", "blockdiagonal", "blockrandom",
            "pattern64by16", "pattern32by16"]
GEN_CASES = [(64, 48, 0.7, 16, 123), (100, 70, 0.5, 16, 7), (128, 128, 0.9, 32, 456)]


def p(a):
    return ctypes.c_void_p(a.ctypes.data)


def main(ref_tree):
    oracle.build(ref_tree)
    R = oracle.ref_lib()
    assert R is not None, "reference build missing"
    out = {}
    for pat in PATTERNS:
        for (r, c, sp, bs, seed) in GEN_CASES:
            m = np.empty((r, c), np.float32)
            assert R.ref_generate_matrix(r, c, sp, pat.encode(), bs, seed, p(m)) == 0
            out["gen/%s/%d_%d_%g_%d_%d" % (pat, r, c, sp, bs, seed)] = m.view(np.uint32)
    # float -> half
    rng = np.random.default_rng(2024)
    x = np.concatenate([
        np.array([0.0, -0.0, np.inf, -np.inf, 65504, 65519.99, 65520, 1e-8, 2.98e-8, 2.99e-8,
                  5.96e-8, 6e-5, 6.1e-5, -6.1e-5, 1e-7, 3e-5, 1.0, -1.0, 0.5, 1e38, 16383.063,
                  -8190.2666], np.float32),
        (rng.standard_normal(4000) * 3e4).astype(np.float32),
        (rng.standard_normal(4000) * 1e-4).astype(np.float32),
        rng.uniform(-1, 1, 4000).astype(np.float32)])
    h = np.empty(x.size, np.uint16)
    R.ref_f32_to_f16(p(x), p(h), x.size)
    out["f16/in"] = x.view(np.uint32)
    out["f16/out"] = h

    def ref_bcsr(Abits, bR, bC):
        rows, cols = Abits.shape
        n = R.ref_bcsr(p(Abits), rows, cols, bR, bC, None, None, None, None)
        if n < 0:
            return None
        hdr = np.empty(rows // bR + 1, np.int32)
        idx = np.empty(max(n, 1), np.int32)
        data = np.empty(max(n * bR * bC, 1), np.uint16)
        nz = ctypes.c_int(0)
        R.ref_bcsr(p(Abits), rows, cols, bR, bC, p(hdr), p(idx), p(data), ctypes.byref(nz))
        return hdr, idx[:n], data[:n * bR * bC], nz.value

    def to_half(f):
        hb = np.empty(f.shape, np.uint16)
        R.ref_f32_to_f16(p(np.ascontiguousarray(f)), p(hb), f.size)
        return hb

    for (pat, r, c, sp, bs, bR, bC) in [("blockrandom", 128, 96, 0.6, 16, 16, 16),
                                        ("pattern32by16", 128, 64, 0.5, 16, 32, 16),
                                        ("pattern64by16", 256, 64, 0.5, 16, 64, 16),
                                        ("random", 64, 64, 0.97, 16, 16, 32),
                                        ("checkerboard", 96, 96, 0.0, 32, 32, 32)]:
        m = np.empty((r, c), np.float32)
        R.ref_generate_matrix(r, c, sp, pat.encode(), bs, 123, p(m))
        hb = to_half(m)
        res = ref_bcsr(hb, bR, bC)
        key = "bcsr/%s/%d_%d_%d_%d" % (pat, r, c, bR, bC)
        out[key + "/A"] = hb
        out[key + "/hdr"], out[key + "/idx"], out[key + "/data"] = res[0], res[1], res[2]
        out[key + "/nonZeros"] = np.array([res[3]], np.int64)
    # -0 and NaN blocks: a block of only -0 is empty, a block with one NaN is kept
    A = np.zeros((32, 64), np.uint16)
    A[0:16, 0:16] = 0x8000                   # -0 everywhere
    A[3, 20] = 0x7e00                        # NaN
    A[20, 40] = 0x0001                       # smallest subnormal
    A[31, 63] = 0xfc00                       # -inf
    res = ref_bcsr(A, 16, 16)
    out["bcsr/special/A"] = A
    out["bcsr/special/hdr"], out["bcsr/special/idx"], out["bcsr/special/data"] = res[0], res[1], res[2]
    out["bcsr/special/density"] = np.array(
        [R.ref_block_density(p(A), 32, 64, i, j, 16, 16) for i in (0, 16) for j in (0, 16, 32, 48)],
        np.float32)
    # invalid block sizes are rejected
    out["bcsr/reject"] = np.array([ref_bcsr(A, 8, 16) is None, ref_bcsr(A, 16, 24) is None], np.int8)
    # C1 workload structure
    m = np.empty((1024, 1024), np.float32)
    R.ref_generate_matrix(1024, 1024, 0.9, b"blockrandom", 16, 123, p(m))
    hb = to_half(m)
    res = ref_bcsr(hb, 16, 16)
    out["c1/hdr"], out["c1/idx"] = res[0], res[1]
    out["c1/data_sha256"] = np.frombuffer(hashlib.sha256(res[2].tobytes()).digest(), np.uint8)
    mb = np.empty((1024, 1024), np.float32)
    R.ref_generate_matrix(1024, 1024, 0.0, b"random", 16, 456, p(mb))
    out["c1/B_sha256"] = np.frombuffer(hashlib.sha256(to_half(mb).tobytes()).digest(), np.uint8)
    # .mat loader
    vals = np.round(rng.uniform(-2, 2, (5, 7)), 3).astype(np.float32)
    vals[1, :3] = 0
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "m.mat")
        with open(path, "w") as f:
            f.write("5 7\n" + "\n".join(" ".join("%g" % v for v in row) for row in vals) + "\n")
        rr, cc, nz = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        buf = np.empty(35, np.uint16)
        R.ref_load_mat(path.encode(), ctypes.byref(rr), ctypes.byref(cc), ctypes.byref(nz), p(buf), 35)
        out["mat/text"] = np.frombuffer(open(path, "rb").read(), np.uint8)
    out["mat/shape_nz"] = np.array([rr.value, cc.value, nz.value], np.int32)
    out["mat/half"] = buf.reshape(5, 7)
    # metrics
    a = rng.standard_normal(256).astype(np.float32)
    b = (a + rng.standard_normal(256).astype(np.float32) * 1e-3).astype(np.float32)
    b[5] = 0.0
    out["metrics/a"], out["metrics/b"] = a, b
    out["metrics/values"] = np.array([R.ref_maxdiff(p(a), p(b), 16), R.ref_avgrelerr(p(a), p(b), 16),
                                      R.ref_rmse(p(a), p(b), 16)], np.float64)
    # HCSRMatrix(matrix, threshold) (formats/HCSRMatrix.cpp:10-36) on square
    # matrices whose 16x16 blocks have mixed densities: a random-pattern matrix
    # (element density 0.7) with every third block row thinned to 25 %
    R.ref_hcsr.restype = ctypes.c_int
    R.ref_hcsr.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_float] + [ctypes.c_void_p] * 8
    def gen(r, c, sp, pat, bs, seed):
        m = np.empty((r, c), np.float32)
        assert R.ref_generate_matrix(r, c, sp, pat.encode(), bs, seed, p(m)) == 0
        return m

    dense = gen(128, 128, 0.3, "random", 16, 11)
    thin = gen(128, 128, 0.75, "random", 16, 12)
    mixed = dense.copy()
    for br in range(0, 8, 3):
        mixed[br * 16:(br + 1) * 16] = thin[br * 16:(br + 1) * 16]
    hb = to_half(mixed)
    out["hcsr/A"] = hb
    for th in (0.0, 0.2, 0.5, 0.65, 0.8, 1.1):
        nnzb, nnz = ctypes.c_longlong(), ctypes.c_longlong()
        R.ref_hcsr(p(hb), 128, 128, th, ctypes.byref(nnzb), ctypes.byref(nnz), *([None] * 6))
        bh = np.zeros(9, np.int32)
        bi = np.zeros(max(nnzb.value, 1), np.int32)
        bd = np.zeros(max(nnzb.value * 256, 1), np.uint16)
        ch = np.zeros(129, np.int32)
        cx = np.zeros(max(nnz.value, 1), np.int32)
        cd = np.zeros(max(nnz.value, 1), np.uint16)
        R.ref_hcsr(p(hb), 128, 128, th, ctypes.byref(nnzb), ctypes.byref(nnz), p(bh), p(bi), p(bd), p(ch), p(cx),
                   p(cd))
        key = "hcsr/%g" % th
        out[key + "/bhdr"], out[key + "/bidx"], out[key + "/bdata"] = bh, bi[:nnzb.value], bd[:nnzb.value * 256]
        out[key + "/chdr"], out[key + "/cidx"], out[key + "/cdata"] = ch, cx[:nnz.value], cd[:nnz.value]
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_golden.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst, os.path.getsize(dst), "bytes,", len(out), "arrays")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else oracle.reference_tree())
