"""Host side of the library (no GPU): exports, generators, formats, .mat I/O,
argument checks, and the C++ drop-in classes."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

import matrixmultiplicationcuda_gb300 as m
from matrixmultiplicationcuda_gb300._lib import BcsrDesc, DenseDesc, Status
from oracle import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    names = set()
    for h in ("bcsr_spmm.h", "bcsr_spmm_host.h"):
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"^\s*(?:spmm_status|int|long long|void|const char\*)\s+(\w+)\s*\(", text,
                                re.M))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    names = header_functions()
    assert "spmm_bcsr_mm" in names and "sparseMatrixMulTensor_launch" in names
    assert "spmm_gen_values" in names and "spmm_mlp_param_count" in names
    L = ctypes.CDLL(m.lib_path)
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert m.lib().spmm_abi_version() == 1


@pytest.mark.parametrize("pattern", ["random", "checkerboard", "diagonal", "blockdiagonal",
                                     "blockrandom", "pattern64by16", "pattern32by16"])
def test_library_generator_matches_oracle(pattern):
    for (r, c, sp, bs, seed) in [(64, 80, 0.6, 16, 123), (130, 70, 0.9, 32, 5)]:
        got = m.generate_matrix(r, c, sp, pattern, bs, seed)
        exp = oracle.generate_matrix(r, c, sp, pattern, bs, seed)
        assert np.array_equal(got.view(np.uint32), exp.view(np.uint32))


def test_library_generator_rejects_unknown_pattern():
    with pytest.raises(m.SpmmError):
        m.generate_matrix(16, 16, 0.5, "spiral", 16, 1)


def test_host_bcsr_matches_golden_and_oracle(golden):
    for key in sorted({k.rsplit("/", 1)[0] for k in golden.files if k.startswith("bcsr/") and k.endswith("/hdr")}):
        A = golden[key + "/A"]
        bR, bC = (16, 16) if key.endswith("special") else (int(x) for x in key.split("/")[-1].split("_")[2:4])
        hdr, idx, data = m.host_dense_to_bcsr(A, bR, bC)
        assert np.array_equal(hdr, golden[key + "/hdr"])
        assert np.array_equal(idx, golden[key + "/idx"])
        assert np.array_equal(data, golden[key + "/data"])
    with pytest.raises(m.SpmmError):
        m.host_dense_to_bcsr(np.zeros((32, 32), np.uint16), 8, 16)


def test_host_csr_uses_column_index():
    A = np.zeros((3, 5), np.float16)
    A[0, 4] = 1
    A[2, 1] = 2
    A[2, 3] = -1
    hdr, idx, data = m.host_dense_to_csr(A.view(np.uint16))
    assert list(hdr) == [0, 1, 1, 3]
    assert list(idx) == [4, 1, 3]  # the reference writes i % rows here (formats/CSRMatrix.cu:32)
    assert list(data.view(np.float16)) == [1, 2, -1]


def test_mat_loader_matches_reference_fixture(golden, tmp_path):
    p = tmp_path / "a.mat"
    p.write_bytes(golden["mat/text"].tobytes())
    half, nz = m.mat_load(p)
    r, c, nz_ref = golden["mat/shape_nz"]
    assert half.shape == (r, c) and nz == nz_ref
    assert np.array_equal(half, golden["mat/half"])


def test_mat_roundtrip_and_errors(tmp_path):
    v = m.gen_dense(7, 9, m.DIST_UNIFORM, 4)
    v[2] = 0
    p = tmp_path / "x.mat"
    m.mat_save(p, v)
    half, nz = m.mat_load(p)
    assert np.array_equal(half, v.astype(np.float16).view(np.uint16))
    assert nz == int(np.count_nonzero(v))
    with pytest.raises(m.SpmmError):
        m.mat_load(tmp_path / "missing.mat")
    bad = tmp_path / "short.mat"
    bad.write_text("3 3\n1 2 3 4\n")
    with pytest.raises(m.SpmmError):
        m.mat_load(bad)


def test_generated_structures_are_valid():
    for pat, dens, param in [(m.PATTERN_RANDOM, 0.05, 0), (m.PATTERN_BAND, 0.01, 8),
                             (m.PATTERN_BLOCKDIAG, 0, 256), (m.PATTERN_LOGNORMAL, 0.05, 1.5)]:
        for bR in (16, 32, 64):
            rp, ci = m.gen_structure(2048, 2048, bR, pat, dens, param, seed=11)
            assert rp[0] == 0 and np.all(np.diff(rp) >= 0) and rp[-1] == len(ci)
            for i in range(len(rp) - 1):
                row = ci[rp[i]:rp[i + 1]]
                assert np.all(np.diff(row) > 0) and (len(row) == 0 or (row[0] >= 0 and row[-1] < 128))
    # block-diagonal 256 x 256 tiles: each 16-row block row sees exactly 16 block columns
    rp, ci = m.gen_structure(1024, 1024, 16, m.PATTERN_BLOCKDIAG, 0, 256, seed=1)
    assert np.all(np.diff(rp) == 16)
    # random density close to requested
    rp, ci = m.gen_structure(8192, 8192, 16, m.PATTERN_RANDOM, 0.05, 0, seed=3)
    assert abs(len(ci) / (512 * 512) - 0.05) < 0.002
    # log-normal row counts: mean ~ 5% of block columns, coefficient of variation ~ 1.5
    rp, ci = m.gen_structure(65536, 8192, 16, m.PATTERN_LOGNORMAL, 0.05, 1.5, seed=5)
    cnt = np.diff(rp)
    assert abs(cnt.mean() / 512 - 0.05) < 0.006
    assert 1.2 < cnt.std() / cnt.mean() < 1.7


def test_generated_values():
    v = m.gen_values(100, 64, 16, m.DIST_SCALED_NORMAL, seed=3).reshape(100, -1)
    mags = np.log10(np.abs(v).max(axis=1))
    assert mags.min() > -4 and mags.max() < 4.2 and mags.max() - mags.min() > 4
    u = m.gen_values(10, 16, 16, m.DIST_UNIFORM, seed=3)
    assert u.min() >= -1 and u.max() <= 1
    assert np.array_equal(u, m.gen_values(10, 16, 16, m.DIST_UNIFORM, seed=3))


def _call_mm(**kw):
    a = BcsrDesc()
    a.M, a.K, a.bR, a.bC = kw.get("M", 64), kw.get("K", 64), kw.get("bR", 16), kw.get("bC", 16)
    a.row_ptr = a.col_idx = a.vals = 16
    a.dtype = kw.get("dtype", 0)
    b = DenseDesc()
    b.data = 16
    b.scale = 1.0
    b.ldb = kw.get("ldb", 64)
    return m.lib().spmm_bcsr_mm(ctypes.byref(a), ctypes.byref(b), kw.get("N", 64),
                                ctypes.c_void_p(16), kw.get("ldc", 64), None, None)


def test_argument_checks_need_no_gpu():
    assert _call_mm(bR=8) == Status.UNSUPPORTED
    assert _call_mm(bC=32) == Status.UNSUPPORTED
    assert _call_mm(M=72) == Status.INVALID_ARG
    assert _call_mm(K=40) == Status.INVALID_ARG
    assert _call_mm(N=60, ldb=64, ldc=64) == Status.UNSUPPORTED
    assert _call_mm(ldb=32) == Status.MISALIGNED
    assert _call_mm(ldc=62) == Status.MISALIGNED
    assert _call_mm(dtype=2) == Status.INVALID_ARG      # E4M3 without scales
    assert _call_mm(dtype=3) == Status.INVALID_ARG      # split without low halves
    assert _call_mm(dtype=9) == Status.INVALID_ARG
    assert "multiple" in m._lib.last_error() or m._lib.last_error()
    assert m.lib().spmm_dense_to_bcsr_count(None, 32, 32, 32, 8, 16, None, None, None) == Status.INVALID_ARG


def test_cpp_dropin_classes(tmp_path):
    """A C++ program written against the reference's host classes compiles and runs."""
    src = tmp_path / "use.cpp"
    src.write_text(r'''
#include "bcsr_spmm.hpp"
#include <cstdio>
int main() {
  auto g = mg::generate_matrix<float>(128, 96, 0.6, "blockrandom", 16, 123);
  Matrix A(128, 96);
  for (int i = 0; i < 128; ++i) for (int j = 0; j < 96; ++j) A.data[i * 96 + j] = __float2half(g[i][j]);
  BCSRMatrix b(A, 32, 16);
  CSRMatrix c(A);
  HCSRMatrix h(A, 0.5f);
  std::printf("%d %d %d %d %d %d %d\n", b.blockRows, b.blockCols, b.hdr[b.blockRows], b.nonZeros, c.hdr[128],
              h.bcsr->hdr[h.bcsr->blockRows], h.csr->hdr[128]);
  try { BCSRMatrix bad(A, 8, 16); return 3; } catch (const std::invalid_argument&) {}
  return 0;
}
''')
    exe = tmp_path / "use"
    inc = os.path.join(ROOT, "include")
    libdir = os.path.dirname(m.lib_path)
    r = subprocess.run(["g++", "-std=c++17", str(src), "-I", inc, "-I/usr/local/cuda/include",
                        "-L", libdir, "-lbcsr_spmm", "-Wl,-rpath," + libdir, "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    br, bc, nnzb, nz, csr_nnz, h_nnzb, h_nnz = map(int, out.stdout.split())
    A = oracle.f32_to_f16(oracle.generate_matrix(128, 96, 0.6, "blockrandom", 16, 123))
    hdr, idx, data = oracle.bcsr(A, 32, 16)
    assert (br, bc, nnzb, nz) == (4, 6, len(idx), len(idx) * 512)
    assert csr_nnz == int(np.count_nonzero(A & 0x7fff))
    (_, hidx, _), (_, cidx, _) = oracle.hcsr(A.view(np.uint16).reshape(128, 96), 0.5)
    assert (h_nnzb, h_nnz) == (len(hidx), len(cidx))


def test_nvbench_benches_registered():
    """The NVBench-form benches list every reference bench name with its axes
    (no GPU needed to list them)."""
    exe = os.path.join(os.path.dirname(m.lib_path), "spmm_nvbench_benches")
    r = subprocess.run([exe, "--list"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    names = [line.split()[1] for line in r.stdout.splitlines()]
    for n in ("sparseMatrixMulTensor", "sparseMatrixMulTensor_v2", "sparseMatrixMulTensor32x16",
              "sparseMatrixMulTensor32x16_v2_shared_vectorized", "sparseMatrixMulTensor64x16",
              "sparseMatrixMulTensorAdaptive_16x16", "sparseMatrixMulTensorAdaptive_32x16"):
        assert n in names
    assert "PAT=[0,1,2,3,4,5,6]" in r.stdout and "SPARS=[60,70,80,90]" in r.stdout


def test_nvbench_benches_argument_errors():
    """The NVBench layer rejects an unknown bench, an unknown axis and a bad
    axis value before touching the GPU (exit status 2)."""
    exe = os.path.join(os.path.dirname(m.lib_path), "spmm_nvbench_benches")
    for args in (["-b", "noSuchBench"], ["-b", "sparseMatrixMulTensor", "-a", "Q=[1]"],
                 ["-b", "sparseMatrixMulTensor", "-a", "M"], ["--no-such-option"]):
        r = subprocess.run([exe] + args, capture_output=True, text=True, timeout=60)
        assert r.returncode == 2, (args, r.stdout, r.stderr)
    r = subprocess.run([exe, "--help"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "--axis" in r.stdout


def test_harness_built_and_prints_usage():
    exe = os.path.join(os.path.dirname(m.lib_path), "spmm_nvbench")
    assert os.path.exists(exe)
    r = subprocess.run([exe, "--help"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "--preset" in r.stderr and "--flush write|clean" in r.stderr
    # the cold-L2 method is checked before any device call
    r = subprocess.run([exe, "--flush", "sometimes"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "--flush takes write or clean" in r.stderr


@pytest.mark.parametrize("th", ["0", "0.2", "0.5", "0.65", "0.8", "1.1"])
def test_hcsr_matches_reference_golden(golden, th):
    """HCSRMatrix(matrix, threshold): the oracle restatement and the library's
    host class give the reference's own arrays for both parts."""
    A = golden["hcsr/A"]
    want = [golden["hcsr/%s/%s" % (th, k)] for k in ("bhdr", "bidx", "bdata", "chdr", "cidx", "cdata")]
    (ob, oc) = oracle.hcsr(A, float(th))
    (hb, hc) = m.host_dense_to_hcsr(A, float(th))
    for got in (list(ob) + list(oc), list(hb) + list(hc)):
        for g, w in zip(got, want):
            np.testing.assert_array_equal(g, w)


def test_hcsr_non_square_and_errors():
    A = oracle.f32_to_f16(oracle.generate_matrix(96, 160, 0.5, "random", 16, 3)).view(np.uint16).reshape(96, 160)
    (hb, hc) = m.host_dense_to_hcsr(A, 0.5)
    (ob, oc) = oracle.hcsr(A, 0.5)
    for g, w in zip(list(hb) + list(hc), list(ob) + list(oc)):
        np.testing.assert_array_equal(g, w)
    assert hc[1].max() < 160          # column indices, not the reference's i % rows
    with pytest.raises(m.SpmmError):
        m.host_dense_to_hcsr(np.zeros((40, 64), np.uint16), 0.5)
