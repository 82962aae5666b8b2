"""The NVBench-form benches and the C++ drop-in call sequence on the GPU.

* spmm_nvbench_benches registers the reference's benches (nvbench_main.cu:
  326-1449) on the NVBench surface of harness/nvbench_compat.cuh; every bench
  checks its own result against a host product at the reference harness's
  1e-2 absolute tolerance and exits non-zero on a mismatch. The tests run each
  registered bench on one small state and one bench over a small axis sweep.
* tests/cpp/dropin_sequence.cu is the reference's host call sequence (generate,
  Matrix, BCSRMatrix, copyToDevice, shaped launcher, copy back) written against
  include/bcsr_spmm.hpp; its BCSR arrays must equal the oracle's bit for bit and
  its product must match the restated reference host multiply within 1e-2.
* spmm_nvbench (the preset harness) runs its 1024^2 preset with its sampled
  FP64 check.
"""
import csv
import os
import subprocess

import numpy as np
import pytest

import matrixmultiplicationcuda_gb300 as m
from oracle import oracle

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.dirname(m.lib_path)
BENCHES = os.path.join(LIBDIR, "spmm_nvbench_benches")

NAMES = {16: ["sparseMatrixMulTensor", "sparseMatrixMulTensor_v2", "sparseMatrixMulTensor_v3",
              "sparseMatrixMulTensor_v1_improved", "sparseMatrixMulTensorAdaptive_16x16"],
         32: ["sparseMatrixMulTensor32x16", "sparseMatrixMulTensor32x16_v2", "sparseMatrixMulTensor32x16_shared",
              "sparseMatrixMulTensor32x16_shared_vectorized", "sparseMatrixMulTensor32x16_v2_shared_vectorized",
              "sparseMatrixMulTensorAdaptive_32x16"],
         64: ["sparseMatrixMulTensor64x16", "sparseMatrixMulTensor64x16_v2", "sparseMatrixMulTensorAdaptive_64x16"]}
PAT = {16: 4, 32: 6, 64: 5}      # blockrandom, pattern32by16, pattern64by16


def _rows(path):
    with open(path) as f:
        return list(csv.DictReader(f))


def test_every_registered_bench_runs_and_checks(tmp_path):
    args = [BENCHES]
    for bR, names in NAMES.items():
        for n in names:
            args += ["-b", n, "-a", "M=[512]", "-a", "K=[256]", "-a", "N=[64]", "-a", "SPARS=[80]",
                     "-a", "PAT=[%d]" % PAT[bR]]
    out = tmp_path / "all.csv"
    r = subprocess.run(args + ["--min-samples", "3", "--min-time", "0", "--csv", str(out)], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    rows = _rows(out)
    assert sorted(x["Benchmark"] for x in rows) == sorted(n for ns in NAMES.values() for n in ns)
    for x in rows:
        assert int(x["Samples"]) >= 3 and float(x["GPU Time (sec)"]) > 0, x


def test_axis_sweep_and_patterns(tmp_path):
    """One bench over the reference's pattern axis and two sizes (every pattern of
    the reference generator through the 16x16 launcher), with the checks on."""
    out = tmp_path / "sweep.csv"
    r = subprocess.run([BENCHES, "-b", "sparseMatrixMulTensor", "-a", "M=[512,1024]", "-a", "K=[256]", "-a",
                        "N=[32]", "-a", "SPARS=[60,90]", "-a", "PAT=[0:6:1]", "--min-samples", "2", "--min-time", "0",
                        "--csv", str(out), "--json", str(tmp_path / "sweep.json")],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    rows = _rows(out)
    assert len(rows) == 2 * 2 * 7
    assert "nv/cold/time/gpu/mean" in open(tmp_path / "sweep.json").read()
    # the markdown table shows the summaries the bench un-hid (min and max)
    assert "nv/cold/time/gpu/min" in r.stdout and "nv/cold/time/gpu/max" in r.stdout


@pytest.mark.parametrize("bR,pattern,sparsity", [(16, "blockrandom", 0.9), (32, "pattern32by16", 0.7),
                                                 (64, "pattern64by16", 0.8), (16, "diagonal", 0.0)])
def test_cpp_dropin_call_sequence(tmp_path, bR, pattern, sparsity):
    src = os.path.join(ROOT, "tests", "cpp", "dropin_sequence.cu")
    exe = tmp_path / "dropin"
    r = subprocess.run(["nvcc", "-std=c++17", "-O2", src, "-I", os.path.join(ROOT, "include"), "-L", LIBDIR,
                        "-lbcsr_spmm", "-Xlinker", "-rpath", "-Xlinker", LIBDIR, "-o", str(exe)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    M, K, N = 512, 384, 96
    prefix = str(tmp_path / "out")
    r = subprocess.run([str(exe), str(M), str(K), str(N), str(sparsity), pattern, str(bR), prefix],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    A = oracle.f32_to_f16(oracle.generate_matrix(M, K, sparsity, pattern, bR, 123))
    B = oracle.f32_to_f16(oracle.generate_matrix(K, N, 0.0, "random", bR, 456))
    hdr, idx, _ = oracle.bcsr(A, bR, 16)
    np.testing.assert_array_equal(np.fromfile(prefix + ".hdr", np.int32), hdr)
    np.testing.assert_array_equal(np.fromfile(prefix + ".idx", np.int32), idx)
    C = np.fromfile(prefix + ".c", np.float32).reshape(M, N)
    assert np.isfinite(C).all()
    assert float(np.max(np.abs(C - oracle.cpu_matmul_ref(A, B)))) <= 1e-2


def test_preset_harness_c1(tmp_path):
    exe = os.path.join(LIBDIR, "spmm_nvbench")
    out = tmp_path / "c1.json"
    r = subprocess.run([exe, "--preset", "c1", "--tuning", "default", "--min-samples", "5", "--min-time", "0.01",
                        "--json", str(out)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    import json
    states = json.load(open(out))["states"]
    assert states and all(s["M"] == 1024 and s["mean_us"] > 0 for s in states)
    # the harness's own sampled check against an FP64 host product (fp16 bar 2e-3)
    assert all(0 <= s["max_rel_err"] <= 2e-3 for s in states), states


def test_preset_floor_and_clean_flush(tmp_path):
    """The empty-kernel floor and C1 under the clean cold-L2 method (a second
    256 MB buffer read after the 256 MB write) run and pass the harness's check."""
    exe = os.path.join(LIBDIR, "spmm_nvbench")
    out = tmp_path / "clean.json"
    r = subprocess.run([exe, "--preset", "floor,c1", "--tuning", "default", "--flush", "clean", "--min-samples", "5",
                        "--min-time", "0.01", "--json", str(out)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert "empty, <<<1, 32>>>" in r.stdout and "second 256 MB buffer read" in r.stdout
    import json
    states = json.load(open(out))["states"]
    assert states and all(s["M"] == 1024 and 0 <= s["max_rel_err"] <= 2e-3 for s in states), states
