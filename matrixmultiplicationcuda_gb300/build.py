"""Builds libbcsr_spmm.so (all CUDA and host sources) for sm_103a, in-tree.

Each translation unit is compiled by its own nvcc process in parallel, then
linked into matrixmultiplicationcuda_gb300/lib/libbcsr_spmm.so. Nothing is
installed outside the package directory.
"""
import os
import platform
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "lib")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libbcsr_spmm.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")
COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + os.path.join(ROOT, "include")]


def sources():
    out = []
    for d in (CSRC, os.path.join(CSRC, "host")):
        for f in sorted(os.listdir(d)):
            if f.endswith((".cu", ".cpp")):
                out.append(os.path.join(d, f))
    return out


def _compile(src, verbose=False):
    obj = os.path.join(OBJ, os.path.relpath(src, CSRC).replace(os.sep, "_") + ".o")
    deps = [src] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    deps += [os.path.join(ROOT, "include", h) for h in os.listdir(os.path.join(ROOT, "include"))]
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj, ""
    cmd = [NVCC] + ARCH + COMMON + ["-x", "cu", "-c", src, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    return obj, r.stdout + r.stderr


def _arch_guard():
    """Objects and the library built on another host architecture are discarded."""
    stamp = os.path.join(OBJ, "ARCH")
    arch = platform.machine()
    if os.path.exists(stamp) and open(stamp).read().strip() == arch:
        return
    for d in (OBJ, OUT):
        if os.path.isdir(d):
            for f in os.listdir(d):
                if f.endswith((".o", ".so", ".tmp")):
                    os.remove(os.path.join(d, f))
    with open(stamp, "w") as f:
        f.write(arch)


def build(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    os.makedirs(OBJ, exist_ok=True)
    _arch_guard()
    srcs = sources()
    with ThreadPoolExecutor(max_workers=max(2, min(len(srcs), os.cpu_count() or 4))) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), srcs))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            if log:
                sys.stderr.write(log)
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(o) for o in objs):
        return LIB
    cmd = [NVCC] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(LIB + ".tmp", LIB)
    return LIB


HARNESS = os.path.join(HERE, "harness")


def build_tools(verbose=False):
    """The harness executables (lib/<name>), linked against the library."""
    build(verbose)
    out = []
    for f in sorted(os.listdir(HARNESS)):
        if not f.endswith(".cu"):
            continue
        src = os.path.join(HARNESS, f)
        exe = os.path.join(OUT, f[:-3])
        deps = [src, LIB] + [os.path.join(ROOT, "include", h) for h in os.listdir(os.path.join(ROOT, "include"))]
        deps += [os.path.join(HARNESS, h) for h in os.listdir(HARNESS) if h.endswith((".cuh", ".h"))]
        if not (os.path.exists(exe) and os.path.getmtime(exe) >= max(os.path.getmtime(d) for d in deps)):
            cmd = [NVCC] + ARCH + ["-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"), src, "-o", exe + ".tmp",
                                   "-L" + OUT, "-lbcsr_spmm", "-lcublas", "-Xlinker", "-rpath", "-Xlinker", "$ORIGIN"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
            os.replace(exe + ".tmp", exe)
        out.append(exe)
    return out


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
