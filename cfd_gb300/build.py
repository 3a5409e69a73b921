"""Build recipe of the in-tree CUDA library cfd_gb300/_build/libcfd_gb300.so (sm_103a).

Each translation unit compiles in parallel (nvcc for .cu, g++ for .cpp) and nvcc links
the shared library.  The FP64 units use --fmad=false so that every double expression is
evaluated as written (no contraction), which is what makes the plain path reproduce the
CPU restatement bit for bit; host code likewise uses -ffp-contract=off.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libcfd_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# (source, extra flags)
UNITS = [
    ("kernels_fp64.cu", ["--fmad=false"]),
    ("kernels_pcg.cu", ["--fmad=false"]),
    ("kernels_mixed.cu", []),
    ("kernels_pcg_mixed.cu", []),
    ("context.cu", ["--fmad=false"]),
    ("abi.cu", ["--fmad=false"]),
    ("noalloc.cu", ["--fmad=false"]),
    ("kernels_mpnn.cu", []),
    ("mpnn.cu", []),
    ("smooth.cu", ["--fmad=false"]),
    ("host_prep.cpp", []),
]


def nvcc():
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _deps():
    files = [os.path.join(SRC, f) for f in os.listdir(SRC)]
    files.append(os.path.join(PKG, "..", "include", "cfd_gpu.h"))
    files.append(os.path.abspath(__file__))
    return files


def _compile(src, extra, verbose):
    path = os.path.join(SRC, src)
    obj = os.path.join(OUT, src + ".o")
    if src.endswith(".cu"):
        cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-c", path, "-o", obj,
               "-Xcompiler", "-fPIC,-ffp-contract=off", *extra]
        if verbose:
            cmd += ["-Xptxas", "-v"]
    else:
        cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall",
               "-I/usr/local/cuda/include", "-c", path, "-o", obj, *extra]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj, (r.stdout + r.stderr)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    if not force and os.path.exists(LIB):
        if os.path.getmtime(LIB) >= max(os.path.getmtime(p) for p in _deps()):
            return LIB
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        futs = [ex.submit(_compile, s, e, verbose) for s, e in UNITS]
        results = [f.result() for f in futs]
    if verbose:
        for _, log in results:
            if log.strip():
                print(log)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-Xcompiler", "-fPIC"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
