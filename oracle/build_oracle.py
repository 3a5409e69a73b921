"""Build recipe of the oracle (test infrastructure: the CPU restatement of the
reference's FP64 step, see cfd_oracle.h).

    python oracle/build_oracle.py      ->  oracle/_build/libcfd_oracle.so

Compiled with -O2 -ffp-contract=off (no FMA contraction, no fast-math) so that every
double operation is the IEEE operation the source spells; -fopenmp gives the threaded
CPU baseline (the reference's OpenMP loops), one thread gives the serial order.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libcfd_oracle.so")


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "cfd_oracle.cpp")
    hdrs = [os.path.join(HERE, "cfd_oracle.h"),
            os.path.join(HERE, "..", "include", "cfd_gpu.h")]
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB):
        newest = max(os.path.getmtime(p) for p in [src] + hdrs)
        if os.path.getmtime(LIB) >= newest:
            return LIB
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
           "-fPIC", "-shared", "-Wall", "-Wno-unused-result", src, "-o", LIB + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
