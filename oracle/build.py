"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/flub_oracle.c into oracle/_build/libflub_oracle.so with gcc,
OpenMP and no floating-point contraction, so that the FP32 variant performs the
same sequence of IEEE operations as the CUDA kernels.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libflub_oracle.so")
SOURCES = [os.path.join(HERE, "flub_oracle.c"), os.path.join(HERE, "oracle_impl.h")]


def needs_build() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(s) > t for s in SOURCES)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not needs_build():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-std=c11", os.path.join(HERE, "flub_oracle.c"), "-o", tmp, "-lm"]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
