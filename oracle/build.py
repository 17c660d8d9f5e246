"""Build recipe for the oracle (test infrastructure only).

Compiles oracle/newman_oracle.cpp into oracle/_build/libnewman_oracle.so with
g++, linked against the runtime GMP library (libgmp.so.10).  The product never
loads this library.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libnewman_oracle.so")
SRC = os.path.join(HERE, "newman_oracle.cpp")
GMP_INC = os.path.join(ROOT, "newman_gb300", "csrc")


def build(force=False, verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    deps = [SRC, os.path.join(GMP_INC, "gmp_abi.h")]
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps)):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-pthread",
           "-I", GMP_INC, SRC, "-o", tmp, "-l:libgmp.so.10"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
