"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/matflat_oracle.cpp into oracle/_build/libmatflat_oracle.so with the flags the
arithmetic contract needs: -ffp-contract=off (MatFlat never fuses multiply-add; GCC on aarch64
would otherwise contract a*b+c into FMA) and no fast-math.  The reference itself is C# and has no
C/C++ sources, so there is no oracle/_ref build.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libmatflat_oracle.so")
SRC = os.path.join(HERE, "matflat_oracle.cpp")

FLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-pthread",
         "-ffp-contract=off", "-fno-fast-math", "-fno-unsafe-math-optimizations"]


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["g++"] + FLAGS + ["-o", LIB + ".tmp", SRC]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
