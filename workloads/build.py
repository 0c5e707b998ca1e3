"""Builds the host helper of the synthetic workloads (workloads/_build/libworkloads_synth.so).

Plain C, compiled for the machine it runs on (x86_64 here, aarch64 on the GPU host), with
-ffp-contract=off so that the Box-Muller arithmetic gives the same bytes on both.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libworkloads_synth.so")
SRC = os.path.join(HERE, "synth.c")


def build(force=False):
    os.makedirs(OUT, exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-pthread", "-ffp-contract=off",
                               "-o", LIB + ".tmp", SRC, "-lm"])
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
