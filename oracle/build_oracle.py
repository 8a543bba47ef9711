"""Builds the oracle's C restatement (test infrastructure): ``oracle/_build/libsph_port.so``.

``gcc -O3 -fopenmp -shared -fPIC`` on ``oracle/sph_port.c`` alone -- no
architecture flags, so the same recipe builds on x86-64 and aarch64 hosts.  The
reference itself (Python + Taichi) has no compiled part to build.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "sph_port.c")
OUT = os.path.join(HERE, "_build", "libsph_port.so")
INC = os.path.join(os.path.dirname(HERE), "include")


def build(verbose=False):
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    hdr = os.path.join(INC, "tichi_sph.h")
    if os.path.exists(OUT) and os.path.getmtime(OUT) >= max(os.path.getmtime(SRC), os.path.getmtime(hdr)):
        return OUT
    cmd = ["gcc", "-O3", "-fopenmp", "-shared", "-fPIC", "-std=c11", "-DREAL=float", "-I", INC, SRC, "-o", OUT, "-lm"]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.run(cmd, check=True)
    return OUT


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
