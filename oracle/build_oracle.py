"""Builds the oracle's C restatement (test infrastructure) twice from one source:

* ``oracle/_build/libsph_port.so`` with ``-DREAL=float``: the reference's FP32
  arithmetic, the timed CPU baseline and a mid-size cross-check;
* ``oracle/_build/libsph_port64.so`` with ``-DREAL=double``: every per-particle
  sum, pair term and reduction in FP64 over the FP32 particle arrays -- the FP64
  oracle for one-step checks at the benchmark sizes, where the numpy oracle is
  too slow.

``gcc -O3 -fopenmp -shared -fPIC`` on ``oracle/sph_port.c`` alone -- no
architecture flags, so the same recipe builds on x86-64 and aarch64 hosts.  The
reference itself (Python + Taichi) has no compiled part to build.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "sph_port.c")
OUTS = {"float": os.path.join(HERE, "_build", "libsph_port.so"),
        "double": os.path.join(HERE, "_build", "libsph_port64.so")}
OUT = OUTS["float"]
INC = os.path.join(os.path.dirname(HERE), "include")


def build(verbose=False, real="float"):
    """Builds both variants (if stale) and returns the path of the `real` one."""
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    hdr = os.path.join(INC, "tichi_sph.h")
    newest = max(os.path.getmtime(SRC), os.path.getmtime(hdr), os.path.getmtime(os.path.abspath(__file__)))
    for r, out in OUTS.items():
        if os.path.exists(out) and os.path.getmtime(out) >= newest:
            continue
        cmd = ["gcc", "-O3", "-fopenmp", "-shared", "-fPIC", "-std=c11", "-DREAL=" + r, "-I", INC, SRC, "-o", out,
               "-lm"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
    return OUTS[real]


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
