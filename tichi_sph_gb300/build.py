"""Builds the CUDA shared library ``_lib/libtichi_sph.so`` for sm_103a.

Each ``csrc/*.cu`` translation unit is compiled by its own nvcc process (in
parallel), then linked with ``nvcc -shared``.  Objects go to ``_build/`` next to
this file; a unit is recompiled when it or any header is newer than its object.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libtichi_sph.so")
SOURCES = ["grid.cu", "sweeps.cu", "fbm.cu", "api.cu", "noalloc.cu", "adjoint.cu", "wcsph.cu", "measure.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE]


def _nvcc():
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cand = os.path.join(cuda, "bin", "nvcc")
    return cand if os.path.exists(cand) else (shutil.which("nvcc") or "nvcc")


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(INCLUDE, "tichi_sph.h"))
    return max(os.path.getmtime(h) for h in hs)


def _compile(src, hdr_mtime, verbose):
    s = os.path.join(CSRC, src)
    o = os.path.join(BUILD, src.replace(".cu", ".o"))
    if os.path.exists(o) and os.path.getmtime(o) >= max(os.path.getmtime(s), hdr_mtime):
        return o, False
    cmd = [_nvcc()] + ARCH + FLAGS + ["-c", s, "-o", o]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    return o, True


def build(force=False, verbose=False):
    """Compiles (if needed) and returns the path of the shared library."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    sources = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    hdr = _headers()
    if force:
        for s in sources:
            o = os.path.join(BUILD, s.replace(".cu", ".o"))
            if os.path.exists(o):
                os.remove(o)
    with cf.ThreadPoolExecutor(max_workers=len(sources)) as ex:
        res = list(ex.map(lambda s: _compile(s, hdr, verbose), sources))
    objs = [o for o, _ in res]
    changed = any(c for _, c in res)
    if changed or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [_nvcc(), "-shared"] + ARCH + objs + ["-o", LIB]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc link failed:\n%s%s" % (r.stdout, r.stderr))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
