"""Build the in-tree CUDA library bpm_gb300/libbpm_gb300.so for sm_103a.

    python -m bpm_gb300.build          # or: python bpm_gb300/build.py

Each .cu translation unit is compiled in parallel by nvcc (one -gencode, sm_103a), then
linked into one shared library with the CUDA runtime linked statically. Host code is
compiled with -ffp-contract=off so the FP32 mask recipes round exactly as written on
both x86-64 and aarch64.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libbpm_gb300.so")
BUILD = os.path.join(HERE, "_build")
SOURCES = ["capi.cu", "bpm_march.cu", "debye.cu", "spheres.cu"]

ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc():
    """The nvcc of CUDA_HOME (default /usr/local/cuda), else the one on PATH."""
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def flags():
    """nvcc flags of every translation unit: sm_103a only, line info for profiles, host
    code without FP contraction."""
    return [ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
            "-Xcompiler", "-ffp-contract=off", "-Xptxas", "-O3"]


def _compile(src):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *flags(), "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return obj


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "bpm_gb300.h"))
    return any(os.path.getmtime(p) > t for p in deps)


def build(force=False, verbose=True):
    """Compile the sources (in parallel) and link libbpm_gb300.so when a source or the
    header is newer than the library (always with force). Returns the library's path."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv)
