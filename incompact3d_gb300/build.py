"""Build libx3dgpu.so in-tree with nvcc for sm_103a (no cmake).

Each translation unit is compiled in its own nvcc process (in parallel), then
linked into incompact3d_gb300/_build/libx3dgpu.so.  Rebuilds only when a source
or header is newer than the library.
"""
import glob
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUTDIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUTDIR, "libx3dgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _deps():
    return (_sources() + glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) +
            [os.path.join(ROOT, "include", "x3d_gpu.h"), os.path.abspath(__file__)])


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(p) <= t for p in _deps())


# Host code (the coefficient tables, stretching metrics, plans) is compiled
# without FMA contraction so it rounds as the reference's formulas do on
# every host (aarch64 compilers contract a*b+c by default).
def _compile(src, extra):
    obj = os.path.join(OUTDIR, os.path.basename(src) + ".o")
    cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off",
           "-I", os.path.join(ROOT, "include"), "-I", CSRC, *extra, "-c", src, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [NVCC, "-x", "cu", *cmd[1:]]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return obj, r.stderr


def build(force=False, verbose=False, extra=()):
    """Compile every CUDA/C++ source of the library; return the .so path."""
    os.makedirs(OUTDIR, exist_ok=True)
    if not force and up_to_date():
        return LIB
    srcs = _sources()
    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, list(extra)), srcs))
    objs = [o for o, _ in results]
    if verbose:
        for _, err in results:
            if err.strip():
                print(err)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True,
                extra=("-Xptxas", "-v") if "--ptxas" in sys.argv else ()))
