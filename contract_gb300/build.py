"""Build libcontract.so (the C ABI plus every CUDA kernel) for sm_103a.

Each translation unit is compiled by nvcc in parallel, then linked into
``contract_gb300/lib/libcontract.so``.  No cmake, no torch extension machinery:
the library is a plain C-ABI shared object that any host language can load.

    python -m contract_gb300.build [--force] [-j N]
"""
import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libcontract.so")
OBJDIR = os.path.join(PKG, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = [
    "abi.cpp",
    "kernels_common.cu",
    "kernels_meson.cu",
    "kernels_baryon.cu",
    "kernels_fused.cu",
    "kernels_field.cu",
    "kernels_momentum.cu",
    "kernels_momentum_tc.cu",
    "kernels_momentum_fused.cu",
    "kernels_batch.cu",
    "noalloc.cu",
    "kernels_quda.cu",
]


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libcontract.so")
    return path


def _flags():
    return ARCH + ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
                   "-Xcompiler", "-fvisibility=hidden", "-I", INCLUDE, "-I", CSRC]


def _deps_mtime():
    paths = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    return max(os.path.getmtime(p) for p in paths)


def _compile(src):
    obj = os.path.join(OBJDIR, os.path.splitext(src)[0] + ".o")
    lang = ["-x", "cu"]
    cmd = [nvcc()] + lang + _flags() + ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force=False, jobs=None, verbose=False):
    """Compile and link libcontract.so unless it is newer than every source."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps_mtime():
        return LIB
    os.makedirs(OBJDIR, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    jobs = jobs or min(len(SOURCES), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(_compile, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-j", type=int, default=None)
    a = ap.parse_args(argv)
    build(force=a.force, jobs=a.j, verbose=True)


if __name__ == "__main__":
    sys.exit(main())
