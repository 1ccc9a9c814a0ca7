"""Builds libnumrs_gb300.so in-tree from numrs_gb300/csrc/*.cu with nvcc.

Every translation unit is compiled for sm_103a only
(-gencode arch=compute_103a,code=sm_103a), in parallel, then linked into one
shared library next to this file. No cmake, no torch extension machinery:
the library's ABI is plain C (include/numrs_gpu.h).
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libnumrs_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xptxas", "-O3", "-DNDEBUG"]


def nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def source_hash() -> str:
    """16 hex digits of SHA-256 over the CUDA sources and the ABI header: the
    build identity that keys saved tuner tables and selector weights."""
    import hashlib
    hsh = hashlib.sha256()
    for p in sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cuh"))) + [
            os.path.join(HERE, "..", "include", "numrs_gpu.h")]:
        hsh.update(os.path.basename(p).encode())
        hsh.update(open(p, "rb").read())
    return hsh.hexdigest()[:16]


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    deps = [src] + glob.glob(os.path.join(CSRC, "*.cuh")) + [
        os.path.join(HERE, "..", "include", "numrs_gpu.h")]
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", src, "-o", obj + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    os.replace(obj + ".tmp", obj)
    return obj


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    """Compile (incrementally) and link the library; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    if force:
        for o in glob.glob(os.path.join(BUILD, "*.o")):
            os.remove(o)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    # tuner.cu carries the build identity; recompile it whenever it changes
    sh = source_hash()
    mark = os.path.join(BUILD, "source_hash.txt")
    tuner_obj = os.path.join(BUILD, "tuner.cu.o")
    if not os.path.exists(mark) or open(mark).read().strip() != sh:
        if os.path.exists(tuner_obj):
            os.remove(tuner_obj)
        with open(mark, "w") as f:
            f.write(sh + "\n")

    def flags(src):
        return extra + ([f'-DNRS_SOURCE_HASH="{sh}"'] if os.path.basename(src) == "tuner.cu" else [])
    workers = min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(workers) as ex:
        objs = list(ex.map(lambda s: _compile(s, flags(s)), srcs))
    if os.path.exists(LIB) and not force and os.path.getmtime(LIB) >= max(os.path.getmtime(o) for o in objs):
        return LIB
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-ldl", "-lrt", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
