"""Builds libgcgb300.so (CUDA kernels + C++ host runtime + C ABI) for sm_103a.

Plain nvcc invocations, one per translation unit, run in parallel; a unit is
rebuilt when its source, a header of this package or include/gc_gb300.h is
newer than its object.  Objects go to _build/ beside this file; the shared
library lands next to this file so that it is loaded from the source tree.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgcgb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code is compiled without FMA contraction as well, so host-side float
# helpers give the same values on x86-64 and aarch64.
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "-I", INCLUDE, "-I", CSRC]
# Per-unit extra flags.  The ray caster is compiled without FMA contraction so
# that every float operation is a separately rounded IEEE operation in source
# order (the host oracle evaluates the same sequence).
EXTRA = {
    "render.cu": ["-fmad=false"],
    "render_fast.cu": ["-fmad=true"],  # the fast build of the same march (render_fast.cu includes render.cu)
}
SOURCES = ["config.cpp", "generate.cu", "preprocess.cu", "cache_kernels.cu", "cache_manager.cu", "render.cu",
           "render_fast.cu", "brickfiles.cpp"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers_mtime():
    paths = [os.path.join(INCLUDE, "gc_gb300.h")]
    paths += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return max(os.path.getmtime(p) for p in paths)


# units that include another unit's source
INCLUDES = {"render_fast.cu": ["render.cu"]}


def _compile(src, hdr_mtime, verbose):
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD, src + ".o")
    newest = max([os.path.getmtime(path), hdr_mtime] + [os.path.getmtime(os.path.join(CSRC, d))
                                                         for d in INCLUDES.get(src, [])])
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest:
        return obj, False
    cmd = [nvcc()] + ARCH + COMMON + EXTRA.get(src, [])
    if src.endswith(".cpp"):
        cmd += ["-x", "cu"]
    cmd += ["-c", path, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, True


def build(verbose=False, force=False):
    """Compile every unit (parallel) and link libgcgb300.so.  Returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    if force:
        for f in os.listdir(BUILD):
            os.remove(os.path.join(BUILD, f))
    hdr = _headers_mtime()
    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda s: _compile(s, hdr, verbose), SOURCES))
    objs = [o for o, _ in results]
    rebuilt = any(r for _, r in results)
    if rebuilt or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lpthread", "-ldl"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
