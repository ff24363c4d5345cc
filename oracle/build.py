"""Build recipes for the oracle (test infrastructure only).

build_oracle():    compiles gc_oracle.c -> oracle/libgcoracle.so with gcc
                   (-ffp-contract=off: float operations rounded one by one,
                   like the CUDA kernels built with -fmad=false).
build_reference(): compiles the reference's own CPU sources where they lie
                   (the bricker, metadata writer and the level-geometry helper)
                   together with oracle/ref_driver.cpp into oracle/_ref/refdriver.
                   Only possible where the reference checkout exists.
"""
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB = os.path.join(HERE, "libgcoracle.so")
REF_OUT = os.path.join(HERE, "_ref")
REF_BIN = os.path.join(REF_OUT, "refdriver")
# the reference checkout: GC_REFERENCE_DIR, else a directory named "reference"
# beside this repository
REFERENCE = os.environ.get("GC_REFERENCE_DIR", os.path.join(os.path.dirname(ROOT), "reference"))


def build_oracle(force=False):
    src = os.path.join(HERE, "gc_oracle.c")
    hdr = [os.path.join(HERE, "gc_oracle.h"), os.path.join(ROOT, "include", "gc_gb300.h")]
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(p) for p in [src] + hdr)):
        return LIB
    cmd = ["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
           "-I", os.path.join(ROOT, "include"), src, "-o", LIB, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


# Reference sources compiled unchanged (paths inside the reference checkout).
REF_CPP = [
    "GcCore/src/libPreprocessor/Bricker_v2.cpp",
    "GcCore/src/libData/BricksManager.cpp",
    "GcCore/src/libData/Brick.cpp",
    "GcCore/src/libData/BrickKey.cpp",
    "GcCore/src/libData/MetaData.cpp",
    "GcCore/src/libData/Configuration.cpp",
    "GcCore/src/libData/ConfigurationPolicies.cpp",
    "GcCore/src/libData/VolumeConfiguration.cpp",
    "GcCore/src/libData/FilesManager.cpp",
    "GcCore/src/libData/FileFactory.cpp",
    "GcCore/src/libData/AbstractFile.cpp",
    "GcCore/src/libData/RAWFile.cpp",
    "GcCore/src/libData/GISFile.cpp",
    "GcCore/src/libData/GISStackFile.cpp",
    "GcCore/src/libCommon/FileSystem.cpp",
    "GcCore/src/libCommon/Logger.cpp",
    "GcCore/src/libCommon/LogWriter.cpp",
    "GcCore/src/libCommon/LogCategory.cpp",
    "GcCore/src/libCommon/LogMessage.cpp",
    "GcCore/src/libCommon/LoggerFormatterFileStd.cpp",
    "GcCore/src/libTinyXml/tinyxml2.cpp",
]


def reference_available():
    return os.path.isdir(os.path.join(REFERENCE, "GcCore"))


def build_reference(force=False):
    """Compile the reference's CPU preprocessing code + our driver.  Returns the
    driver path, or None when the reference checkout or a dependency is absent."""
    if not reference_available():
        return None
    driver = os.path.join(HERE, "ref_driver.cpp")
    if not force and os.path.exists(REF_BIN) and os.path.getmtime(REF_BIN) >= os.path.getmtime(driver):
        return REF_BIN
    os.makedirs(REF_OUT, exist_ok=True)
    lz4 = None
    for cand in ("/usr/lib/x86_64-linux-gnu/liblz4.so.1", "/usr/lib/aarch64-linux-gnu/liblz4.so.1",
                 "/usr/lib64/liblz4.so.1"):
        if os.path.exists(cand):
            lz4 = cand
            break
    if lz4 is None:
        return None
    inc = ["-I", os.path.join(REFERENCE, "GcCore/include"),
           "-I", os.path.join(REFERENCE, "GcCore/dependencies/lz4-1.8.1/include")]
    defs = ["-DTDNS_LINUX", "-DTDNS_RELEASE", "-DTDNS_STATIC", "-DNDEBUG"]
    srcs = [os.path.join(REFERENCE, p) for p in REF_CPP] + [driver]
    cmd = [shutil.which("g++") or "g++", "-O1", "-std=c++17", "-w"] + defs + inc + srcs + [
        "-o", REF_BIN, lz4, "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference build failed:\n{r.stderr[-4000:]}")
    return REF_BIN


# ---------------------------------------------------------------------------
# The reference's own GPU code -- the mipmapper (Mipmapper.cu), the GPU cache
# (CacheManager.hpp + CacheManagerKernels.cu + RequestHandler.hpp) and the ray
# caster (RayCasters.cu) -- run headless on the GPU by oracle/ref_gpu_driver.cu.
# The GPU machine has no reference checkout, so stage_reference_gpu() copies the
# files it needs, unchanged, into oracle/_ref/src/ (git-ignored: never part of
# the repository's history) where the reference checkout exists; whichever
# machine runs the tests then compiles them with its own nvcc and g++
# (build_reference_gpu) into oracle/_ref/librefgpu.so.
REF_GPU_SRC = os.path.join(REF_OUT, "src")
REF_GPU_MANIFEST = os.path.join(REF_GPU_SRC, "STAGED")
REF_GPU_LIB = os.path.join(REF_OUT, "librefgpu.so")
# (directory inside the reference, sub-directories left out)
REF_GPU_TREES = [
    ("GcCore/include", ("libNetwork", "libPython")),
    ("GcCore/api/glm-0.9.9.0/glm/glm", ("gtx",)),
    ("GcCore/dependencies/lz4-1.8.1/include", ()),
]
REF_GPU_CU = [
    "GcCore/src/cuda/libPreprocessor/Mipmapper.cu",
    "GcCore/src/cuda/libGPUCache/CacheManagerKernels.cu",
]
REF_GPU_FILES = REF_CPP + REF_GPU_CU + [
    "Applications/DVR-ray-caster/src/RayCasters.cu",
    "Applications/DVR-ray-caster/include/RayCasters_helpers.hpp",
    "Applications/DVR-ray-caster/include/helper_math.h",
]
REF_DEFS = ["-DTDNS_LINUX", "-DTDNS_RELEASE", "-DTDNS_STATIC", "-DNDEBUG"]
GPU_ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def stage_reference_gpu():
    """Copy the reference files the GPU harness compiles into oracle/_ref/src/.
    Returns the staging directory, or None where the reference checkout is
    absent (the GPU machine: it uses the copy made here)."""
    if not reference_available():
        return None
    for rel, skip in REF_GPU_TREES:
        src_root = os.path.join(REFERENCE, rel)
        for d, dirs, files in os.walk(src_root):
            dirs[:] = [x for x in dirs if os.path.relpath(os.path.join(d, x), src_root).split(os.sep)[0] not in skip]
            for f in files:
                s = os.path.join(d, f)
                t = os.path.join(REF_GPU_SRC, os.path.relpath(s, REFERENCE))
                if not os.path.exists(t) or os.path.getmtime(t) < os.path.getmtime(s):
                    os.makedirs(os.path.dirname(t), exist_ok=True)
                    shutil.copy2(s, t)
    for rel in REF_GPU_FILES:
        s, t = os.path.join(REFERENCE, rel), os.path.join(REF_GPU_SRC, rel)
        if not os.path.exists(t) or os.path.getmtime(t) < os.path.getmtime(s):
            os.makedirs(os.path.dirname(t), exist_ok=True)
            shutil.copy2(s, t)
    with open(REF_GPU_MANIFEST, "w") as f:
        f.write("\n".join(REF_GPU_FILES) + "\n")
    return REF_GPU_SRC


def reference_gpu_staged():
    return os.path.exists(REF_GPU_MANIFEST)


def _find_lz4():
    for cand in ("/usr/lib/x86_64-linux-gnu/liblz4.so.1", "/usr/lib/aarch64-linux-gnu/liblz4.so.1",
                 "/usr/lib64/liblz4.so.1", "/usr/lib/liblz4.so.1"):
        if os.path.exists(cand):
            return cand
    return None


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def build_reference_gpu(force=False, verbose=False):
    """Compile the staged reference GPU code with oracle/ref_gpu_driver.cu into
    oracle/_ref/librefgpu.so for sm_103a.  Returns its path, or None when no
    staged copy exists.  Objects go to oracle/_ref/obj-<machine>/ so that the
    x86-64 and aarch64 builds never mix."""
    import concurrent.futures as cf
    import platform

    if not reference_gpu_staged():
        return None
    lz4 = _find_lz4()
    if lz4 is None:
        raise RuntimeError("liblz4.so.1 (the reference's brick codec) not found")
    obj_dir = os.path.join(REF_OUT, "obj-" + platform.machine())
    os.makedirs(obj_dir, exist_ok=True)
    driver = os.path.join(HERE, "ref_gpu_driver.cu")
    stamp = os.path.join(obj_dir, "librefgpu.stamp")
    inc = ["-I", os.path.join(REF_GPU_SRC, "GcCore/include"),
           "-I", os.path.join(REF_GPU_SRC, "GcCore/dependencies/lz4-1.8.1/include"),
           "-I", os.path.join(REF_GPU_SRC, "GcCore/api/glm-0.9.9.0/glm"),
           "-I", os.path.join(REF_GPU_SRC, "Applications/DVR-ray-caster/include"),
           "-I", os.path.join(REF_GPU_SRC, "Applications/DVR-ray-caster/src")]
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(_nvcc())), "include")
    jobs = []
    for rel in REF_CPP:
        jobs.append((os.path.join(REF_GPU_SRC, rel),
                     [shutil.which("g++") or "g++", "-O2", "-std=c++17", "-fPIC", "-w", "-I", cuda_inc] + REF_DEFS + inc))
    nv = [_nvcc()] + GPU_ARCH + ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-w", "-Xcudafe", "--diag_suppress=esa_on_defaulted_function_ignored"] + REF_DEFS + inc
    for rel in REF_GPU_CU:
        jobs.append((os.path.join(REF_GPU_SRC, rel), nv))
    jobs.append((driver, nv))

    def compile_one(job):
        src, cmd = job
        obj = os.path.join(obj_dir, os.path.basename(src) + ".o")
        if not force and os.path.exists(obj) and os.path.getmtime(obj) >= os.path.getmtime(src):
            return obj, False
        full = cmd + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(full), flush=True)
        r = subprocess.run(full, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference GPU build failed for {src}:\n{r.stderr[-4000:]}")
        return obj, True

    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        results = list(ex.map(compile_one, jobs))
    objs = [o for o, _ in results]
    if (force or any(r for _, r in results) or not os.path.exists(REF_GPU_LIB) or not os.path.exists(stamp)
            or os.path.getmtime(REF_GPU_LIB) < max(os.path.getmtime(o) for o in objs)):
        cmd = [_nvcc()] + GPU_ARCH + ["-shared", "-o", REF_GPU_LIB] + objs + ["-Xlinker", lz4, "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference GPU link failed:\n{r.stderr[-4000:]}")
        with open(stamp, "w") as f:
            f.write(platform.machine() + "\n")
    return REF_GPU_LIB


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_reference(force=True))
    print(stage_reference_gpu())
    print(build_reference_gpu(verbose=True))
