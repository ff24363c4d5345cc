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
REFERENCE = os.environ.get("GC_REFERENCE_DIR", "/root/reference")


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


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_reference(force=True))
