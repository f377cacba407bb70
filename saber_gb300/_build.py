"""In-tree build of libsaber_gb300.so (nvcc, sm_103a) and of the test oracle."""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libsaber_gb300.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
SOURCES = ["saber_gpu.cu", "band_kernels.cu", "probe.cu", "noalloc.cu", "traceback.cu", "scan.cu", "triage.cu", "tantan.cu", "translate.cu", "engine.cpp"]
# host C++ of the search engine and of the tantan model tables: f64 arithmetic must round like the
# reference's (no fused multiply-add)
HOST_FLAGS = {"engine.cpp": ["-Xcompiler", "-ffp-contract=off"], "tantan.cu": ["-Xcompiler", "-ffp-contract=off"]}


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def build_library(verbose=False):
    """Compile every CUDA translation unit in parallel and link the shared library."""
    os.makedirs(os.path.join(LIBDIR, "obj"), exist_ok=True)
    nvcc = _nvcc()
    common = [ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
              "-I" + os.path.join(REPO, "include"), "-I" + CSRC]

    def compile_one(src):
        obj = os.path.join(LIBDIR, "obj", os.path.splitext(src)[0] + ".o")
        cmd = [nvcc] + common + HOST_FLAGS.get(src, []) + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
        if verbose:
            sys.stderr.write(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc, ARCH, "-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


def build_oracle():
    """Build the CPU oracle (test infrastructure) with its Makefile."""
    subprocess.check_call(["make", "-s", "-C", os.path.join(REPO, "oracle"), "all"])
    return os.path.join(REPO, "oracle", "_build", "liboracle.so")


if __name__ == "__main__":
    print(build_library(verbose="-v" in sys.argv))
    print(build_oracle())
