"""Build libnbg.so (CUDA, sm_103a) in-tree with nvcc.

Each translation unit under csrc/ is compiled in parallel for
compute_103a/sm_103a and linked into nbodysimulator.jl_gb300/libnbg.so.
--debug builds libnbg_debug.so instead (-DNBG_DEBUG: every neighbour and cell
index a kernel reads from a device table is checked before use; loaded when
NBG_DEBUG=1 is set).
Usage: python nbodysimulator.jl_gb300/build.py [--force] [--debug]
"""
import concurrent.futures
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libnbg.so")
BUILD_DEBUG = os.path.join(HERE, "_build_debug")
LIB_DEBUG = os.path.join(HERE, "libnbg_debug.so")
INCLUDE = os.path.join(HERE, "..", "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
              "--expt-relaxed-constexpr", "-I", INCLUDE]


def _nvcc():
    for cand in ("/usr/local/cuda/bin/nvcc", "nvcc"):
        if os.path.sep not in cand or os.path.exists(cand):
            return cand
    return "nvcc"


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps():
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hdrs.append(os.path.join(INCLUDE, "nbg.h"))
    return max(os.path.getmtime(h) for h in hdrs)


def _compile(src, extra, bdir=BUILD):
    obj = os.path.join(bdir, os.path.basename(src) + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), _deps()):
        return obj
    cmd = [_nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", src, "-o", obj + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    os.replace(obj + ".tmp", obj)
    return obj


def build(force=False, verbose_ptxas=False, debug=False):
    bdir, lib = (BUILD_DEBUG, LIB_DEBUG) if debug else (BUILD, LIB)
    os.makedirs(bdir, exist_ok=True)
    srcs = sources()
    if force:
        for f in os.listdir(bdir):
            os.remove(os.path.join(bdir, f))
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    if debug:
        extra.append("-DNBG_DEBUG")
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra, bdir), srcs))
    if (not force and os.path.exists(lib)
            and os.path.getmtime(lib) >= max(os.path.getmtime(o) for o in objs)):
        return lib
    cmd = [_nvcc(), *ARCH, "-shared", "-o", lib + ".tmp", *objs, "-lcudart", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(lib + ".tmp", lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv, debug="--debug" in sys.argv))
