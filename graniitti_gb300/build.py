"""In-tree build of the CUDA library graniitti_gb300/_build/libgrn.so (sm_103a).

The translation units compiled in parallel by nvcc, linked as a shared library
with the CUDA runtime linked statically (nothing else to ship).
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libgrn.so")
SOURCES = ["grn_kernels.cu", "grn_kernels_wide.cu", "grn_kernels_wide_f32.cu",
           "grn_kernels_wide_f64.cu", "grn_api.cu", "grn_noalloc.cu", "grn_flow.cu",
           "grn_flow_wide.cu", "grn_record.cc"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _flags(extra=()):
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-I" + os.path.join(REPO, "include"), "-I" + CSRC] + list(extra)


def build_library(verbose=False, extra=(), force=False):
    os.makedirs(OUT, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    deps = srcs + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")] + \
        [os.path.join(REPO, "include", "graniitti_gb300.h")]
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in deps):
            return LIB
    objs = [os.path.join(OUT, os.path.splitext(os.path.basename(s))[0] + ".o") for s in srcs]

    def compile_one(pair):
        src, obj = pair
        # grn_kernels.cu launches the >8-dimensional instantiations of its kernel templates that
        # the grn_kernels_wide*.cu units define (explicit instantiation declarations and
        # definitions, each instantiation in exactly one unit): their host stubs need external
        # linkage across those units
        own = ["-static-global-template-stub=false"] if os.path.basename(src).startswith(
            "grn_kernels") else []
        cmd = [nvcc()] + _flags(extra) + own + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s" % (src, r.stderr))
        return r.stderr

    with ThreadPoolExecutor(len(srcs)) as ex:
        logs = list(ex.map(compile_one, zip(srcs, objs)))
    if verbose:
        for l in logs:
            if l.strip():
                print(l)
    cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-cudart", "static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s" % r.stderr)
    return LIB


if __name__ == "__main__":
    v = "-v" in sys.argv
    ex = ["-Xptxas", "-v"] if "--ptxas" in sys.argv else []
    print(build_library(verbose=v, extra=ex, force=True))
