"""In-tree build of the CUDA library (sm_103a) and of the CPU oracle.

The CUDA translation units are compiled in parallel with nvcc and linked into
amressif_gb300/libamressif_gb300.so; kernels_exact.cu is compiled with
-fmad=false so that its kernels round every operation separately, in the
reference's order. The same units compiled with -DNS_BOUNDS_CHECK make the
bounds-check build libamressif_gb300_check.so (bounds.cuh), a debugging
library that the tests load beside the normal one.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libamressif_gb300.so")
LIB_CHECK = os.path.join(PKG, "libamressif_gb300_check.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-warn-spills"]

# translation unit -> extra flags
UNITS = {
    "kernels_exact.cu": ["-fmad=false"],
    "kernels_fast.cu": [],
    "kernels_mixed.cu": [],
    "kernels_adjoint.cu": [],
    "ns_api.cu": [],
    "adjoint_api.cu": [],
    "kernels3d.cu": [],
    "ns3d_api.cu": [],
    "adjoint3d_api.cu": [],
    "noalloc.cu": ["-fmad=false"],
}


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), p.stdout))
    return p.stdout


def build_cuda(verbose=False, checked=False):
    """The library; checked=True: the bounds-check build."""
    out_dir = os.path.join(BUILD, "check") if checked else BUILD
    os.makedirs(out_dir, exist_ok=True)
    nvcc = _nvcc()
    units = [u for u in UNITS if os.path.exists(os.path.join(CSRC, u))]
    extra = ["-DNS_BOUNDS_CHECK"] if checked else []

    def one(u):
        obj = os.path.join(out_dir, u.replace(".cu", ".o"))
        cmd = [nvcc] + ARCH + NVCC_FLAGS + extra + UNITS[u] + ["-c", os.path.join(CSRC, u), "-o", obj]
        out = _run(cmd)
        if verbose and out.strip():
            sys.stdout.write(out)
        return obj

    with ThreadPoolExecutor(max_workers=len(units)) as ex:
        objs = list(ex.map(one, units))
    lib = LIB_CHECK if checked else LIB
    _run([nvcc] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart"])
    return lib


def build_oracle():
    src = os.path.join(ROOT, "oracle", "ns_oracle.cpp")
    out_dir = os.path.join(ROOT, "oracle", "_build")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "libns_oracle.so")
    _run(["g++", "-std=c++17", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-o", out, src])
    return out


def build(verbose=False):
    with ThreadPoolExecutor(max_workers=3) as ex:
        a = ex.submit(build_cuda, verbose)
        c = ex.submit(build_cuda, verbose, True)
        b = ex.submit(build_oracle)
        return a.result(), c.result(), b.result()


if __name__ == "__main__":
    print(build(verbose=True))
