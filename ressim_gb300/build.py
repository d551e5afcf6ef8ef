"""Builds libresgpu.so (the CUDA library behind include/rsg.h) in-tree.

Each translation unit is compiled for sm_103a in parallel, then linked.
Fused multiply-add contraction is disabled (--fmad=false for device code,
-ffp-contract=off for host code) so that every product and sum in the
property, MPFA and assembly code rounds as the Java reference evaluates it.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIB_DIR, "libresgpu.so")
SOURCES = ["context.cu", "csr.cu", "precond.cu", "amg.cu", "krylov.cu", "mesh.cu", "sim.cu", "noalloc.cu", "adjoint.cu",
           "ensemble.cu", "mmio.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr"]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _compile(src, extra):
    obj = os.path.join(LIB_DIR, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    return src, obj, r.returncode, r.stdout + r.stderr


def build(verbose=False, ptxas_info=False):
    os.makedirs(LIB_DIR, exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    log = []
    for src, obj, rc, out in results:
        if rc != 0 or verbose or ptxas_info:
            log.append(f"== {src}\n{out}")
        if rc != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{out}")
    objs = [r[1] for r in results]
    cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    if log and (verbose or ptxas_info):
        print("\n".join(log))
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
