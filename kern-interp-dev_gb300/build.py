"""Build libki_gpu.so (the C-ABI library behind include/ki_gpu.h) in-tree.

nvcc compiles the CUDA translation units for sm_103a only, g++ the host
tree code; the shared library is written next to this file.  Rebuilds only
when a source changed (content hash).
"""
import hashlib
import platform
import os
import shutil
import subprocess
import sys
import time
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libki_gpu.so")
OBJ = os.path.join(ROOT, "_build", "obj")

CU_SOURCES = ["ki_factor.cu", "ki_dense.cu", "ki_abi.cu", "ki_fmm.cu", "ki_pool.cu", "ki_mlp.cu",
              "ki_tree_gpu.cu"]
CPP_SOURCES = ["ki_tree.cpp", "ki_tune.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    p = os.path.join(cuda, "bin", "nvcc")
    return p if os.path.exists(p) else (shutil.which("nvcc") or "nvcc")


def _digest():
    h = hashlib.sha1()
    for d in (CSRC, os.path.join(ROOT, "include")):
        for f in sorted(os.listdir(d)):
            if f.endswith((".cu", ".cuh", ".h", ".cpp")):
                h.update(f.encode())
                h.update(open(os.path.join(d, f), "rb").read())
    h.update(" ".join(ARCH).encode())
    h.update(platform.machine().encode())   # a library built on another host arch never matches
    return h.hexdigest()


def build(force=False, verbose=False):
    stamp = LIB + ".stamp"
    dig = _digest()
    if not force and os.path.exists(LIB) and os.path.exists(stamp) and open(stamp).read() == dig:
        print("libki_gpu.so up to date (sources unchanged, %s)" % platform.machine(), file=sys.stderr)
        return LIB
    t0 = time.time()
    os.makedirs(OBJ, exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    for s in CU_SOURCES:
        jobs.append([nvcc] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                                    "-I" + os.path.join(ROOT, "include"), "-c",
                                    os.path.join(CSRC, s), "-o", os.path.join(OBJ, s + ".o")])
    for s in CPP_SOURCES:
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-c", os.path.join(CSRC, s), "-o",
                     os.path.join(OBJ, s + ".o")])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)

    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        list(ex.map(run, jobs))
    objs = [os.path.join(OBJ, s + ".o") for s in CU_SOURCES + CPP_SOURCES]
    tmp = LIB + ".tmp"
    run([nvcc] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs)
    os.replace(tmp, LIB)
    with open(stamp, "w") as f:
        f.write(dig)
    print("libki_gpu.so built: %d translation units for %s on %s in %.0f s" %
          (len(jobs), " ".join(ARCH), platform.machine(), time.time() - t0), file=sys.stderr)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
