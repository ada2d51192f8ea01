"""Build recipe for the reference CPU solver, used as a checker (test
infrastructure only; the product never links or loads it).

Compiles the reference's own kern_interp sources, unmodified, from where they
lie (default /root/reference, override with KI_REFERENCE_ROOT) together with
oracle/ref_driver.cpp into a shared library under oracle/_ref/.  Three small
shim headers (oracle/shim/) map CBLAS/LAPACKE names onto the OpenBLAS build
bundled with scipy and stand in for boost::hash.

The reference fixes its tree/proxy parameters with unguarded macros
(MAX_LEAF_DOFS kern_interp/quadtree/quadtree.h:11, NUM_PROXY_POINTS and
RADIUS_RATIO kern_interp/kernel/kernel.h:13-14, MIN_DOFS_TO_COMPRESS
kern_interp/skel_factorization/skel_factorization.h:12).  For non-default
values this script writes patched copies of those three headers into the
variant's build folder (oracle/_ref/<variant>/include), which shadow the
originals on the include path.  Nothing is copied into the repository.

Usage: python oracle/build_ref.py [--leaf 64] [--proxy 128] [--ratio 2]
                                  [--min-compress 64]
Returns the path of the built library.
"""
import argparse
import glob
import hashlib
import os
import re
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
SOURCES = [
    "kern_interp/ki_mat.cpp",
    "kern_interp/pointvec.cpp",
    "kern_interp/legendre.cpp",
    "kern_interp/linear_solve.cpp",
    "kern_interp/kernel/kernel.cpp",
    "kern_interp/quadtree/quadtree.cpp",
    "kern_interp/skel_factorization/skel_factorization.cpp",
    "kern_interp/boundaries/boundary.cpp",
]
PATCHED = {
    "kern_interp/quadtree/quadtree.h": [("MAX_LEAF_DOFS", "leaf")],
    "kern_interp/kernel/kernel.h": [("NUM_PROXY_POINTS", "proxy"), ("RADIUS_RATIO", "ratio")],
    "kern_interp/skel_factorization/skel_factorization.h": [("MIN_DOFS_TO_COMPRESS", "min_compress")],
}


def reference_root():
    """Where the reference sources are read: KI_REFERENCE_ROOT, else the
    checkout this recipe was written against."""
    return os.environ.get("KI_REFERENCE_ROOT", "/root/reference")


def reference_present():
    return os.path.isdir(os.path.join(reference_root(), "kern_interp"))


def openblas_path():
    import scipy
    libs = os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs")
    cands = sorted(glob.glob(os.path.join(libs, "libscipy_openblas*.so")))
    if not cands:
        raise RuntimeError("scipy's bundled OpenBLAS not found in " + libs)
    return cands[0]


def variant_name(leaf, proxy, ratio, min_compress):
    return "leaf%d_proxy%d_ratio%s_min%d" % (leaf, proxy, repr(float(ratio)).replace(".", "p"), min_compress)


def build(leaf=64, proxy=128, ratio=2.0, min_compress=64, verbose=False):
    root = reference_root()
    if not os.path.isdir(os.path.join(root, "kern_interp")):
        raise FileNotFoundError("reference sources not found at " + root)
    name = variant_name(leaf, proxy, ratio, min_compress)
    vdir = os.path.join(OUT, name)
    lib = os.path.join(vdir, "libkiref.so")
    drv = os.path.join(HERE, "ref_driver.cpp")
    stamp_src = open(drv, "rb").read() + repr((leaf, proxy, ratio, min_compress)).encode()
    stamp = hashlib.sha1(stamp_src).hexdigest()
    stamp_file = os.path.join(vdir, "stamp")
    if os.path.exists(lib) and os.path.exists(stamp_file) and open(stamp_file).read() == stamp:
        return lib
    inc = os.path.join(vdir, "include")
    vals = {"leaf": str(leaf), "proxy": str(proxy), "ratio": repr(float(ratio)),
            "min_compress": str(min_compress)}
    for rel, macros in PATCHED.items():
        text = open(os.path.join(root, rel)).read()
        for macro, key in macros:
            text, n = re.subn(r"#define\s+%s\s+\S+" % macro, "#define %s %s" % (macro, vals[key]), text)
            if n != 1:
                raise RuntimeError("could not patch %s in %s" % (macro, rel))
        dst = os.path.join(inc, rel)
        os.makedirs(os.path.dirname(dst), exist_ok=True)
        with open(dst, "w") as f:
            f.write(text)
    objdir = os.path.join(vdir, "obj")
    os.makedirs(objdir, exist_ok=True)
    flags = ["g++", "-O2", "-fopenmp", "-std=c++14", "-fPIC", "-w",
             "-I" + inc, "-I" + os.path.join(HERE, "shim"), "-I" + root]

    def compile_one(src):
        obj = os.path.join(objdir, os.path.basename(src).replace(".cpp", ".o"))
        subprocess.run(flags + ["-c", src, "-o", obj], check=True)
        return obj

    srcs = [os.path.join(root, s) for s in SOURCES] + [drv]
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        objs = list(ex.map(compile_one, srcs))
    blas = openblas_path()
    subprocess.run(["g++", "-shared", "-fopenmp", "-o", lib] + objs +
                   ["-L" + os.path.dirname(blas), "-l:" + os.path.basename(blas),
                    "-Wl,-rpath," + os.path.dirname(blas)], check=True)
    with open(stamp_file, "w") as f:
        f.write(stamp)
    if verbose:
        print(lib)
    return lib


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--leaf", type=int, default=64)
    ap.add_argument("--proxy", type=int, default=128)
    ap.add_argument("--ratio", type=float, default=2.0)
    ap.add_argument("--min-compress", type=int, default=64)
    a = ap.parse_args()
    print(build(a.leaf, a.proxy, a.ratio, a.min_compress))
