"""Build the sm_103a shared library libh2w.so in-tree with nvcc.

Every translation unit is compiled for one target, compute_103a/sm_103a,
in parallel; the objects are linked into h2weak_gb300/_lib/libh2w.so
against the shared CUDA runtime (the one PyTorch also loads).
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libh2w.so")
SOURCES = ["kernels.cu", "multi.cu", "mrtc.cu", "mrws.cu", "gmbatch.cu", "batch.cu", "learn.cu", "ncabig.cu", "m2lfly.cu", "noalloc.cu", "helm.cu", "capi.cpp", "tree.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O3", "--cudart", "shared",
                   "-I" + os.path.join(HERE, "..", "include")]


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    deps = [os.path.join(SRC, f) for f in os.listdir(SRC)] + [os.path.join(HERE, "..", "include", "h2w.h")]
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in deps):
            return LIB
    cc = nvcc()
    objs = []

    def comp(src):
        obj = os.path.join(OUT, src + ".o")
        cmd = [cc] + _flags() + ["-c", os.path.join(SRC, src), "-o", obj]
        if src.endswith(".cu"):
            cmd += ["-Xptxas", "-v"] if verbose else []
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
        if verbose:
            sys.stderr.write(r.stderr)
        return obj

    with concurrent.futures.ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(comp, SOURCES))
    tmp = LIB + ".tmp"
    r = subprocess.run([cc] + ARCH + ["-shared", "--cudart", "shared", "-o", tmp] + objs, capture_output=True,
                       text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
