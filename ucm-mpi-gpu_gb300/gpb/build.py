"""Builds libgpb.so (the CUDA library, sm_103a) in-tree with nvcc.

Each translation unit compiles in its own nvcc process, in parallel, then
one link step; the whole build takes well under a minute.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(ROOT, "csrc")
OBJ = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "libgpb.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
          "-I" + CSRC, "-I" + os.path.join(os.path.dirname(ROOT), "include")]
# host code whose loops the compiler should vectorise (results are the same
# to the bit: -ffp-contract=off and no reassociation)
HOST_O3 = {"eig_host.cpp"}
SOURCES = ["tables.cpp", "eig_host.cpp", "gpb_api.cpp", "gpb_damascene.cpp", "io_writers.cpp", "k_block.cu",
           "k_front.cu", "k_static.cu", "k_stitch.cu", "k_spfeat.cu", "k_cues.cu", "k_buildw.cu", "k_eig.cu", "k_spb.cu",
           "ucm_host.cpp", "ucm_api.cpp", "k_ucm.cu", "k_warmnet.cu", "k_learned.cu"]


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _compile(src):
    os.makedirs(OBJ, exist_ok=True)
    out = os.path.join(OBJ, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    deps = [path] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith(".h")]
    deps.append(os.path.join(os.path.dirname(ROOT), "include", "gpb.h"))
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
        return out
    cmd = [nvcc()] + ARCH + COMMON + ["-c", path, "-o", out]
    if src in HOST_O3:
        cmd += ["-Xcompiler", "-O3"]
    if src.endswith(".cu"):
        cmd += ["-Xptxas", "-warn-spills"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed on %s:\n%s%s" % (src, r.stdout, r.stderr))
    return out


def build(verbose=False):
    objs = []
    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        for o in ex.map(_compile, SOURCES):
            objs.append(o)
    if os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(o) for o in objs):
        return LIB
    cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
