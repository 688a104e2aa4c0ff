"""Builds libpovgpu.so in-tree with nvcc for sm_103a.

Each translation unit is compiled in its own nvcc process (in parallel), then
linked into povray_gb300/lib/libpovgpu.so.  No cmake, one -gencode.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "lib")
OBJ_DIR = os.path.join(HERE, "lib", "obj")
LIB = os.path.join(OUT_DIR, "libpovgpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["povgpu_host.cpp", "povgpu_reftree.cpp", "povgpu_kernels.cu", "povgpu_radiosity.cu", "povgpu_nic.cu"]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def _flags(src):
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include"), "-I", CSRC]
    if src.endswith(".cu"):
        return common + ARCH + ["-lineinfo", "-Xptxas", "-O3"]
    return common + ARCH


def build(verbose=False, ptxas_info=False):
    os.makedirs(OBJ_DIR, exist_ok=True)
    exe = nvcc()

    def compile_one(src):
        path = os.path.join(CSRC, src)
        obj = os.path.join(OBJ_DIR, src + ".o")
        cmd = [exe, "-c", path, "-o", obj] + _flags(src)
        if ptxas_info and src.endswith(".cu"):
            cmd += ["-Xptxas", "-v"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
        return obj, r.stderr

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(compile_one, SOURCES))
    objs = [o for o, _ in results]
    if verbose or ptxas_info:
        for _, err in results:
            if err:
                sys.stderr.write(err)
    cmd = [exe, "-shared", "-o", LIB] + objs + ARCH + ["-lcudart_static", "-lpthread", "-ldl", "-lrt"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="-v" in sys.argv))
