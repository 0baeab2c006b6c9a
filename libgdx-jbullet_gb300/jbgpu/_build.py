"""Builds libjbgpu.so (the C-ABI rigid-body step) in-tree with nvcc for sm_103a.

Translation units are compiled in parallel.  Device code uses -fmad=false with IEEE
division and square root so that every float operation is a separately rounded
binary32 operation, as in the reference's Java arithmetic; host code is compiled
without floating-point contraction for the same reason.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)                       # libgdx-jbullet_gb300/
CSRC = os.path.join(ROOT, "csrc")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(BUILD, "libjbgpu.so")
SOURCES = ["prims.cu", "bodies.cu", "broadphase.cu", "narrowphase.cu", "solver.cu", "mlp.cu", "query.cu", "meshes.cu",
           "world.cu"]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def flags():
    return [ARCH, "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
            "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-Xptxas", "-O3"]


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    deps.append(os.path.join(os.path.dirname(ROOT), "include", "jbgpu.h"))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    jobs = []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s.replace(".cu", ".o"))
        if force or _stale(obj, src):
            jobs.append([cc] + flags() + ["-c", src, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for cmd, res in zip(jobs, ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs)):
                if verbose and res.stderr:
                    print(res.stderr)
                if res.returncode != 0:
                    raise RuntimeError("nvcc failed: %s\n%s%s" % (" ".join(cmd), res.stdout, res.stderr))
    objs = [os.path.join(BUILD, s.replace(".cu", ".o")) for s in SOURCES]
    if force or jobs or not os.path.exists(LIB):
        cmd = [cc, ARCH, "-shared", "-o", LIB] + objs + ["-lcudart"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("link failed: %s\n%s" % (" ".join(cmd), res.stderr))
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
