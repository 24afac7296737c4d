"""Builds the in-tree CUDA library libvkhr_cuda.so for sm_103a with nvcc.

Each translation unit compiles in parallel; the shared library is linked
with the static CUDA runtime so it has no dependency beyond the driver.
Host code is compiled with -ffp-contract=off: the voxelizer's host-side FP32
set-up must not be fused into FMAs on aarch64.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libvkhr_cuda.so")
BUILD = os.path.join(HERE, "_build")
SOURCES = ["context.cu", "prepare.cu", "voxelize.cu", "raymarch.cu", "adjoint.cu", "frame.cu", "hair.cu", "composite.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libvkhr_cuda.so")


def _flags(verbose_ptxas=False):
    f = ["-O3", "-lineinfo", "-std=c++17", "--extended-lambda", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2"] + ARCH
    if verbose_ptxas:
        f += ["-Xptxas", "-v"]
    return f


def _stale(obj, src, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + deps)


def build(force=False, verbose_ptxas=False, quiet=False):
    os.makedirs(BUILD, exist_ok=True)
    exe = nvcc()
    deps = [os.path.join(CSRC, "common.cuh"), os.path.join(HERE, "..", "include", "vkhr_cuda.h")]
    jobs = []
    objs = []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, src, deps):
            jobs.append([exe, "-c", src, "-o", obj] + _flags(verbose_ptxas))
    logs = []

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for cmd, r in ex.map(run, jobs):
            logs.append(r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError("nvcc failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    if jobs or not os.path.exists(OUT) or any(os.path.getmtime(o) > os.path.getmtime(OUT) for o in objs):
        tmp = OUT + ".tmp"
        cmd = [exe, "-shared", "-o", tmp] + objs + ARCH + ["-cudart", "static"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        os.replace(tmp, OUT)
    if not quiet:
        for log in logs:
            if log.strip():
                sys.stderr.write(log)
    return OUT


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv)
    print(OUT)
