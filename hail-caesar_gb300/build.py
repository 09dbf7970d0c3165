"""Builds libhc_gpu.so in-tree with nvcc for sm_103a (GB300).

Every translation unit is compiled in parallel, then linked.  --fmad=false
keeps every multiply and add separately rounded, as in the reference's CPU
build, so the hydraulic state is bit-identical to it.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libhc_gpu.so")
BUILD = os.path.join(HERE, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "--fmad=false", "-lineinfo", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-ffp-contract=off", "-Xptxas", "-warn-spills"]
SOURCES = ["hc_api.cu", "hc_flow.cu", "hc_erode.cu", "hc_slide.cu", "hc_lateral.cu",
           "hc_host.cpp", "hc_drain.cu", "hc_adjoint.cu", "hc_noalloc.cu",
           "hc_sort.cu", "hc_tune.cu"]


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _newer(out, deps):
    if not os.path.exists(out):
        return False
    t = os.path.getmtime(out)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(verbose=False, force=False, extra=None):
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "hc_gpu.h"))
    nv = nvcc()
    extra = extra or []

    def one(src):
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src + ".o")
        if not force and _newer(obj, [path] + headers):
            return obj
        if src.endswith(".cpp"):
            cmd = [nv, "-x", "c++", "-O2", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-Xcompiler", "-ffp-contract=off", "-c", path, "-o", obj]
        else:
            cmd = [nv] + ARCH + NVFLAGS + extra + ["-c", path, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed on %s:\n%s%s" % (src, r.stdout, r.stderr))
        if verbose and (r.stderr.strip() or r.stdout.strip()):
            print(r.stdout + r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(one, SOURCES))
    if force or not _newer(OUT, objs):
        cmd = [nv] + ARCH + ["-shared", "-o", OUT] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    return OUT


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv,
          extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else None)
    print(OUT)
