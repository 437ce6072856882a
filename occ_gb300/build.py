"""Build the GB300 XC library in-tree: occ_gb300/lib/libocc_xc.so.

CUDA sources are compiled for sm_103a only; host C++ sources with g++ and
OpenMP.  Translation units compile in parallel; the link uses nvcc.
usage: python -m occ_gb300.build   (or occ_gb300.build.build())
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "lib")
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libocc_xc.so")

CU_SOURCES = ["xc_fp64.cu", "xc_mixed.cu", "xc_engine.cu", "xc_noalloc.cu", "xc_server.cu",
              "xc_tune.cu", "xc_grad.cu", "xc_grid.cu", "xc_uks.cu",
              "xc_vv10.cu", "xc_plan.cu", "xc_cosx.cu"]
CXX_SOURCES = ["host/basis.cpp", "host/grid.cpp", "host/plan.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else (shutil.which("nvcc") or "nvcc")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _obj(src):
    return os.path.join(BUILD_DIR, src.replace("/", "_") + ".o")


def _stale(src, obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in [src] + deps)


def build(verbose=False, extra_nvcc=()):
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(BUILD_DIR, exist_ok=True)
    headers = []
    for root, _, files in os.walk(CSRC):
        headers += [os.path.join(root, f) for f in files if f.endswith((".h", ".hpp", ".cuh"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "occ_xc.h"))
    jobs = []
    for s in CU_SOURCES:
        src = os.path.join(CSRC, s)
        obj = _obj(s)
        if _stale(src, obj, headers):
            jobs.append([nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-Xptxas", "-v" if verbose else "-O3", *extra_nvcc,
                         "-I", CSRC, "-c", src, "-o", obj])
    for s in CXX_SOURCES:
        src = os.path.join(CSRC, s)
        obj = _obj(s)
        if _stale(src, obj, headers):
            jobs.append(["g++", "-O3", "-fPIC", "-fopenmp", "-std=c++17", "-I", CSRC, "-c", src,
                         "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    objs = [_obj(s) for s in CU_SOURCES + CXX_SOURCES]
    if jobs or not os.path.exists(LIB):
        _run([nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-Xcompiler", "-fopenmp"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
