"""Builds libfedem_solver_core.so (the GB300 solver core) in-tree.

nvcc compiles the CUDA translation units for sm_103a only; g++ compiles the
host set-up.  Translation units build in parallel; outputs go to
fedem-solvers_gb300/lib/ (git-ignored).
"""
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(PKG_ROOT, "csrc")
LIB_DIR = os.path.join(PKG_ROOT, "lib")
LIB_PATH = os.path.join(LIB_DIR, "libfedem_solver_core.so")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["engine.cu", "element_kernels.cu", "front_kernels.cu", "front_cascade.cu", "norms_noalloc.cu",
              "joint_kernels.cu", "front_large.cu", "peaks.cu", "part_kernels.cu", "results.cu"]
CPP_SOURCES = ["host_model.cpp", "symbolic.cpp", "server.cpp", "eigen.cpp", "capi.cpp"]


def _run(cmd):
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + proc.stdout)
    return proc.stdout


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False, ptxas_info=False):
    """Compiles every translation unit (parallel) and links the shared library."""
    obj_dir = os.path.join(LIB_DIR, "obj")
    os.makedirs(obj_dir, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers += [os.path.join(PKG_ROOT, "..", "include", f) for f in ("fedem_solver_core.h", "fgpu.h")]
    jobs = []
    for src in CU_SOURCES:
        obj = os.path.join(obj_dir, src + ".o")
        deps = [os.path.join(CSRC, src)] + headers
        if force or _stale(obj, deps):
            cmd = [NVCC] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                                   "-c", os.path.join(CSRC, src), "-o", obj]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for src in CPP_SOURCES:
        obj = os.path.join(obj_dir, src + ".o")
        deps = [os.path.join(CSRC, src)] + headers
        if force or _stale(obj, deps):
            cxx = shutil.which("g++") or "g++"
            jobs.append([cxx, "-O2", "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-function",
                         "-I" + os.path.join(CUDA_HOME, "include"), "-c", os.path.join(CSRC, src), "-o", obj])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    objs = [os.path.join(obj_dir, s + ".o") for s in CU_SOURCES + CPP_SOURCES]
    if force or jobs or not os.path.exists(LIB_PATH):
        _run([NVCC] + ARCH + ["-shared", "-o", LIB_PATH] + objs + ["-lpthread"])
    return LIB_PATH


if __name__ == "__main__":
    import sys
    print(build(verbose=True, force="--force" in sys.argv, ptxas_info="--ptxas" in sys.argv))
