"""Builds libchipmunk_gb300.so in-tree (chipmunk2d_gb300/_build/).

CUDA sources are compiled for sm_103a only, with --fmad=false so that no
multiply-add contraction changes FP64 rounding; C sources are compiled with
-ffp-contract=off for the same reason.  Translation units compile in
parallel.  Usage: python -m chipmunk2d_gb300.build [--debug]
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
REPO = os.path.dirname(PKG)
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc") if os.path.exists(os.path.join(CUDA_HOME, "bin", "nvcc")) else "nvcc"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["cpg_kernels.cu", "cpg_schedule_api.cu", "cpg_rollout.cu", "cpg_query.cu"]
C_SOURCES = ["cp_host.c"]
# The seeded workloads the tests and the benchmark build through the public
# API: a library of their own that links against the product, so the
# product exports nothing but the API.
SCENE_SOURCES = ["scenes.c", "scene_export_gpu.c"]


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def build(verbose=False, ptxas_info=False):
    os.makedirs(OUT, exist_ok=True)
    inc = ["-I" + SRC, "-I" + os.path.join(REPO, "include"), "-I" + os.path.join(CUDA_HOME, "include")]
    jobs = []
    objs = []
    for f in CU_SOURCES:
        obj = os.path.join(OUT, f + ".o")
        cmd = [NVCC] + ARCH + ["-O3", "-lineinfo", "--fmad=false", "-prec-div=true", "-prec-sqrt=true",
                               "-std=c++17", "-Xcompiler", "-fPIC", "-c", os.path.join(SRC, f), "-o", obj] + inc
        if ptxas_info:
            cmd += ["-Xptxas", "-v"]
        jobs.append(cmd)
        objs.append(obj)
    for f in C_SOURCES + SCENE_SOURCES:
        obj = os.path.join(OUT, f + ".o")
        cmd = ["gcc", "-std=gnu11", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
               "-c", os.path.join(SRC, f), "-o", obj] + inc
        jobs.append(cmd)
        if f in C_SOURCES:
            objs.append(obj)
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose or ptxas_info:
        for o in outs:
            if o.strip():
                print(o)
    lib = os.path.join(OUT, "libchipmunk_gb300.so")
    tmp = lib + ".tmp"
    _run([NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lm"])
    shutil.move(tmp, lib)
    scenes = os.path.join(OUT, "libcpx_scenes.so")
    _run(["gcc", "-shared", "-o", scenes + ".tmp"] + [os.path.join(OUT, f + ".o") for f in SCENE_SOURCES] +
         ["-L" + OUT, "-lchipmunk_gb300", "-Wl,-rpath,$ORIGIN", "-lm"])
    shutil.move(scenes + ".tmp", scenes)
    return lib


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="--ptxas" in sys.argv))
