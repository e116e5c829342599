"""Build libmcphylo_gpu.so (sm_103a) in-tree with nvcc.

    python mcphylo.jl_gb300/build.py [--force] [--verbose]

Translation units compile in parallel into mcphylo.jl_gb300/_build/ and link into
mcphylo.jl_gb300/mcphylo_gb300/libmcphylo_gpu.so (CUDA runtime linked statically).
``--verbose`` passes -Xptxas -v (registers, spills, shared memory per kernel).
"""
import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "mcphylo_gb300", "libmcphylo_gpu.so")
SOURCES = ["schedule.cpp", "api.cu", "noalloc.cu", "kernels_common.cu", "kernels_f32.cu",
           "kernels_f32_g20.cu", "kernels_f32_g32.cu", "kernels_f32_narrow.cu", "kernels_f32_wide.cu", "kernels_f64.cu",
           "kernels_f64_g20.cu", "kernels_f64_g32.cu", "kernels_f64_rnarrow.cu", "kernels_f64_rwide.cu", "kernels_tc.cu",
           "kernels_level.cu", "tc_selftest.cu"]
HEADERS = ["mcphy_internal.h", "kernels.cuh", "engine_state.h", "tc.cuh", "launch_attr.h",
           "prune_launch.cuh", "kernels_walk.cuh", "walk_subsets.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "mcphylo_gpu.h")]
    common = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
                     "-I", INCLUDE, "-I", CSRC]
    if verbose:
        common += ["-Xptxas", "-v"]
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or verbose or _stale(o, [s] + hdrs):
            jobs.append([nvcc()] + common + ["-c", s, "-o", o])

    def run(cmd):
        p = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, p

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        for cmd, p in ex.map(run, jobs):
            if p.returncode != 0:
                sys.stderr.write(p.stdout + p.stderr)
                raise RuntimeError("nvcc failed: " + " ".join(cmd))
            if verbose and (p.stdout or p.stderr):
                sys.stderr.write(p.stdout + p.stderr)
    if force or jobs or _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-cudart", "static"]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            sys.stderr.write(p.stdout + p.stderr)
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose", action="store_true")
    a = ap.parse_args()
    print(build(force=a.force, verbose=a.verbose))
