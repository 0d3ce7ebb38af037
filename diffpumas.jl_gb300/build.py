"""Builds libdpgpu.so (sm_103a) in-tree: diffpumas.jl_gb300/_build/libdpgpu.so.

Each CUDA translation unit is compiled in parallel with nvcc, then linked.
Usage: python diffpumas.jl_gb300/build.py [--force]
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libdpgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no FMA contraction, so the host table builders give the same
# bits on x86 and Arm (the device code keeps nvcc's default contraction)
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr", "--extended-lambda"]
UNITS = ["api.cu", "physics_build.cu", "csda_mc.cu", "tomo.cu", "mc.cu", "dir_mc.cu",
         "inverse.cu", "wtomo.cu", "voxel_trace.cu", "topo_trace.cu"]
# per-unit flags: the stochastic transport's FP32 kernel uses the hardware
# (MUFU) transcendentals; FP64 arithmetic is not affected by these flags
UNIT_FLAGS = {"mc.cu": ["--use_fast_math"], "dir_mc.cu": ["--use_fast_math"],
              "wtomo.cu": ["--use_fast_math"]}


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _stale(obj, src_files):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(f) > t for f in src_files)


def build(force=False, verbose=False, extra=()):
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".cuh", ".h", ".inc"))]
    headers.append(os.path.join(HERE, "..", "include", "dpgpu.h"))
    jobs = []
    for u in UNITS:
        src = os.path.join(SRC, u)
        obj = os.path.join(OUT, u.replace(".cu", ".o"))
        if force or _stale(obj, [src, *headers, __file__]):
            jobs.append((src, obj))
    cmdline = [nvcc(), *ARCH, *FLAGS, *extra]

    def run(job):
        src, obj = job
        cmd = [*cmdline, *UNIT_FLAGS.get(os.path.basename(src), []), "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stderr}")
        return r.stderr

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for msg in ex.map(run, jobs):
            if verbose and msg:
                print(msg)
    objs = [os.path.join(OUT, u.replace(".cu", ".o")) for u in UNITS]
    if jobs or not os.path.exists(LIB):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stderr)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
