"""Builds libkiyosi_gpu.so in-tree with nvcc for sm_103a (GB300).

Translation units compile in parallel; kernels_fp64.cu is compiled with --fmad=false so
the FP64 kernels round every product and sum separately, as the Rust reference does, and
the host planner (planner.cpp) with floating-point contraction off for the same reason
(an Arm host compiler would otherwise fuse its products and sums).
Usage: python -m kiyosi_gb300.build [--force]
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libkiyosi_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
          "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]
UNITS = {
    "api.cu": [],
    "kernels_fp64.cu": ["--fmad=false"],
    "kernels_fp32.cu": [],
    "lsmc.cu": [],
    "mlp.cu": [],
    "noalloc.cu": [],
    "pipes.cu": [],
    "planner.cpp": ["-Xcompiler", "-ffp-contract=off"],
}
HEADERS = ["device_rng.cuh", "path_engine.cuh", "kernels.cuh", "kernels_impl.cuh", "launch.h",
           "api_internal.h", "joe_kuo_6_21201.inc", "shared_grid.cuh", "lsmc_common.cuh", "tcgen05.cuh", "phased.cuh", "segmented.cuh", "straight.cuh"]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build kiyosi_gb300")
    return path


def _newest(paths):
    return max((os.path.getmtime(p) for p in paths if os.path.exists(p)), default=0.0)


def _compile(unit: str, flags, verbose: bool) -> str:
    src = os.path.join(CSRC, unit)
    obj = os.path.join(BUILD, os.path.splitext(unit)[0] + ".o")
    deps = [src, os.path.join(HERE, "..", "include", "kgpu.h")] + [
        os.path.join(CSRC, h) for h in HEADERS]
    if os.path.exists(obj) and os.path.getmtime(obj) >= _newest(deps) and not verbose:
        return obj
    cmd = [nvcc(), *ARCH, *COMMON, *flags, "-c", src, "-o", obj]
    if verbose:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{r.stdout}\n{r.stderr}")
    if verbose:
        sys.stderr.write(r.stderr)
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if force:
        for f in os.listdir(BUILD):
            os.remove(os.path.join(BUILD, f))
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as pool:
        objs = list(pool.map(lambda kv: _compile(kv[0], kv[1], verbose), UNITS.items()))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < _newest(objs) or force:
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
