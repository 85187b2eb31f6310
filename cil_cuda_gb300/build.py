"""Builds libcilgpu.so in-tree for sm_103a (GB300).

Each translation unit under csrc/ is compiled in parallel with
`nvcc -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo`, then linked into
cil_cuda_gb300/_build/libcilgpu.so. No CMake, no torch extension machinery.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libcilgpu.so")
RUNNER = os.path.join(OUT, "cil_gpu_run")
SOURCES = ["cil_api.cu", "cil_bins.cu", "cil_force.cu", "cil_events.cu", "cil_skin.cu", "cil_mlp.cu", "cil_noalloc.cu",
           "cil_frame.cu", "cil_input.cpp", "cil_cycle.cu", "cil_h5.cpp"]
# per-file flags: the single-element cycle model keeps FP64 products and sums separate (no FMA
# contraction) so that it computes exactly what its host restatement computes; the force kernels
# flush FP32 denormals (no denormal fix-up code around the reciprocal square roots of the FP32
# pair laws; the FP64 paths are unaffected)
EXTRA = {"cil_cycle.cu": ["--fmad=false"], "cil_force.cu": ["-ftz=true"]}
# sources compiled a second time into another object with extra defines: the force kernels'
# 3D instances build in parallel with the 2D ones
SECOND = {"cil_force.cu": ("cil_force3.o", ["-DCIL_FORCE_DIM=3"])}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def flags(extra=()):
    # host code: no FMA contraction, so that the oracle-mode host draws and the INIT draws give
    # the same bits on x86-64 and aarch64 hosts
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
                   "-Xcompiler", "-ffp-contract=off",
                   "-I", os.path.join(ROOT, "include"), "-I", CSRC, *extra]


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    procs = []
    objs = []
    units = [(src, os.path.splitext(src)[0] + ".o", []) for src in SOURCES]
    units += [(src, o, d) for src, (o, d) in SECOND.items()]
    for src, obj_name, defines in units:
        obj = os.path.join(OUT, obj_name)
        objs.append(obj)
        src_path = os.path.join(CSRC, src)
        deps = [src_path] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
        deps += [os.path.join(ROOT, "include", h) for h in os.listdir(os.path.join(ROOT, "include"))]
        if (not ptxas_info and os.path.exists(obj)
                and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps)):
            continue
        cmd = [nvcc(), *flags(extra), *EXTRA.get(src, []), *defines, "-c", src_path, "-o", obj]
        procs.append((obj_name, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        if verbose or p.returncode != 0 or ptxas_info:
            sys.stdout.write(out)
        if p.returncode != 0:
            failed.append(src)
    if failed:
        raise RuntimeError(f"nvcc failed for {failed}")
    cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lpthread"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        sys.stdout.write(r.stdout)
        raise RuntimeError("link failed")
    # the reference-shaped runner: JSON run description -> GPU step -> GSD frames
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), os.path.join(HERE, "host", "run_json.cpp"),
           "-L", OUT, "-lcilgpu", "-Wl,-rpath,$ORIGIN", "-o", RUNNER]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        sys.stdout.write(r.stdout)
        raise RuntimeError("cil_gpu_run build failed")
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="-v" in sys.argv)
    print(LIB)
