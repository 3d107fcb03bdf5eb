"""Build libcmcgpu.so (sm_103a CUDA kernels + C host code) in-tree.

    python cmc-cosmic_gb300/build.py            # build if sources changed
    python cmc-cosmic_gb300/build.py --force    # rebuild everything

Every translation unit compiles in parallel with one -gencode for sm_103a.
Physics kernels build with -fmad=false: the reference's FP64 expressions are
evaluated one rounded operation at a time (its C is compiled without FP
contraction), and the kernels must round identically to be bit-comparable.
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libcmcgpu.so")

CUDA_SOURCES = [
    "cmcg_host.cu",
    "cmcg_relax.cu",
    "cmcg_orbit.cu",
    "cmcg_sort.cu",
    "cmcg_potential.cu",
    "cmcg_phi.cu",
    "cmcg_energy.cu",
    "cmcg_noalloc.cu",
    "cmcg_diag.cu",
    "cmcg_mlp.cu",
]
C_SOURCES = ["cmcg_ic.c", "cmcg_h5.c"]
# the synthetic-cluster generator alone (plain C, no CUDA): what the CPU
# baselines and the oracle tests load to build their models
IC_LIB = os.path.join(BUILD, "libcmcic.so")
# the reference-named drop-in layer: a second library on the public C ABI
DROPIN_SOURCE = "cmc_dropin.cpp"
DROPIN_LIB = os.path.join(BUILD, "libcmc_dropin.so")
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + res.stdout)
        raise RuntimeError(f"compile failed: {cmd[-1]}")
    if res.stdout.strip():
        sys.stderr.write(res.stdout)


def build_ic(force: bool = False) -> str:
    """libcmcic.so: cmcg_ic_generate, cmcg_derive_seed and cmcg_read_cmc_hdf5
    without the GPU library."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in C_SOURCES]
    hdr = os.path.join(ROOT, "include", "cmcgpu.h")
    if force or not _newer(IC_LIB, srcs + [hdr]):
        _run(["gcc", "-O2", "-fPIC", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-shared",
              "-I" + os.path.join(ROOT, "include"), "-o", IC_LIB, *srcs, "-lm"])
    return IC_LIB


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    build_ic(force)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "cmcgpu.h"))
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
    jobs = []
    objs = []
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or not _newer(o, [s] + headers):
            cmd = [nvcc(), GENCODE, "-O3", "-lineinfo", "-std=c++17", "-fmad=false",
                   "-Xcompiler", "-fPIC", "-c", *inc, "-o", o, s]
            if verbose_ptxas:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for src in C_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or not _newer(o, [s] + headers):
            jobs.append(["gcc", "-O2", "-fPIC", "-std=c11", "-ffp-contract=off", "-fno-fast-math",
                         *inc, "-c", "-o", o, s])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(_run, jobs))
    if jobs or not os.path.exists(LIB):
        _run([nvcc(), GENCODE, "-shared", "-o", LIB, *objs, "-lm"])
    src = os.path.join(CSRC, DROPIN_SOURCE)
    if force or not _newer(DROPIN_LIB, [src, LIB] + headers):
        _run(["g++", "-O2", "-fPIC", "-std=c++17", "-shared", *inc, "-o", DROPIN_LIB, src,
              "-L" + BUILD, "-lcmcgpu", "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--ptxas", action="store_true", help="print -Xptxas -v resource usage")
    a = ap.parse_args()
    print(build(force=a.force, verbose_ptxas=a.ptxas))
