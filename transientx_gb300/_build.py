"""In-tree build of the native libraries (no cmake): the CUDA library libtxgpu.so for sm_103a
and the host-only synthetic-data library libtxsynth.so."""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libtxgpu.so")
SYNTH = os.path.join(PKG, "libtxsynth.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SRC = ["txg_pre.cu", "txg_dedisp.cu", "txg_boxcar.cu", "txg_api.cu", "txg_noalloc.cu",
          "txg_replot.cu"]
# files whose device arithmetic follows the reference's mixed float/double expressions as
# written: no multiply-add contraction anywhere in them
NO_FMAD = {"txg_replot.cu"}
CPP_SRC = ["txg_plan.cpp", "txg_cluster.cpp"]


def nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build transientx_gb300")


def cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, "txg_internal.h"),
               os.path.join(os.path.dirname(PKG), "include", "transientx_gb300.h")]
    jobs, objs = [], []
    nv = nvcc()
    for src in CU_SRC:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            cmd = [nv, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                   "-c", s, "-o", o]
            if src in NO_FMAD:
                cmd.insert(1, "-fmad=false")
            if verbose:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for src in CPP_SRC:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append(["g++", "-O3", "-std=c++17", "-fPIC", "-ffp-contract=off",
                         f"-I{cuda_home()}/include", "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        list(ex.map(_run, jobs))
    if force or jobs or _stale(LIB, objs):
        _run([nv, *ARCH, "-shared", "-cudart", "static", "-o", LIB, *objs])
    synth_src = os.path.join(CSRC, "synth.c")
    if force or _stale(SYNTH, [synth_src]):
        _run(["gcc", "-O3", "-std=gnu11", "-fPIC", "-fopenmp", "-ffp-contract=off", "-shared",
              synth_src, "-o", SYNTH, "-lm"])
    return LIB


if __name__ == "__main__":
    import sys
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
