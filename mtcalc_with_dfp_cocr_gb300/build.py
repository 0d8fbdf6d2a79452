"""Build recipe for libmtgpu (sm_103a) and the drop-in COCR_FP executable.

Everything is compiled in-tree into mtcalc_with_dfp_cocr_gb300/_build/:
    libmtgpu.so       the CUDA library behind include/mtgpu.h
    mtgpu_cocr_fp     drop-in for the reference's COCR_FP.exe
Translation units are compiled in parallel with one -gencode for sm_103a.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libmtgpu.so")
EXE = os.path.join(OUT, "mtgpu_cocr_fp")

CU_SOURCES = ["sell.cu", "folded.cu", "cocr.cu", "assemble.cu", "survey.cu", "capi.cu", "capi_assembly.cu",
              "noalloc.cu", "receivers.cu", "adjoint.cu", "smoothing.cu", "regular_mesh.cu", "scan.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmtgpu")
    return p


def _flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-I", os.path.join(ROOT, "include"), "--expt-relaxed-constexpr"]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "mtgpu.h"))
    objs, jobs = [], []
    for s in CU_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OUT, s.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([nvcc()] + _flags() + ["-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for cmd, res in zip(jobs, ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs)):
            if res.returncode != 0:
                raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
            if verbose and (res.stdout or res.stderr):
                print(res.stdout, res.stderr)
    if force or _stale(LIB, objs):
        subprocess.check_call([nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    main = os.path.join(CSRC, "cocr_fp_main.cpp")
    if os.path.exists(main) and (force or _stale(EXE, [main, LIB])):
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
                               main, "-o", EXE, "-L", OUT, "-lmtgpu", "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True))
