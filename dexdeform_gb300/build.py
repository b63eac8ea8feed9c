"""Build libdexmpm.so (the product's CUDA kernels and C ABI) for sm_103a.

Each translation unit in csrc/ is compiled by nvcc in parallel and linked into
dexdeform_gb300/_lib/libdexmpm.so (CUDA runtime linked statically, no torch
dependency).  `python -m dexdeform_gb300.build` or `build()`.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libdexmpm.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
SOURCES = ["batched.cu", "sort.cu", "ref_abi.cu", "noalloc.cu", "render.cu"]
# the renderer keeps the reference's unfused float arithmetic (its images are
# compared pixel by pixel with the reference's code run on the host)
SOURCE_FLAGS = {"render.cu": ["-fmad=false"]}


def nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand) and shutil.which(cand) is None:
        raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build libdexmpm.so")
    return cand


def _flags(extra=()):
    return [ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
            "-I", os.path.join(HERE, "..", "include"), *extra]


def build(verbose: bool = False, extra_flags=()) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = os.path.join(OUT_DIR, "obj")
    os.makedirs(tmp, exist_ok=True)
    cc = nvcc()
    objs, cmds = [], []
    for src in SOURCES:
        obj = os.path.join(tmp, src.replace(".cu", ".o"))
        objs.append(obj)
        cmds.append([cc, *_flags(extra_flags), *SOURCE_FLAGS.get(src, []), "-c", os.path.join(CSRC, src), "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=len(cmds)) as ex:
        for cmd, res in zip(cmds, ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), cmds)):
            if res.returncode != 0:
                raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
            if verbose and (res.stdout or res.stderr):
                print(res.stdout, res.stderr, file=sys.stderr)
    link = [cc, ARCH, "-shared", "-o", LIB + ".tmp", *objs]
    res = subprocess.run(link, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(link)}\n{res.stdout}\n{res.stderr}")
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
