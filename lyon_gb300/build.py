"""Builds liblyon_gb300.so in-tree (lyon_gb300/_lib/) with nvcc for sm_103a.

Each .cu translation unit compiles in parallel with `--fmad=false` (lyon's arithmetic has no fused
multiply-add: positions must round exactly as lyon's f32 code does) and IEEE division/sqrt; the
objects are linked into one shared library whose C ABI is include/lyon_gpu.h.
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
BUILD_DIR = os.path.join(HERE, "_build")
LIB_NAME = "liblyon_gb300.so"
LIB_PATH = os.path.join(OUT_DIR, LIB_NAME)

SOURCES = ["stroke.cu", "stroke_seq.cu", "attributes.cu", "arcs.cu", "hatch.cu", "scan.cu", "flatten.cu", "fill.cu", "api.cu", "noalloc.cu", "serve.cu",
           "shapes.cu", "svg.cu", "coverage.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "--fmad=false", "-prec-div=true",
              "-prec-sqrt=true", "-Xcompiler", "-fPIC", "-Xcompiler", "-fno-fast-math",
              "-Xcompiler", "-ffp-contract=off"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps_mtime() -> float:
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(os.path.dirname(HERE), "include", "lyon_gpu.h"))
    return max(os.path.getmtime(f) for f in files if os.path.exists(f))


def up_to_date() -> bool:
    return os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= _deps_mtime()


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB_PATH
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(BUILD_DIR, exist_ok=True)
    cc = nvcc()
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]

    def compile_one(src):
        obj = os.path.join(BUILD_DIR, src.replace(".cu", ".o"))
        cmd = [cc, *NVCC_FLAGS, *ARCH, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB_PATH + ".tmp"
    cmd = [cc, "-shared", *ARCH, "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
