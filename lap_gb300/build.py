"""Builds lap_gb300/libgblap.so in-tree with nvcc for sm_103a only.

    python -m lap_gb300.build [--jobs N] [--debug]

Each translation unit is compiled in parallel (one -gencode, -lineinfo),
then linked into one shared library with the CUDA runtime linked
statically, so the library has no dependency beyond the driver.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgblap.so")

SOURCES = ["kernels.cu", "sptrsv.cu", "tri_plan.cu", "pcg.cu", "precond.cu", "system.cu", "lap_abi.cu",
           "lap_host.cu", "extras.cu", "batch.cu", "noalloc.cu", "mmio.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found")
    return path


def flags(debug: bool = False) -> list[str]:
    f = ARCH + ["-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + os.path.join(ROOT, "include"),
                "-I" + CSRC]
    f += ["-O0", "-G"] if debug else ["-O3"]
    return f


def _compile(src: str, debug: bool) -> str:
    obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
    deps = [os.path.join(CSRC, s) for s in os.listdir(CSRC)] + \
        [os.path.join(ROOT, "include", h) for h in os.listdir(os.path.join(ROOT, "include"))]
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc()] + flags(debug) + ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(jobs: int | None = None, debug: bool = False, quiet: bool = True) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, debug), srcs))
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    _build_driver(LIB)
    if not quiet:
        print("built", LIB)
    return LIB


DRIVER_SRC = os.path.join(CSRC, "lap_mm_driver.c")
DRIVER = os.path.join(HERE, "lap_mm_driver")


def _build_driver(lib: str) -> None:
    """LAP's SpMV benchmark program (mm_driver.c) on the library: a plain C
    host program linked against libgblap.so (found next to it at run time)."""
    if os.path.exists(DRIVER) and os.path.getmtime(DRIVER) >= max(os.path.getmtime(lib),
                                                                   os.path.getmtime(DRIVER_SRC)):
        return
    cc = shutil.which("gcc") or shutil.which("cc")
    cmd = [cc, "-O2", "-std=c11", "-I" + os.path.join(ROOT, "include"), DRIVER_SRC, "-L" + HERE, "-lgblap",
           "-Wl,-rpath,$ORIGIN", "-lm", "-o", DRIVER]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"driver build failed:\n{r.stdout}\n{r.stderr}")


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--jobs", type=int, default=None)
    ap.add_argument("--debug", action="store_true")
    a = ap.parse_args()
    try:
        build(a.jobs, a.debug, quiet=False)
    except RuntimeError as e:
        print(e, file=sys.stderr)
        sys.exit(1)
