"""LAP's own C sources link against libgblap.so as INTEGRATION.md's link line
says: the driver and solver layer of LAP's CUDA build (cg_driver2.c, cg.c,
prec.c, GS.c, it_jacobi.c, line_jacobi.c, io_utils.c, compiled with
-DCUDA=1 exactly as MakefileCUDA:5-20 configures them), with libgblap in
place of blas.o, cuda_blas.o, devMem.o, -lcublas and -lcusparse.

Runs where LAP's sources are mounted ($LAP_REFERENCE_DIR); nothing is
copied out of them.  No GPU is needed: the test checks that the link
resolves and that every symbol those objects need is either libc/libm's or
exported by libgblap.
"""
import os
import shutil
import subprocess

import pytest

import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_DIR = os.path.join(ROOT, "lap_gb300")
LAP_SOURCES = ["cg_driver2", "cg", "prec", "GS", "it_jacobi", "line_jacobi", "io_utils"]
# MakefileCUDA's configuration flags
CONF = ["-DV100=0", "-DNOACC=0", "-DCUDA=1", "-DOPENMP=0", "-DHIP=0"]
# what the C runtime provides to these objects
LIBC = {"__isoc99_sscanf", "__printf_chk", "__stack_chk_fail", "calloc", "fclose", "fgets", "fopen", "free",
        "gettimeofday", "malloc", "printf", "puts", "qsort", "sqrt", "srand", "rand", "strcmp", "strstr",
        "strtod", "strtol", "sscanf", "fprintf", "memcpy", "memset", "putchar", "exit", "fwrite", "fputs",
        "stderr", "stdout", "realloc", "atoi", "atof", "strlen", "strcpy", "strncpy", "fscanf", "__fprintf_chk",
        "__isoc99_fscanf", "__memcpy_chk", "__sprintf_chk", "sprintf", "fabs", "pow"}


def _exported(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True, check=True).stdout
    return {ln.split()[-1] for ln in out.splitlines() if ln.strip()}


@pytest.mark.skipif(oracle.reference_dir() is None, reason="LAP sources not mounted")
@pytest.mark.skipif(shutil.which("gcc") is None or shutil.which("nm") is None, reason="needs gcc and nm")
def test_lap_cuda_build_links_against_libgblap(tmp_path):
    lib = os.path.join(LIB_DIR, "libgblap.so")
    if not os.path.exists(lib):
        pytest.skip("libgblap.so not built")
    ref = oracle.reference_dir()
    objs = []
    for name in LAP_SOURCES:
        obj = str(tmp_path / f"{name}.o")
        subprocess.run(["gcc", "-O2", *CONF, "-I" + ref, "-c", os.path.join(ref, name + ".c"), "-o", obj],
                       check=True, capture_output=True)
        objs.append(obj)
    undef = set()
    for obj in objs:
        out = subprocess.run(["nm", "-u", obj], capture_output=True, text=True, check=True).stdout
        undef |= {ln.split()[-1] for ln in out.splitlines() if ln.strip()}
    defined = set()
    for obj in objs:
        out = subprocess.run(["nm", "--defined-only", obj], capture_output=True, text=True, check=True).stdout
        defined |= {ln.split()[-1] for ln in out.splitlines() if ln.strip()}
    exported = _exported(lib)
    missing = sorted(s for s in undef - defined - LIBC if s not in exported)
    assert not missing, f"LAP symbols libgblap does not export: {missing}"
    # the backend calls LAP's CUDA build makes all resolve to libgblap
    for sym in ("dot", "axpy", "csr_matvec", "lower_triangular_solve", "upper_triangular_solve", "ichol",
                "initialize_handles", "initialize_spmv_buffer", "initialize_and_analyze_L_and_U_solve",
                "initialize_L_and_U_descriptors", "initialize_ichol", "mallocForDevice", "memcpyDevice",
                "freeDevice"):
        assert sym in undef - defined and sym in exported, sym
    exe = str(tmp_path / "lap_gb300_cg")
    r = subprocess.run(["gcc", "-o", exe, *objs, "-L" + LIB_DIR, "-Wl,-rpath," + LIB_DIR, "-lgblap", "-lm"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert os.path.getsize(exe) > 0
