"""Regenerates the golden fixtures in this folder FROM THE REFERENCE ITSELF.

Needs the LAP sources ($LAP_REFERENCE_DIR, default /root/reference) so that ``oracle/Makefile``
can compile the reference's NOACC objects into ``oracle/_ref/libref.so``;
every output array below is produced by the reference's own functions
(cg(), simple_csr_matvec(), simple_*_triangular_solve(), initialize_ichol(),
read_mm_file()+coo_to_csr(), create_L_and_split()).  The inputs are the
seeded generators of ``lap_gb300.gen`` at small sizes.

    python tests/golden/make_golden.py [--ref-dir /path/to/LAP]

Outputs (committed): ``golden.npz`` and the small Matrix Market files the
I/O fixtures were read from.
"""
from __future__ import annotations

import argparse
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from lap_gb300 import gen  # noqa: E402

# (name, prec, M, K, tol, maxit)
PRECS = [("line_jacobi", 1, 1, 1e-10, 2000), ("GS_std", 1, 1, 1e-10, 2000),
         ("ichol", 1, 1, 1e-10, 2000), ("it_jacobi", 1, 2, 1e-10, 2000),
         ("GS_it", 1, 1, 1e-8, 60), ("GS_it2", 1, 1, 1e-10, 400), ("none", 1, 1, 1e-10, 2000)]


def small_cases():
    A1, b1 = gen.grid2d_unit(16, seed=1001)
    A2, b2 = gen.grid3d_lognormal(8, seed=1002)
    A3, b3 = gen.chung_lu(1500, seed=1003)
    A4 = gen.knn_graph(400, seed=1004)
    b4 = np.random.default_rng(1004).uniform(-1, 1, A4.n)
    A5, b5, _ = gen.grid2d_aniso(24, seed=1006)
    return {"grid2d": (A1, b1), "grid3d": (A2, b2), "chunglu": (A3, b3), "knn": (A4, b4),
            "aniso": (A5, b5)}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-dir", default=os.environ.get("LAP_REFERENCE_DIR", "/root/reference"))
    args = ap.parse_args()
    oracle.build(args.ref_dir)
    R = oracle.ref_lib()
    assert R is not None, "reference library did not build"
    out: dict[str, np.ndarray] = {}

    # --- test_spmv_omp.c:14-21 fixture through the reference's simple_csr_matvec
    a = np.array([1.0, 2.0, 3.0, 7.0, 4.0, 1.0, 2.0, 3.0, 1.0, 9.0])
    ja = np.array([0, 1, 2, 1, 2, 3, 4, 3, 4, 4], dtype=np.int32)
    ia = np.array([0, 3, 4, 7, 9, 10], dtype=np.int32)
    x = np.array([1.0, 2.0, 3.0, 4.0, 5.0])
    y = np.ones(5)
    R.simple_csr_matvec(5, 10, ia, ja, a, x, y, C.byref(C.c_double(-2.0)), C.byref(C.c_double(1.5)))
    out["kat_spmv_y"] = y

    # --- test_tri_solve_omp.c:17-21 fixture through simple_upper_triangular_solve
    ua = np.array([2.0, 3.0, 1.0, 2.0, 1.0])
    uja = np.array([1, 2, 3, 4, 4], dtype=np.int32)
    uia = np.array([0, 2, 2, 4, 5, 5], dtype=np.int32)
    diag = np.array([1.0, 7.0, 4.0, 3.0, 9.0])
    res = np.zeros(5)
    R.simple_upper_triangular_solve(5, 5, uia, uja, ua, diag, np.full(5, 8.0), res)
    out["kat_trisolve_x"] = res

    for name, (A, b) in small_cases().items():
        out[f"{name}_ia"], out[f"{name}_ja"], out[f"{name}_a"], out[f"{name}_b"] = A.ia, A.ja, A.a, b
        rng = np.random.default_rng(7)
        xs = rng.uniform(-1, 1, A.n)
        ys = rng.uniform(-1, 1, A.n)
        for tag, (al, be) in {"spmv": (1.0, 0.0), "spmv_ab": (-1.0, 1.0), "spmv_odd": (0.37, -2.5)}.items():
            yy = ys.copy()
            R.simple_csr_matvec(A.n, A.nnz, A.ia, A.ja, A.a, xs, yy, C.byref(C.c_double(al)),
                                C.byref(C.c_double(be)))
            out[f"{name}_{tag}_y"] = yy
        out[f"{name}_spmv_x"], out[f"{name}_spmv_y0"] = xs, ys
        (lia, lja, la), (uia_, uja_, ua_), d = oracle.split(A.n, A.ia, A.ja, A.a)
        lo = np.zeros(A.n)
        up = np.zeros(A.n)
        R.simple_lower_triangular_solve(A.n, len(lja), lia, lja, la, d, xs, lo)
        R.simple_upper_triangular_solve(A.n, len(uja_), uia_, uja_, ua_, d, xs, up)
        out[f"{name}_lsolve"], out[f"{name}_usolve"] = lo, up

        for prec, M, K, tol, maxit in PRECS:
            hist = np.zeros(maxit + 3)
            xx = np.zeros(A.n)
            flag = C.c_int(0)
            nl = (A.nnz - A.n) // 2 + A.n
            lf = np.zeros(nl)
            uf = np.zeros(nl)
            it = R.ref_solve_csr(A.n, A.nnz, A.ia.copy(), A.ja.copy(), A.a.copy(), b.copy(), xx,
                                 prec.encode(), tol, maxit, M, K, C.byref(flag), hist,
                                 lf.ctypes.data_as(C.c_void_p), uf.ctypes.data_as(C.c_void_p))
            key = f"{name}_{prec}"
            out[f"{key}_x"] = xx
            out[f"{key}_it"] = np.array([it, flag.value, M, K, maxit], dtype=np.int64)
            out[f"{key}_tol"] = np.array([tol])
            out[f"{key}_hist"] = hist[: it + 1]
            if prec == "ichol":
                out[f"{name}_ichol_L"], out[f"{name}_ichol_U"] = lf, uf

    # --- Matrix Market reader fixtures: reference read_mm_file + coo_to_csr
    A, _ = gen.grid2d_unit(6, seed=1001)
    mm = os.path.join(HERE, "grid6.mtx")
    gen.write_mm(mm, A)
    n, nnz = C.c_int(), C.c_int()
    pia, pja, pa = C.POINTER(C.c_int)(), C.POINTER(C.c_int)(), C.POINTER(C.c_double)()
    R.ref_read_mm_csr(mm.encode(), C.byref(n), C.byref(nnz), C.byref(pia), C.byref(pja), C.byref(pa))
    out["mm_ia"] = np.ctypeslib.as_array(pia, (n.value + 1,)).copy()
    out["mm_ja"] = np.ctypeslib.as_array(pja, (nnz.value,)).copy()
    out["mm_a"] = np.ctypeslib.as_array(pa, (nnz.value,)).copy()
    # adjacency -> unweighted Laplacian (cg_driver.c path)
    idx = np.arange(25).reshape(5, 5)
    ei = np.concatenate([idx[:, :-1].ravel(), idx[:-1, :].ravel()])
    ej = np.concatenate([idx[:, 1:].ravel(), idx[1:, :].ravel()])
    adj = os.path.join(HERE, "adj5.mtx")
    gen.write_adjacency(adj, 25, ei, ej)
    R.ref_read_laplacian_csr(adj.encode(), 0, C.byref(n), C.byref(nnz), C.byref(pia), C.byref(pja),
                             C.byref(pa))
    out["adj_ia"] = np.ctypeslib.as_array(pia, (n.value + 1,)).copy()
    out["adj_ja"] = np.ctypeslib.as_array(pja, (nnz.value,)).copy()
    out["adj_a"] = np.ctypeslib.as_array(pa, (nnz.value,)).copy()
    rhs = os.path.join(HERE, "rhs6.mtx")
    gen.write_rhs(rhs, np.random.default_rng(3).uniform(-1, 1, 36))

    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    print("wrote", len(out), "arrays")

    # the reference's SpMV benchmark program (mm_driver.c) on grid6.mtx, 3 trials:
    # its report, against which the library's lap_mm_driver is compared
    import subprocess

    drv = os.path.join(ROOT, "oracle", "_ref", "mm_driver")
    rep = subprocess.run([drv, mm, "3"], capture_output=True, text=True, check=True).stdout
    with open(os.path.join(HERE, "mm_driver_grid6.txt"), "w") as f:
        f.write(rep)


if __name__ == "__main__":
    main()
