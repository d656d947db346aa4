"""Pins the CPU oracle (oracle/oracle.c) to fixtures produced by the reference.

Every expected array comes from tests/golden/golden.npz, written by
tests/golden/make_golden.py through the reference's own compiled functions.
The oracle keeps the reference's operation order, so these comparisons are
bit-exact (array_equal), not tolerance checks.
"""
import ctypes as C
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN_CASES, GOLDEN_PRECS, ROOT, golden_matrix
from lap_gb300 import gen


def test_kat_spmv_fixture(golden):
    # test_spmv_omp.c:14-21, alpha=-2, beta=1.5, y0=1
    a = np.array([1.0, 2.0, 3.0, 7.0, 4.0, 1.0, 2.0, 3.0, 1.0, 9.0])
    ja = np.array([0, 1, 2, 1, 2, 3, 4, 3, 4, 4], dtype=np.int32)
    ia = np.array([0, 3, 4, 7, 9, 10], dtype=np.int32)
    y = oracle.csr_matvec(5, ia, ja, a, np.arange(1.0, 6.0), np.ones(5), -2.0, 1.5)
    assert np.array_equal(y, [-26.5, -26.5, -50.5, -32.5, -88.5])
    assert np.array_equal(y, golden["kat_spmv_y"])


def test_kat_trisolve_fixture(golden):
    # test_tri_solve_omp.c:17-21: strict upper CSR + separate diagonal, x = 8
    ua = np.array([2.0, 3.0, 1.0, 2.0, 1.0])
    uja = np.array([1, 2, 3, 4, 4], dtype=np.int32)
    uia = np.array([0, 2, 2, 4, 5, 5], dtype=np.int32)
    d = np.array([1.0, 7.0, 4.0, 3.0, 9.0])
    x = oracle.upper_solve(5, uia, uja, ua, d, np.full(5, 8.0))
    assert np.array_equal(x, golden["kat_trisolve_x"])
    np.testing.assert_allclose(x, [2.8253968253968254, 1.1428571428571428, 0.9629629629629629,
                                   2.3703703703703702, 0.8888888888888888], rtol=1e-15)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_spmv_bit_exact(golden, name):
    n, ia, ja, a, _ = golden_matrix(golden, name)
    xs, y0 = golden[f"{name}_spmv_x"], golden[f"{name}_spmv_y0"]
    for tag, (al, be) in {"spmv": (1.0, 0.0), "spmv_ab": (-1.0, 1.0), "spmv_odd": (0.37, -2.5)}.items():
        y = oracle.csr_matvec(n, ia, ja, a, xs, y0.copy(), al, be)
        assert np.array_equal(y, golden[f"{name}_{tag}_y"]), tag


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_triangular_solves_bit_exact(golden, name):
    n, ia, ja, a, _ = golden_matrix(golden, name)
    (lia, lja, la), (uia, uja, ua), d = oracle.split(n, ia, ja, a)
    xs = golden[f"{name}_spmv_x"]
    assert np.array_equal(oracle.lower_solve(n, lia, lja, la, d, xs), golden[f"{name}_lsolve"])
    assert np.array_equal(oracle.upper_solve(n, uia, uja, ua, d, xs), golden[f"{name}_usolve"])


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_ichol_factor_bit_exact(golden, name):
    n, ia, ja, a, _ = golden_matrix(golden, name)
    (lia, lja, la), (uia, uja, ua) = oracle.ichol_factor(n, ia, ja, a)
    assert np.array_equal(la, golden[f"{name}_ichol_L"])
    assert np.array_equal(ua, golden[f"{name}_ichol_U"])


@pytest.mark.parametrize("prec", GOLDEN_PRECS)
@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_pcg_bit_exact(golden, name, prec):
    n, ia, ja, a, b = golden_matrix(golden, name)
    it, flag, M, K, maxit = (int(v) for v in golden[f"{name}_{prec}_it"])
    tol = float(golden[f"{name}_{prec}_tol"][0])
    r = oracle.solve(n, ia, ja, a, b, prec, tol, maxit, M, K)
    assert r["iters"] == it and r["flag"] == flag
    assert np.array_equal(r["res_hist"], golden[f"{name}_{prec}_hist"])
    assert np.array_equal(r["x"], golden[f"{name}_{prec}_x"])


def test_mm_reader_matches_reference(golden):
    L = oracle.lib()
    path = os.path.join(ROOT, "tests", "golden", "grid6.mtx").encode()

    class MM(C.Structure):
        _fields_ = [("n", C.c_int), ("m", C.c_int), ("nnz", C.c_int), ("nnz_unpacked", C.c_int),
                    ("symmetric", C.c_int), ("coo_rows", C.POINTER(C.c_int)),
                    ("coo_cols", C.POINTER(C.c_int)), ("coo_vals", C.POINTER(C.c_double)),
                    ("csr_ia", C.POINTER(C.c_int)), ("csr_ja", C.POINTER(C.c_int)),
                    ("csr_vals", C.POINTER(C.c_double))]

    mm = MM()
    assert L.orc_read_mm(path, C.byref(mm)) == 0
    L.orc_coo_to_csr(C.byref(mm))
    n, nnz = mm.n, mm.nnz_unpacked
    assert np.array_equal(np.ctypeslib.as_array(mm.csr_ia, (n + 1,)), golden["mm_ia"])
    assert np.array_equal(np.ctypeslib.as_array(mm.csr_ja, (nnz,)), golden["mm_ja"])
    assert np.array_equal(np.ctypeslib.as_array(mm.csr_vals, (nnz,)), golden["mm_a"])
    # the generator wrote the same matrix it returns
    A6, _ = gen.grid2d_unit(6, seed=1001)
    assert np.array_equal(A6.ia, golden["mm_ia"]) and np.array_equal(A6.a, golden["mm_a"])
    L.orc_free_matrix(C.byref(mm))


def test_reference_library_agrees_when_built(golden):
    """Cross-check against the live reference build where it exists."""
    R = oracle.ref_lib()
    if R is None:
        pytest.skip("oracle/_ref/libref.so not built here")
    A, b = gen.grid2d_unit(20, seed=5)
    for prec in ("line_jacobi", "GS_std", "ichol"):
        r0 = oracle.ref_solve(A.n, A.ia, A.ja, A.a, b, prec, 1e-9, 3000)
        r1 = oracle.solve(A.n, A.ia, A.ja, A.a, b, prec, 1e-9, 3000)
        assert r0["iters"] == r1["iters"]
        assert np.array_equal(r0["x"], r1["x"])


# ---------------------------------------------------------------- Matrix Market
def test_mm_csr_oracle_matches_reference_fixture(golden):
    """oracle.mm_csr (read_mm_file + coo_to_csr restated) against the CSR the
    reference's own reader produced for grid6.mtx."""
    with open(os.path.join(ROOT, "tests", "golden", "grid6.mtx"), "rb") as f:
        n, m, sym, ia, ja, a = oracle.mm_csr(f.read())
    assert (n, m, sym) == (36, 36, True)
    assert np.array_equal(ia, golden["mm_ia"]) and np.array_equal(ja, golden["mm_ja"])
    assert np.array_equal(a.view(np.int64), golden["mm_a"].view(np.int64))


@pytest.mark.parametrize("kind", ["general", "symmetric", "pattern"])
def test_mm_csr_oracle_matches_reference_reader(kind, tmp_path):
    """The same against the reference's compiled reader on harder texts:
    duplicates, CRLF ends, tabs, every value spelling of tests/mm_cases.py
    (skipped where the reference was not compiled)."""
    import mm_cases

    L = oracle.ref_lib()
    if L is None:
        pytest.skip("reference library not built here")
    text = {"general": mm_cases.general_text, "symmetric": mm_cases.symmetric_text,
            "pattern": mm_cases.pattern_text}[kind]()
    p = tmp_path / f"{kind}.mtx"
    p.write_text(text)
    L.ref_read_mm_csr.argtypes = [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                  C.POINTER(C.POINTER(C.c_int)), C.POINTER(C.POINTER(C.c_int)),
                                  C.POINTER(C.POINTER(C.c_double))]
    n, nnz = C.c_int(), C.c_int()
    pia, pja, pa = C.POINTER(C.c_int)(), C.POINTER(C.c_int)(), C.POINTER(C.c_double)()
    L.ref_read_mm_csr(str(p).encode(), C.byref(n), C.byref(nnz), C.byref(pia), C.byref(pja), C.byref(pa))
    ia = np.ctypeslib.as_array(pia, (n.value + 1,)).copy()
    ja = np.ctypeslib.as_array(pja, (nnz.value,)).copy()
    a = np.ctypeslib.as_array(pa, (nnz.value,)).copy()
    _, _, _, oia, oja, oa = oracle.mm_csr(text.encode())
    assert np.array_equal(ia, oia) and np.array_equal(ja, oja)
    assert np.array_equal(a.view(np.int64), oa.view(np.int64))


def test_laplacian_oracle_matches_reference_fixture(golden):
    with open(os.path.join(ROOT, "tests", "golden", "adj5.mtx"), "rb") as f:
        n, ia, ja, a = oracle.laplacian_csr(f.read(), weighted=0)
    assert np.array_equal(ia, golden["adj_ia"]) and np.array_equal(ja, golden["adj_ja"])
    assert np.array_equal(a, golden["adj_a"])


def _random_adjacency(tmp_path, weights, seed=5, n=200, m=800):
    rng = np.random.default_rng(seed)
    ei, ej = rng.integers(0, n, m), rng.integers(0, n, m)
    keep = ei != ej
    ei, ej = ei[keep], ej[keep]
    w = rng.uniform(0.1, 3.0, ei.shape[0]) if weights else None
    p = tmp_path / f"adj_{int(weights)}.mtx"
    gen.write_adjacency(str(p), n, ei, ej, w)
    return p


@pytest.mark.parametrize("weights", [False, True])
@pytest.mark.parametrize("weighted", [0, 1])
def test_laplacian_oracle_matches_reference_builder(tmp_path, weights, weighted):
    """oracle.laplacian_csr against the reference's read_adjacency_file +
    coo_to_csr + create_L_and_split on random graphs with repeated edges;
    non-integer weights exercise its int degree truncation."""
    L = oracle.ref_lib()
    if L is None:
        pytest.skip("reference library not built here")
    p = _random_adjacency(tmp_path, weights)
    L.ref_read_laplacian_csr.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                         C.POINTER(C.POINTER(C.c_int)), C.POINTER(C.POINTER(C.c_int)),
                                         C.POINTER(C.POINTER(C.c_double))]
    n, nnz = C.c_int(), C.c_int()
    pia, pja, pa = C.POINTER(C.c_int)(), C.POINTER(C.c_int)(), C.POINTER(C.c_double)()
    L.ref_read_laplacian_csr(str(p).encode(), weighted, C.byref(n), C.byref(nnz), C.byref(pia), C.byref(pja),
                             C.byref(pa))
    ia = np.ctypeslib.as_array(pia, (n.value + 1,)).copy()
    ja = np.ctypeslib.as_array(pja, (nnz.value,)).copy()
    a = np.ctypeslib.as_array(pa, (nnz.value,)).copy()
    _, oia, oja, oa = oracle.laplacian_csr(p.read_bytes(), weighted)
    assert np.array_equal(ia, oia) and np.array_equal(ja, oja)
    assert np.array_equal(a.view(np.int64), oa.view(np.int64))
