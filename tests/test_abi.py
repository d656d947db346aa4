"""CPU-side checks of the C-ABI library: it loads without a GPU, exports every
symbol the public headers declare, and its host-only LAP functions (Matrix
Market I/O, splitting, Laplacian construction) reproduce the reference's
results on the golden files."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT

import lap_gb300 as gb


@pytest.fixture(scope="module")
def L():
    if not os.path.exists(gb.LIB_PATH):
        from lap_gb300 import build

        build.build()
    return gb.lib()


def declared_functions():
    names = []
    for h in ("gblap.h", "lap_gblap.h"):
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b([A-Za-z_]\w*)\s*\(", src, flags=re.M):
            name = m.group(1)
            if name not in ("if", "typedef", "struct"):
                names.append(name)
    return sorted(set(names))


def test_exports_every_declared_symbol(L):
    names = declared_functions()
    assert len(names) > 60
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_status_and_names(L):
    assert L.gb_status_str(0) == b"ok"
    assert L.gb_prec_from_name(b"ichol") == 6
    assert L.gb_prec_from_name(b"GS_std") == 3
    assert L.gb_prec_from_name(b"bogus") == -1
    assert b"sm_103a" in L.gb_version()


def _csr(mm):
    n, nnz = mm.n, mm.nnz_unpacked
    return (np.ctypeslib.as_array(mm.csr_ia, (n + 1,)).copy(),
            np.ctypeslib.as_array(mm.csr_ja, (nnz,)).copy(),
            np.ctypeslib.as_array(mm.csr_vals, (nnz,)).copy())


def test_read_mm_file_matches_reference(L, golden):
    A = gb.MMatrix()
    L.read_mm_file(os.path.join(ROOT, "tests", "golden", "grid6.mtx").encode(), C.byref(A))
    assert A.symmetric == 1 and A.n == 36
    L.coo_to_csr(C.byref(A))
    ia, ja, a = _csr(A)
    assert np.array_equal(ia, golden["mm_ia"]) and np.array_equal(ja, golden["mm_ja"])
    assert np.array_equal(a, golden["mm_a"])
    Lm, Um, Dm = gb.MMatrix(), gb.MMatrix(), gb.MMatrix()
    L.split(C.byref(A), C.byref(Lm), C.byref(Um), C.byref(Dm))
    import oracle

    (lia, lja, la), (uia, uja, ua), d = oracle.split(36, ia, ja, a)
    assert np.array_equal(_csr(Lm)[0], lia) and np.array_equal(_csr(Lm)[2], la)
    assert np.array_equal(_csr(Um)[1], uja) and np.array_equal(_csr(Um)[2], ua)
    assert np.array_equal(np.ctypeslib.as_array(Dm.csr_vals, (36,)), d)


def test_laplacian_from_adjacency_matches_reference(L, golden):
    A = gb.MMatrix()
    L.read_adjacency_file(os.path.join(ROOT, "tests", "golden", "adj5.mtx").encode(), C.byref(A))
    L.coo_to_csr(C.byref(A))
    Lm, Um, Dm = gb.MMatrix(), gb.MMatrix(), gb.MMatrix()
    L.create_L_and_split(C.byref(A), C.byref(Lm), C.byref(Um), C.byref(Dm), 0)
    ia, ja, a = _csr(A)
    assert np.array_equal(ia, golden["adj_ia"]) and np.array_equal(ja, golden["adj_ja"])
    assert np.array_equal(a, golden["adj_a"])


def test_read_rhs(L):
    out = np.zeros(36)
    L.read_rhs(os.path.join(ROOT, "tests", "golden", "rhs6.mtx").encode(), out.ctypes.data)
    want = np.random.default_rng(3).uniform(-1, 1, 36)
    np.testing.assert_allclose(out, want, rtol=1e-16)


def test_missing_file_is_reported_not_crashing(L, capfd):
    A = gb.MMatrix()
    L.read_mm_file(b"/nonexistent/file.mtx", C.byref(A))
    assert A.n == 0
    assert "cannot open" in capfd.readouterr().err
