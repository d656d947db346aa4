"""LAP's own solver entry points (cg, the initialize_* setup calls, the
triangular solves) used the way LAP's CUDA driver uses them, against the
reference's CPU PCG (the oracle).

* cg() applies the preconditioner data the caller's pdata holds (d_r,
  la / ua, ichol_vals), as prec_function does (prec.c:6-45), and re-reads
  A's values on every call: changing a in place (and, as LAP's driver would,
  the pdata arrays) between two calls gives the new system's solution.
* Analyses cached by array address are revalidated by the pattern's
  fingerprint: a factor rewritten at the same address with another pattern
  is solved with its own schedule.
* The setup calls in cg_driver2.c's order (:211, :278-286, :316-349).
"""
import ctypes as C

import numpy as np
import pytest

from conftest import golden_matrix

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a GPU", allow_module_level=True)

import lap_gb300 as gb  # noqa: E402
import oracle  # noqa: E402
from lap_gb300 import gen  # noqa: E402
from test_gpu_pcg import _pdata_gpu_convention, iters_ok  # noqa: E402

X_TOL = 1e-6


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _cg(n, nnz, dia, dja, da, db, p, tol, maxit):
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    hist = np.zeros(maxit + 3)
    it, flag = C.c_int(), C.c_int()
    torch.cuda.synchronize()
    gb.lib().cg(n, float(nnz), gb.ptr(dia), gb.ptr(dja), gb.ptr(da), gb.ptr(x), gb.ptr(db), tol, C.byref(p),
                maxit, C.byref(it), C.byref(flag), hist.ctypes.data)
    torch.cuda.synchronize()
    return x.cpu().numpy(), it.value, flag.value


def _write_pdata_values(A, prec, keep, p):
    """Rewrites the pdata arrays' values in place for A (same layout), as a
    driver re-running its setup for a new matrix would."""
    fresh = {}
    q = _pdata_gpu_convention(A, prec, fresh)
    for k in ("la", "ua", "d", "dr"):
        keep[k].copy_(fresh[k])
    return q


@pytest.mark.parametrize("prec", ["ichol", "GS_std", "line_jacobi", "it_jacobi"])
def test_cg_rereads_values_and_applies_pdata(prec):
    A1, b = gen.grid3d_lognormal(14, seed=501)
    A2, _ = gen.grid3d_lognormal(14, seed=502)  # same pattern, other weights
    assert np.array_equal(A1.ia, A2.ia) and np.array_equal(A1.ja, A2.ja)
    n, nnz, tol, maxit = A1.n, A1.nnz, 1e-10, 5000
    keep = {}
    p = _pdata_gpu_convention(A1, prec, keep)
    dia, dja, da, db = dev(A1.ia), dev(A1.ja), dev(A1.a), dev(b)
    L = gb.lib()
    iv = None
    if prec == "ichol":
        iv = dev(A1.a.copy())
        L.initialize_ichol(n, nnz, gb.ptr(dia), gb.ptr(dja), gb.ptr(iv))
        p.ichol_vals = gb.ptr(iv)
    for A in (A1, A2):
        if A is A2:  # the same device buffers, new values
            da.copy_(dev(A2.a))
            _write_pdata_values(A2, prec, keep, p)
            if iv is not None:
                iv.copy_(dev(A2.a))
                L.initialize_ichol(n, nnz, gb.ptr(dia), gb.ptr(dja), gb.ptr(iv))
        ref = oracle.solve(n, A.ia, A.ja, A.a, b, prec, tol, maxit)
        x, it, flag = _cg(n, nnz, dia, dja, da, db, p, tol, maxit)
        assert flag == 0 and iters_ok(it, ref["iters"], prec), (it, ref["iters"])
        assert np.linalg.norm(x - ref["x"]) / np.linalg.norm(ref["x"]) < X_TOL


def test_cg_uses_the_callers_ichol_factor():
    """cg() applies pdata->ichol_vals, not a factor of its own: handing it
    the IC(0) factor of another matrix (same pattern) changes the iterates,
    while the solution still solves A -- and handing back A's own factor
    restores the reference's iteration count."""
    A1, b = gen.grid3d_lognormal(14, seed=503)
    A2, _ = gen.grid3d_lognormal(14, seed=504)
    n, nnz, tol, maxit = A1.n, A1.nnz, 1e-10, 5000
    keep = {}
    p = _pdata_gpu_convention(A1, "ichol", keep)
    dia, dja, da, db = dev(A1.ia), dev(A1.ja), dev(A1.a), dev(b)
    L = gb.lib()
    iv = dev(A2.a.copy())  # the factor of A2, applied while solving A1
    L.initialize_ichol(n, nnz, gb.ptr(dia), gb.ptr(dja), gb.ptr(iv))
    p.ichol_vals = gb.ptr(iv)
    ref = oracle.solve(n, A1.ia, A1.ja, A1.a, b, "ichol", tol, maxit)
    x, it_other, flag = _cg(n, nnz, dia, dja, da, db, p, tol, maxit)
    assert flag == 0
    assert np.linalg.norm(x - ref["x"]) / np.linalg.norm(ref["x"]) < X_TOL  # still A1's solution
    assert it_other != ref["iters"]  # ... reached with the other preconditioner
    iv.copy_(da)
    L.initialize_ichol(n, nnz, gb.ptr(dia), gb.ptr(dja), gb.ptr(iv))
    x, it, flag = _cg(n, nnz, dia, dja, da, db, p, tol, maxit)
    assert flag == 0 and iters_ok(it, ref["iters"], "ichol")


def test_cg_rejects_pdata_that_does_not_match_a(capfd):
    A, b = gen.grid3d_lognormal(10, seed=505)
    keep = {}
    p = _pdata_gpu_convention(A, "GS_std", keep)
    p.lnnz = p.lnnz - 1  # not the layout LAP's driver builds from this A
    dia, dja, da, db = dev(A.ia), dev(A.ja), dev(A.a), dev(b)
    x, it, flag = _cg(A.n, A.nnz, dia, dja, da, db, p, 1e-8, 100)
    assert flag == 2 and it == 0
    assert "does not match A" in capfd.readouterr().err


def _lower_embedded(A):
    Lp, Up, d = oracle.split(A.n, A.ia, A.ja, A.a)
    return oracle.embed_diagonal(A.n, Lp, Up, d)[0]


def test_tri_solve_new_pattern_at_same_address(golden):
    """cuda_lower_triangular_solve caches its schedule per factor address;
    a factor rewritten in place with another pattern (same n, same nnz)
    must be solved with the new pattern's schedule, bit-exact."""
    n, ia, ja, a, b = golden_matrix(golden, "grid2d")
    lia, lja, la = _lower_embedded(gen.CSR(n, ia, ja, a))
    # another lower pattern with the same nnz: in the last row, move its
    # first off-diagonal entry to a column that row does not have
    r = n - 1
    cols = set(lja[lia[r]:lia[r + 1]].tolist())
    new_c = next(c for c in range(r) if c not in cols)
    lja2, la2 = lja.copy(), la.copy()
    seg = slice(lia[r], lia[r + 1] - 1)  # off-diagonal part of row r (diagonal last)
    row_cols = sorted(list(lja[seg][1:]) + [new_c])
    lja2[seg] = row_cols
    la2[seg] = -0.25
    x = np.random.default_rng(7).standard_normal(n)
    L = gb.lib()
    dlia, dlja, dla = dev(lia), dev(lja), dev(la)
    dx, y = dev(x), torch.zeros(n, dtype=torch.float64, device="cuda")
    for cj, cv in ((lja, la), (lja2, la2), (lja, la)):
        dlja.copy_(dev(cj))
        dla.copy_(dev(cv))
        L.cuda_lower_triangular_solve(n, len(cj), gb.ptr(dlia), gb.ptr(dlja), gb.ptr(dla), 0, gb.ptr(dx), gb.ptr(y))
        torch.cuda.synchronize()
        # the oracle's strict-lower + diagonal form of the same factor
        rows = np.repeat(np.arange(n), np.diff(lia))
        off = cj != rows
        sl = np.zeros(n + 1, dtype=np.int32)
        np.cumsum(np.bincount(rows[off], minlength=n), out=sl[1:])
        want = oracle.lower_solve(n, sl, np.ascontiguousarray(cj[off], dtype=np.int32),
                                  np.ascontiguousarray(cv[off]), np.ascontiguousarray(cv[~off]), x)
        assert np.array_equal(y.cpu().numpy(), want)


@pytest.mark.parametrize("prec", ["GS_std", "ichol"])
def test_driver_setup_sequence_then_cg(golden, prec):
    """initialize_handles, initialize_spmv_buffer, initialize_and_analyze_L_and_U_solve
    (GS_std), initialize_ichol (ichol) and initialize_L_and_U_descriptors in
    cg_driver2.c's order, then cg(): the reference's iterations and x."""
    n, ia, ja, a, b = golden_matrix(golden, "grid3d")
    it_ref, flag_ref, M, K, maxit = (int(v) for v in golden[f"grid3d_{prec}_it"])
    tol = float(golden[f"grid3d_{prec}_tol"][0])
    A = gen.CSR(n, ia, ja, a)
    L = gb.lib()
    keep = {}
    L.initialize_handles()
    p = _pdata_gpu_convention(A, prec, keep)
    p.k = K
    dia, dja, da, db = dev(ia), dev(ja), dev(a), dev(b)
    x0 = torch.zeros(n, dtype=torch.float64, device="cuda")
    one, minusone = C.c_double(1.0), C.c_double(1.0)  # cg_driver2.c:272 passes 1.0 for both
    L.initialize_spmv_buffer(n, len(ja), gb.ptr(dia), gb.ptr(dja), gb.ptr(da), gb.ptr(x0), gb.ptr(db),
                             C.byref(one), C.byref(minusone))
    if prec == "GS_std":
        L.initialize_and_analyze_L_and_U_solve(n, p.lnnz, p.lia, p.lja, p.la, p.unnz, p.uia, p.uja, p.ua)
    if prec == "ichol":
        iv = dev(a.copy())
        keep["iv"] = iv
        L.initialize_ichol(n, len(ja), gb.ptr(dia), gb.ptr(dja), gb.ptr(iv))
        p.ichol_vals = gb.ptr(iv)
    L.initialize_L_and_U_descriptors(n, p.lnnz, p.lia, p.lja, p.la, p.unnz, p.uia, p.uja, p.ua)
    torch.cuda.synchronize()
    assert np.array_equal(db.cpu().numpy(), b)  # the SpMV-buffer setup leaves b alone
    x, it, flag = _cg(n, len(ja), dia, dja, da, db, p, tol, maxit)
    assert flag == 0 and iters_ok(it, it_ref, prec), (it, it_ref)
    xref = golden[f"grid3d_{prec}_x"]
    assert np.linalg.norm(x - xref) / np.linalg.norm(xref) < X_TOL
