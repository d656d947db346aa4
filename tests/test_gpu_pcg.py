"""GPU parity of the device-resident PCG (gb_pcg_solve and LAP's cg()) against
the reference's own results (golden fixtures) and the CPU oracle.

Acceptance: relative residual <= tol, solution within 1e-6 relative of the
reference's, iteration count within +-2% for GS/IC0 and +-1 for the Jacobi
family.  Iterates are not bit-exact because dot products are reduced in a
different order than the reference's sequential loop.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import GOLDEN_CASES, golden_matrix

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a GPU", allow_module_level=True)

import lap_gb300 as gb  # noqa: E402
import oracle  # noqa: E402
from lap_gb300 import gen  # noqa: E402

X_TOL = 1e-6  # solution tolerance vs the reference (the acceptance bar)


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def iters_ok(got, want, prec):
    slack = 1 if prec in ("line_jacobi", "it_jacobi") else max(1, int(np.ceil(0.02 * want)))
    return abs(got - want) <= slack


@pytest.mark.parametrize("prec", ["line_jacobi", "GS_std", "ichol", "it_jacobi", "GS_it2", "none"])
@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_pcg_matches_reference(golden, name, prec):
    n, ia, ja, a, b = golden_matrix(golden, name)
    it, flag, M, K, maxit = (int(v) for v in golden[f"{name}_{prec}_it"])
    tol = float(golden[f"{name}_{prec}_tol"][0])
    xref = golden[f"{name}_{prec}_x"]
    sysm = gb.System(dev(ia), dev(ja), dev(a), prec, M, K)
    x, r, hist = sysm.solve(dev(b), tol=tol, maxit=maxit, hist_len=maxit + 2)
    assert r["flag"] == flag == 0
    assert iters_ok(r["iters"], it, prec), (r["iters"], it)
    xs = x.cpu().numpy()
    assert np.linalg.norm(xs - xref) / np.linalg.norm(xref) < X_TOL
    assert hist[0] == pytest.approx(golden[f"{name}_{prec}_hist"][0], rel=1e-12)
    assert r["res"] < tol * hist[0]
    sysm.close()


def test_gs_it_diverging_case_hits_maxit(golden):
    """GS_it with M=K=1 does not converge on these inputs in the reference either."""
    n, ia, ja, a, b = golden_matrix(golden, "grid2d")
    it, flag, M, K, maxit = (int(v) for v in golden["grid2d_GS_it_it"])
    sysm = gb.System(dev(ia), dev(ja), dev(a), "GS_it", M, K)
    x, r = sysm.solve(dev(b), tol=float(golden["grid2d_GS_it_tol"][0]), maxit=maxit)
    assert flag == 1 and r["flag"] == 1 and r["iters"] == it == maxit + 1
    sysm.close()


@pytest.mark.parametrize("prec", ["line_jacobi", "GS_std", "ichol"])
def test_graph_and_eager_agree(prec):
    A, b = gen.grid2d_unit(48, seed=11)
    sysm = gb.System.from_csr(A, prec)
    x1, r1 = sysm.solve(dev(b), tol=1e-9, maxit=3000, use_graph=True)
    x2, r2 = sysm.solve(dev(b), tol=1e-9, maxit=3000, use_graph=False)
    assert r1["iters"] == r2["iters"] and r1["flag"] == r2["flag"] == 0
    assert torch.equal(x1, x2)  # deterministic reductions: bitwise identical
    x3, r3 = sysm.solve(dev(b), tol=1e-9, maxit=3000)
    assert torch.equal(x1, x3)  # and run-to-run reproducible
    sysm.close()


@pytest.mark.parametrize("prec", ["line_jacobi", "ichol", "GS_std"])
def test_mixed_precision_error_vs_fp64_oracle(prec):
    A, b = gen.grid3d_lognormal(20, seed=1002)
    ref = oracle.solve(A.n, A.ia, A.ja, A.a, b, prec, 1e-13, 20000)
    sysm = gb.System.from_csr(A, prec)
    x, r = sysm.solve(dev(b), tol=1e-10, maxit=20000, precision=1)
    assert r["flag"] == 0 and r["outer"] >= 2
    assert r["rel_true_res"] < 1e-10 * 1.01
    err = np.linalg.norm(x.cpu().numpy() - ref["x"]) / np.linalg.norm(ref["x"])
    assert err < 1e-8, err
    sysm.close()


@pytest.mark.parametrize("prec", ["ichol", "GS_std"])
def test_split_precision_error_vs_fp64_oracle(prec):
    """precision=2: FP64 recurrence around the FP32 SpMV and FP32 triangular
    solves; at tol 1e-10 the error against the FP64 oracle stays at the FP64
    level (more iterations than FP64: each replacement cycle is limited by the
    FP32 operator's rounding)."""
    A, b = gen.grid3d_lognormal(20, seed=1002)
    ref = oracle.solve(A.n, A.ia, A.ja, A.a, b, prec, 1e-13, 20000)
    sysm = gb.System.from_csr(A, prec)
    x, r = sysm.solve(dev(b), tol=1e-10, maxit=20000, precision=2)
    assert r["flag"] == 0 and r["status"] == 0 and r["outer"] >= 1
    assert r["rel_true_res"] < 1e-10 * 1.01
    err = np.linalg.norm(x.cpu().numpy() - ref["x"]) / np.linalg.norm(ref["x"])
    assert err < 1e-8, err
    sysm.close()


@pytest.mark.parametrize("prec", ["ichol", "GS_std"])
def test_split_precision_iterations_at_1e8(prec):
    """At tol 1e-8 the split recurrence needs as many iterations as the FP64
    PCG, within the +-2% asked of GS / IC0 (64^3; very small systems, where a
    last replacement cycle weighs more, may need a few more)."""
    A, b = gen.grid3d_lognormal(64, seed=1002)
    sysm = gb.System.from_csr(A, prec)
    _, r = sysm.solve(dev(b), tol=1e-8, maxit=20000, precision=2)
    _, r64 = sysm.solve(dev(b), tol=1e-8, maxit=20000, precision=0)
    assert r["flag"] == 0 and r["rel_true_res"] < 1e-8 * 1.01
    assert iters_ok(r["iters"], r64["iters"], prec), (r["iters"], r64["iters"])
    sysm.close()


@pytest.mark.parametrize("prec", ["ichol", "GS_std"])
def test_split_precision_graph_eager_and_x0(prec):
    A, b = gen.grid2d_unit(48, seed=11)
    sysm = gb.System.from_csr(A, prec)
    x1, r1 = sysm.solve(dev(b), tol=1e-9, maxit=3000, precision=2, use_graph=True)
    x2, r2 = sysm.solve(dev(b), tol=1e-9, maxit=3000, precision=2, use_graph=False)
    assert r1["iters"] == r2["iters"] and r1["flag"] == r2["flag"] == 0
    assert torch.equal(x1, x2)
    # a nonzero x0 (tolerance relative to ||b - A x0||, as cg.c)
    x4, r4 = sysm.solve(dev(b), x=x1 * 0.5, tol=1e-9, maxit=3000, precision=2)
    assert r4["flag"] == 0 and r4["rel_true_res"] < 1e-9 * 1.01
    sysm.close()


def test_split_precision_unsupported_preconditioner():
    A, b = gen.grid2d_unit(16, seed=3)
    sysm = gb.System.from_csr(A, "line_jacobi")
    with pytest.raises(RuntimeError):
        sysm.solve(dev(b), precision=2)
    sysm.close()


def test_host_buffers_solve():
    A, b = gen.grid2d_unit(40, seed=5)
    ref = oracle.solve(A.n, A.ia, A.ja, A.a, b, "ichol", 1e-10, 3000)
    sysm = gb.System.from_csr(A, "ichol")
    x, r = sysm.solve_host(b, tol=1e-10, maxit=3000)
    assert iters_ok(r["iters"], ref["iters"], "ichol")
    assert np.linalg.norm(x - ref["x"]) / np.linalg.norm(ref["x"]) < X_TOL
    sysm.close()


def test_nonzero_initial_guess():
    A, b = gen.grid2d_unit(30, seed=9)
    x0 = np.random.default_rng(1).standard_normal(A.n)
    ref = oracle.solve(A.n, A.ia, A.ja, A.a, b, "GS_std", 1e-10, 3000, x0=x0)
    sysm = gb.System.from_csr(A, "GS_std")
    x, r = sysm.solve(dev(b), dev(x0), tol=1e-10, maxit=3000)
    assert iters_ok(r["iters"], ref["iters"], "GS_std")
    assert np.linalg.norm(x.cpu().numpy() - ref["x"]) / np.linalg.norm(ref["x"]) < X_TOL
    sysm.close()


def _pdata_gpu_convention(A, prec, keep):
    """LAP's CUDA-driver setup (cg_driver2.c:95-144, :210-351) on the device."""
    L_ = gb.lib()
    n = A.n
    Lp, Up, d = oracle.split(n, A.ia, A.ja, A.a)
    if prec == "GS_std":
        Lp, Up = oracle.embed_diagonal(n, Lp, Up, d)
    p = gb.PData()
    p.n, p.m, p.k = n, 1, 1
    p.prec_op = prec.encode()
    arrs = {k: dev(v) for k, v in dict(lia=Lp[0], lja=Lp[1], la=Lp[2], uia=Up[0], uja=Up[1],
                                        ua=Up[2], d=d).items()}
    keep.update(arrs)
    for k in ("lia", "lja", "la", "uia", "uja", "ua", "d"):
        setattr(p, k, gb.ptr(arrs[k]))
    p.lnnz, p.unnz = len(Lp[1]), len(Up[1])
    dr = torch.zeros(n, dtype=torch.float64, device="cuda")
    L_.cuda_vector_reciprocal(n, gb.ptr(arrs["d"]), gb.ptr(dr))
    keep["dr"] = dr
    p.d_r = gb.ptr(dr)
    for k in ("aux_vec1", "aux_vec2", "aux_vec3"):
        keep[k] = torch.zeros(n, dtype=torch.float64, device="cuda")
        setattr(p, k, gb.ptr(keep[k]))
    return p


@pytest.mark.parametrize("prec", ["line_jacobi", "GS_std", "ichol", "it_jacobi"])
def test_lap_cg_dropin(golden, prec):
    """LAP's cg() symbol on device pointers, set up the way cg_driver2.c's CUDA
    branch does, reproduces the reference's iterations and solution."""
    n, ia, ja, a, b = golden_matrix(golden, "grid3d")
    it_ref, flag_ref, M, K, maxit = (int(v) for v in golden[f"grid3d_{prec}_it"])
    tol = float(golden[f"grid3d_{prec}_tol"][0])
    A = gen.CSR(n, ia, ja, a)
    keep = {}
    p = _pdata_gpu_convention(A, prec, keep)
    p.k = K
    dia, dja, da, db = dev(ia), dev(ja), dev(a), dev(b)
    if prec == "ichol":
        iv = dev(a.copy())
        gb.lib().initialize_ichol(n, len(ja), gb.ptr(dia), gb.ptr(dja), gb.ptr(iv))
        keep["iv"] = iv
        p.ichol_vals = gb.ptr(iv)
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    hist = np.zeros(maxit + 3)
    it, flag = C.c_int(), C.c_int()
    torch.cuda.synchronize()
    gb.lib().cg(n, float(len(ja)), gb.ptr(dia), gb.ptr(dja), gb.ptr(da), gb.ptr(x), gb.ptr(db), tol,
                C.byref(p), maxit, C.byref(it), C.byref(flag), hist.ctypes.data)
    assert flag.value == 0 and iters_ok(it.value, it_ref, prec)
    xs = x.cpu().numpy()
    xref = golden[f"grid3d_{prec}_x"]
    assert np.linalg.norm(xs - xref) / np.linalg.norm(xref) < X_TOL
    # prec_function applies the same preconditioner as the reference, in the
    # reference's operation order: bit-identical to the oracle
    y = torch.zeros(n, dtype=torch.float64, device="cuda")
    gb.lib().prec_function(gb.ptr(dia), gb.ptr(dja), gb.ptr(da), len(ja), C.byref(p), gb.ptr(db), gb.ptr(y))
    assert np.array_equal(y.cpu().numpy(), oracle.prec_apply(n, ia, ja, a, b, prec, 1, K))


@pytest.mark.parametrize("prec", ["line_jacobi", "GS_std", "ichol", "it_jacobi", "GS_it", "GS_it2", "none"])
def test_precond_apply_bit_exact(golden, prec):
    n, ia, ja, a, b = golden_matrix(golden, "knn")
    sysm = gb.System(dev(ia), dev(ja), dev(a), prec, 1, 2)
    y = sysm.precond(dev(b))
    assert np.array_equal(y.cpu().numpy(), oracle.prec_apply(n, ia, ja, a, b, prec, 1, 2))
    sysm.close()


def test_breakdown_on_zero_rhs():
    A, _ = gen.grid2d_unit(16, seed=1)
    sysm = gb.System.from_csr(A, "ichol")
    x, r = sysm.solve(torch.zeros(A.n, dtype=torch.float64, device="cuda"), tol=1e-8, maxit=100)
    assert r["flag"] == 2 and r["status"] == 2  # rho = p'q = 0: breakdown, not NaN
    assert not x.any()
    sysm.close()


def test_bad_inputs_rejected():
    A, _ = gen.grid2d_unit(8, seed=1)
    rows = np.repeat(np.arange(A.n), np.diff(A.ia))
    keep = rows != A.ja
    keep[A.ia[3]:A.ia[4]] = True  # drop every diagonal but row 3's
    ja2 = A.ja[keep]
    ia2 = np.zeros(A.n + 1, dtype=np.int32)
    np.cumsum(np.bincount(rows[keep], minlength=A.n), out=ia2[1:])
    with pytest.raises(gb.GbError) as e:
        gb.System(dev(ia2), dev(ja2), dev(A.a[keep]), "ichol")
    assert e.value.status == 5
    with pytest.raises(gb.GbError):
        gb.System.from_csr(A, "no_such_preconditioner")


def test_zero_pivot_reported():
    A, b = gen.grid2d_unit(8, seed=1)
    a = A.a.copy()
    rows = np.repeat(np.arange(A.n), np.diff(A.ia))
    a[(rows == A.ja) & (rows == 5)] = -1.0
    sysm = gb.System(dev(A.ia), dev(A.ja), dev(a), "ichol")
    assert sysm.info()["status"] == 3
    x, r = sysm.solve(dev(b), tol=1e-8, maxit=50)
    assert r["flag"] == 2
    sysm.close()


def test_sync_free_wait_timeout_reports_status():
    """Failure path of the sync-free solves without faulting or hanging the GPU:
    a 1 ns wait budget makes every wait that has to spin give up at its first
    clock check; the solve must come back with GB_TIMEOUT, and the system must
    work normally again once the default budget is restored."""
    A, b = gen.grid2d_unit(512, seed=2)  # 1023 levels: later rows always spin
    sysm = gb.System.from_csr(A, "GS_std")
    gb.check(gb.lib().gb_debug_set_spin_budget(sysm.h, 1), "set budget")
    x, r = sysm.solve(dev(b), tol=1e-8, maxit=20)
    assert r["status"] == 4
    gb.check(gb.lib().gb_debug_set_spin_budget(sysm.h, 0), "reset budget")
    x, r = sysm.solve(dev(b), tol=1e-8, maxit=5000)
    assert r["status"] == 0 and r["flag"] == 0
    sysm.close()


def test_large_grid3d_properties():
    """64^3 lognormal: converges, true residual meets tol, IC0 beats Jacobi in iterations."""
    A, b = gen.grid3d_lognormal(64, seed=1002)
    res = {}
    for prec in ("line_jacobi", "ichol", "GS_std"):
        sysm = gb.System.from_csr(A, prec)
        x, r = sysm.solve(dev(b), tol=1e-8, maxit=10000)
        assert r["flag"] == 0 and r["rel_true_res"] < 2e-8
        res[prec] = r["iters"]
        sysm.close()
    assert res["ichol"] < res["line_jacobi"] and res["GS_std"] < res["line_jacobi"]


_CLUSTER_CHILD = r"""
import sys, numpy as np, torch
sys.path.insert(0, sys.argv[1])
import lap_gb300 as gb
from lap_gb300 import gen
A, b = gen.grid3d_lognormal(40, seed=1002)
for prec in ("ichol", "GS_std"):
    s = gb.System.from_csr(A, prec)
    for p in (0, 1, 2):
        x, r = s.solve(torch.from_numpy(b).cuda(), tol=1e-9, maxit=5000, precision=p)
        np.save(f"{sys.argv[2]}_{prec}_{p}.npy", x.cpu().numpy())
    s.close()
"""


def test_cluster_form_matches_per_cta_form(tmp_path):
    """The solves in thread-block clusters pass boundary values through
    distributed shared memory instead of L2 -- pushed into an inbox (FP32)
    or pulled from the previous tile's CTA (FP64): the arithmetic is the
    same, so every precision mode's solution must be bitwise identical to
    the per-CTA form's (GBLAP_TRI_CLUSTER=0), in clusters of 8 and of 16
    alike.  The switch is read once per process."""
    import os
    import subprocess
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = {}
    for mode in ("0", "8", "16"):
        env = dict(os.environ, GBLAP_TRI_CLUSTER=mode)
        stem = str(tmp_path / f"cl{mode}")
        subprocess.run([sys.executable, "-c", _CLUSTER_CHILD, root, stem], env=env, check=True,
                       timeout=600)
        out[mode] = stem
    for prec in ("ichol", "GS_std"):
        for p in (0, 1, 2):
            a = np.load(f"{out['0']}_{prec}_{p}.npy")
            for cl in ("8", "16"):
                c = np.load(f"{out[cl]}_{prec}_{p}.npy")
                assert np.array_equal(a, c), (prec, p, cl)


def test_fixed_record_layout_matches_general_layout(tmp_path):
    """The FP32 records of a short-only plan are kept in the fixed layout
    (one 48-byte block per row, read by the short-record kernel); with
    GBLAP_TRI_FIXED=0 they keep the general layout and run the general
    kernel.  Each row's terms are folded in the same order in both, so the
    FP32-Krylov and split solutions must be bitwise identical."""
    import os
    import subprocess
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = {}
    for fixed in ("1", "0"):
        env = dict(os.environ, GBLAP_TRI_FIXED=fixed)
        stem = str(tmp_path / f"fx{fixed}")
        subprocess.run([sys.executable, "-c", _CLUSTER_CHILD, root, stem], env=env, check=True,
                       timeout=600)
        out[fixed] = stem
    for prec in ("ichol", "GS_std"):
        for p in (1, 2):
            a = np.load(f"{out['1']}_{prec}_{p}.npy")
            c = np.load(f"{out['0']}_{prec}_{p}.npy")
            assert np.array_equal(a, c), (prec, p)


_LEVELS_CHILD = r"""
import sys, json, ctypes as C, numpy as np, torch
sys.path.insert(0, sys.argv[1])
import lap_gb300 as gb
import oracle
from lap_gb300 import gen
g = np.load(sys.argv[1] + "/tests/golden/golden.npz")
L = gb.lib()
dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
out = {"exact": {}, "pcg": {}, "split": {}}
for name in ["grid2d", "grid3d", "chunglu", "knn", "aniso"]:
    ia, ja, a = g[name + "_ia"], g[name + "_ja"], g[name + "_a"]
    n = len(ia) - 1
    Lp, Up, d = oracle.split(n, ia, ja, a)
    (lia, lja, la), (uia, uja, ua) = oracle.embed_diagonal(n, Lp, Up, d)
    xs = dev(g[name + "_spmv_x"])
    ok = True
    for (p, j, v, fn, key) in ((lia, lja, la, L.cuda_lower_triangular_solve, "lsolve"),
                               (uia, uja, ua, L.cuda_upper_triangular_solve, "usolve")):
        dp, dj, dv, y = dev(p), dev(j), dev(v), dev(np.zeros(n))
        fn(n, len(j), gb.ptr(dp), gb.ptr(dj), gb.ptr(dv), 0, gb.ptr(xs), gb.ptr(y))
        got, want = y.cpu().numpy(), g[name + "_" + key]
        if name == "chunglu":  # rows of > 32 dependencies are reduced by a whole warp
            ok = ok and bool(np.allclose(got, want, rtol=1e-12, atol=1e-14 * np.abs(want).max()))
        else:
            ok = ok and bool(np.array_equal(got, want))
    out["exact"][name] = ok
    A = gen.CSR(n, ia, ja, a)
    for prec in ("ichol", "GS_std"):
        s = gb.System.from_csr(A, prec)
        x, r = s.solve(dev(g[name + "_b"]), tol=1e-10, maxit=5000)
        ref = oracle.solve(n, ia, ja, a, g[name + "_b"], prec, 1e-10, 5000)
        out["pcg"][name + "_" + prec] = [r["iters"], ref["iters"],
            float(np.linalg.norm(x.cpu().numpy() - ref["x"]) / np.linalg.norm(ref["x"]))]
        s.close()
A, b = gen.chung_lu(20000, seed=1003)
for prec in ("ichol", "GS_std"):
    s = gb.System.from_csr(A, prec)
    res = []
    for p in (0, 2):
        x, r = s.solve(dev(b), tol=1e-10, maxit=5000, precision=p)
        res.append([r["iters"], r["flag"], r["rel_true_res"]])
        np.save(sys.argv[2] + "_" + prec + "_" + str(p) + ".npy", x.cpu().numpy())
    out["split"][prec] = res
    s.close()
json.dump(out, open(sys.argv[2] + ".json", "w"))
"""


def test_levels_form(tmp_path):
    """The levels form of the triangular solves (records in global level
    order, every dependency through L2; chosen for random labellings) forced
    on every case: the exact solves stay bit-identical to the reference's
    (to 1e-12 where rows of more than 32 dependencies are warp-reduced, as
    in the tile form),
    PCG matches the oracle (iterations +-2%, x within 1e-6), and on a
    Chung-Lu graph both forms give the same solutions to the solve's
    accuracy."""
    import json
    import os
    import subprocess
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    res = {}
    for form in ("levels", "tiles"):
        env = dict(os.environ, GBLAP_TRI_FORM=form)
        stem = str(tmp_path / form)
        subprocess.run([sys.executable, "-c", _LEVELS_CHILD, root, stem], env=env, check=True, timeout=900)
        res[form] = json.load(open(stem + ".json"))
    lv = res["levels"]
    assert all(lv["exact"].values()), lv["exact"]
    for key, (it, ref_it, err) in lv["pcg"].items():
        assert abs(it - ref_it) <= max(1, int(np.ceil(0.02 * ref_it))), (key, it, ref_it)
        assert err < 1e-6, (key, err)
    for prec in ("ichol", "GS_std"):
        for p, (it, flag, rt) in zip((0, 2), lv["split"][prec]):
            assert flag == 0 and rt < 1e-10 * 1.01
            it_t = res["tiles"]["split"][prec][(0, 2).index(p)][0]
            assert abs(it - it_t) <= max(1, int(np.ceil(0.02 * it_t))), (prec, p, it, it_t)
            a = np.load(str(tmp_path / f"levels_{prec}_{p}.npy"))
            t = np.load(str(tmp_path / f"tiles_{prec}_{p}.npy"))
            assert np.linalg.norm(a - t) / np.linalg.norm(t) < 1e-8, (prec, p)


@pytest.mark.parametrize("prec", ["ichol", "GS_std"])
@pytest.mark.parametrize("part_deps", [None, "32"])
def test_split_hub_rows_match_oracle(prec, part_deps, monkeypatch):
    """Rows of more than two parts of dependencies (with the default 1024-
    entry parts, three in each factor of this 65,475-row Chung-Lu graph, up
    to 6159) are solved as parts on several warps plus a combine record: the
    PCG solution still matches the reference's CPU PCG (oracle) within 1e-6
    and its iteration count within 2%, in FP64 and in split precision (whose
    target is the same tol). 32-entry parts split every row of more than 64
    dependencies and give the largest row 193 parts, which the combine reads
    in several loads per lane."""
    if part_deps:
        monkeypatch.setenv("GBLAP_TRI_PART_DEPS", part_deps)
    A, b = gen.chung_lu(1 << 16, seed=1003)
    ref = oracle.solve(A.n, A.ia, A.ja, A.a, b, prec, 1e-10, 5000)
    s = gb.System.from_csr(A, prec)
    for p in (0, 2):
        x, r = s.solve(torch.from_numpy(b).cuda(), tol=1e-10, maxit=5000, precision=p)
        assert r["flag"] == 0
        err = np.linalg.norm(x.cpu().numpy() - ref["x"]) / np.linalg.norm(ref["x"])
        assert err < 1e-6, (p, err)
        if p == 0:
            assert abs(r["iters"] - ref["iters"]) <= max(1, int(np.ceil(0.02 * ref["iters"]))), (r["iters"], ref["iters"])
    s.close()
