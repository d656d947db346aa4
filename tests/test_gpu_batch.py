"""Batching through the C ABI (gb_batch_*, gb_pcg_solve_multi): every system
of a batch must give what the single-system solver gives for it alone -- the
same iteration count (+-1, Jacobi family) and x within 1e-7 relative -- and
the reference's result through the oracle (x within 1e-6, iterations +-1)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a GPU", allow_module_level=True)

import lap_gb300 as gb  # noqa: E402
import oracle  # noqa: E402
from lap_gb300 import gen  # noqa: E402


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _mixed_batch(seed=7):
    rng = np.random.default_rng(seed)
    mats = [gen.knn_graph(int(n), rng=rng) for n in (300, 1500, 40, 5000, 800)]
    mats += [gen.grid2d_unit(24, seed=3)[0], gen.grid3d_lognormal(12, seed=4)[0]]
    rhs = [rng.uniform(-1, 1, A.n) for A in mats]
    return mats, rhs


@pytest.mark.parametrize("prec", ["line_jacobi", "none"])
def test_batch_matches_single_solves_and_oracle(prec):
    mats, rhs = _mixed_batch()
    bt = gb.Batch(mats, prec)
    x, its, flags, r = bt.solve(dev(np.concatenate(rhs)), tol=1e-9, maxit=20000)
    assert r["flag"] == 0 and (flags == 0).all()
    for s, (A, b) in enumerate(zip(mats, rhs)):
        single = gb.System.from_csr(A, prec)
        xs, rs = single.solve(dev(b), tol=1e-9, maxit=20000)
        single.close()
        assert abs(int(its[s]) - rs["iters"]) <= 1, (s, its[s], rs["iters"])
        xb = bt.split(x)[s].cpu().numpy()
        # different reduction order than the single solver: agreement to the solve's accuracy
        assert np.linalg.norm(xb - xs.cpu().numpy()) / np.linalg.norm(xs.cpu().numpy()) < 1e-7
        ref = oracle.solve(A.n, A.ia, A.ja, A.a, b, prec, 1e-9, 20000)
        assert abs(int(its[s]) - ref["iters"]) <= 1
        assert np.linalg.norm(xb - ref["x"]) / np.linalg.norm(ref["x"]) < 1e-6
    assert r["rel_true_res"] < 1e-8
    bt.close()


def test_batch_graph_eager_and_rerun_identical():
    mats, rhs = _mixed_batch(11)
    bt = gb.Batch(mats)
    b = dev(np.concatenate(rhs))
    x1, i1, _, _ = bt.solve(b, tol=1e-8, use_graph=True)
    x2, i2, _, _ = bt.solve(b, tol=1e-8, use_graph=False)
    x3, i3, _, _ = bt.solve(b, tol=1e-8)
    assert (i1 == i2).all() and (i1 == i3).all()
    assert torch.equal(x1, x2) and torch.equal(x1, x3)  # fixed-order reductions
    bt.close()


def test_batch_split_precision_error_vs_fp64():
    mats, rhs = _mixed_batch(5)
    bt = gb.Batch(mats)
    b = dev(np.concatenate(rhs))
    x64, i64, _, _ = bt.solve(b, tol=1e-10, maxit=20000, precision=0)
    x32, i32, fl, r = bt.solve(b, tol=1e-10, maxit=20000, precision=2)
    assert (fl == 0).all() and r["outer"] >= 1
    assert r["rel_true_res"] < 1e-10 * 1.01  # x0 = 0: tol is relative to ||b|| per system
    for s in range(bt.count):
        a, c = bt.split(x32)[s].cpu().numpy(), bt.split(x64)[s].cpu().numpy()
        assert np.linalg.norm(a - c) / np.linalg.norm(c) < 1e-8
    bt.close()


def test_batch_maxit_flags_per_system():
    mats, rhs = _mixed_batch(2)
    bt = gb.Batch(mats)
    _, its, flags, r = bt.solve(dev(np.concatenate(rhs)), tol=1e-12, maxit=5)
    assert (flags == 1).all() and (its == 6).all() and r["flag"] == 1
    bt.close()


def test_batch_rejects_bad_input():
    A = gen.grid2d_unit(8, seed=1)[0]
    with pytest.raises(gb.GbError):
        gb.Batch([A], "ichol")  # batches run line_jacobi / none
    # a row without its diagonal
    ia, ja, a = A.ia.copy(), A.ja.copy(), A.a.copy()
    row0 = slice(ia[0], ia[1])
    a[row0][ja[row0] == 0] = 0.0
    with pytest.raises(gb.GbError):
        gb.Batch([gen.CSR(A.n, ia, ja, a)])


@pytest.mark.parametrize("prec", ["line_jacobi", "none"])
def test_multi_rhs_matches_single_solves(prec):
    A, _ = gen.grid3d_lognormal(16, seed=1002)
    Bm = gen.multi_rhs(A.n, 6, seed=1005)
    sysm = gb.System.from_csr(A, prec)
    X, its, r = gb.solve_multi(sysm, dev(Bm), tol=1e-9, maxit=20000)
    assert r["flag"] == 0
    # unpreconditioned CG is the most sensitive to reduction order: 3%
    slack = (lambda it: 1) if prec == "line_jacobi" else (lambda it: max(1, int(np.ceil(0.03 * it))))
    for k in range(Bm.shape[0]):
        xs, rs = sysm.solve(dev(Bm[k]), tol=1e-9, maxit=20000)
        assert abs(int(its[k]) - rs["iters"]) <= slack(rs["iters"]), (k, its[k], rs["iters"])
        assert torch.linalg.norm(X[k] - xs) / torch.linalg.norm(xs) < 1e-7
    # split precision on the same columns
    X2, its2, r2 = gb.solve_multi(sysm, dev(Bm), tol=1e-10, maxit=20000, precision=2)
    X64, _, _ = gb.solve_multi(sysm, dev(Bm), tol=1e-10, maxit=20000, precision=0)
    assert r2["flag"] == 0
    assert float(torch.linalg.norm(X2 - X64) / torch.linalg.norm(X64)) < 1e-8
    sysm.close()


@pytest.mark.parametrize("nrhs", [1, 7, 32, 33, 70])
def test_multi_rhs_layouts_match_single_solves(nrhs):
    """Up to 32 right-hand sides run on interleaved vectors (32 // nrhs rows per
    warp step; 7 leaves idle lanes); 33 and 70 as chunks of 32 and a last one
    of 1 or 6 (the 32-column batch reused for two chunks); a nonzero x0 goes
    through the transposes in both directions."""
    A, _ = gen.grid3d_lognormal(10, seed=1003)
    Bm = gen.multi_rhs(A.n, nrhs, seed=1006)
    X0 = np.random.default_rng(1007).uniform(-1, 1, Bm.shape)
    sysm = gb.System.from_csr(A, "line_jacobi")
    X, its, r = gb.solve_multi(sysm, dev(Bm), dev(X0), tol=1e-9, maxit=20000)
    assert r["flag"] == 0
    for k in range(nrhs):
        xs, rs = sysm.solve(dev(Bm[k]), dev(X0[k]), tol=1e-9, maxit=20000)
        assert abs(int(its[k]) - rs["iters"]) <= 1, (k, its[k], rs["iters"])
        assert torch.linalg.norm(X[k] - xs) / torch.linalg.norm(xs) < 1e-7
    # fixed-order reductions: the graph loop, the eager loop and a rerun agree bitwise
    X1, i1, _ = gb.solve_multi(sysm, dev(Bm), dev(X0), tol=1e-9, maxit=20000, use_graph=False)
    X2, i2, _ = gb.solve_multi(sysm, dev(Bm), dev(X0), tol=1e-9, maxit=20000)
    assert (i1 == its).all() and (i2 == its).all()
    assert torch.equal(X1, X) and torch.equal(X2, X)
    sysm.close()


@pytest.mark.parametrize("nrhs", [5, 32])
def test_multi_rhs_split_inline_replacement(nrhs):
    """Interleaved split precision replaces each right-hand side's residual
    inside the loop, when its own recurrence pauses: every column meets the
    FP64 target, agrees with the FP64 multi-RHS solution, takes about the
    iterations it takes when solved alone, and the graph and eager loops
    agree bitwise.  The partial sums are taken in another order when a column
    runs alone; with FP32 products that can move a replacement by one
    iteration, which costs or saves up to ~5% of the iterations (the same
    spread the concatenated layout shows), so a column may differ by 8% and
    the mean by 2%."""
    A, _ = gen.grid3d_lognormal(16, seed=1004)
    Bm = gen.multi_rhs(A.n, nrhs, seed=1008)
    sysm = gb.System.from_csr(A, "line_jacobi")
    kw = dict(tol=1e-10, maxit=20000)
    X, its, r = gb.solve_multi(sysm, dev(Bm), precision=2, **kw)
    X64, _, _ = gb.solve_multi(sysm, dev(Bm), precision=0, **kw)
    assert r["flag"] == 0 and r["outer"] >= 2
    assert r["rel_true_res"] < 1e-10  # x0 = 0: the target is tol * ||b|| per column
    alone = []
    for k in range(nrhs):
        assert float(torch.linalg.norm(X[k] - X64[k]) / torch.linalg.norm(X64[k])) < 1e-8
        _, i1, r1 = gb.solve_multi(sysm, dev(Bm[k:k + 1]), precision=2, **kw)
        assert r1["flag"] == 0
        alone.append(int(i1[0]))
        assert abs(int(its[k]) - alone[-1]) <= max(2, int(np.ceil(0.08 * alone[-1]))), (k, its[k], alone[-1])
    assert abs(float(np.mean(its)) - float(np.mean(alone))) <= 0.02 * float(np.mean(alone))
    Xe, ie, _ = gb.solve_multi(sysm, dev(Bm), precision=2, use_graph=False, **kw)
    assert (ie == its).all() and torch.equal(Xe, X)
    sysm.close()


@pytest.mark.parametrize("prec", [0, 2])
def test_multi_rhs_chunks_match_block_form(prec, monkeypatch):
    """More than 32 right-hand sides in chunks of 32 agree with the block
    form (all 45 columns in one launch as concatenated vectors,
    GBLAP_MULTI_FORM=blocks) within a few iterations and 1e-8 per column;
    the per-column counts and the aggregate are in column order; and the
    cached chunk batches survive a solve of another count in between."""
    A, _ = gen.grid3d_lognormal(12, seed=1009)
    Bm = gen.multi_rhs(A.n, 45, seed=1010)
    sysm = gb.System.from_csr(A, "line_jacobi")
    kw = dict(tol=1e-10, maxit=20000, precision=prec)
    X, its, r = gb.solve_multi(sysm, dev(Bm), **kw)
    assert r["flag"] == 0 and r["iters"] == int(its.max())
    gb.solve_multi(sysm, dev(Bm[:5]), **kw)
    Xr, itr, _ = gb.solve_multi(sysm, dev(Bm), **kw)
    assert (itr == its).all() and torch.equal(Xr, X)
    monkeypatch.setenv("GBLAP_MULTI_FORM", "blocks")
    Xb, itb, rb = gb.solve_multi(sysm, dev(Bm), **kw)
    monkeypatch.delenv("GBLAP_MULTI_FORM")
    assert rb["flag"] == 0
    slack = 1 if prec == 0 else 3
    for k in range(45):
        assert abs(int(its[k]) - int(itb[k])) <= max(slack, int(np.ceil(0.08 * int(itb[k])))), (k, its[k], itb[k])
        assert float(torch.linalg.norm(X[k] - Xb[k]) / torch.linalg.norm(Xb[k])) < 1e-8
    sysm.close()


def test_multi_rhs_unsupported_preconditioner():
    A, b = gen.grid2d_unit(16, seed=3)
    sysm = gb.System.from_csr(A, "ichol")
    with pytest.raises(gb.GbError):
        gb.solve_multi(sysm, dev(np.stack([b, b])))
    sysm.close()


def test_batch_autotune_same_results_no_slower():
    """gb_batch_autotune times rows-per-bundle x chunk-row choices on the
    batch's own loop and applies the fastest: the tuned batch converges like
    the default one (every system, iterations +-1) to the same solutions (to
    the rounding of the regrouped reductions), the chosen plan timed no
    slower than the default, and a second batch of the same class takes the
    cached choice without timing; split precision works on the tuned plan."""
    mats, rhs = _mixed_batch(seed=11)
    b = dev(np.concatenate(rhs))
    bt = gb.Batch(mats, "line_jacobi")
    x0, it0, f0, _ = bt.solve(b, tol=1e-10, maxit=20000)
    t = bt.autotune(b, iters=12)
    assert t["rows_per_bundle"] in (32, 16, 8) and t["chunk_rows"] in (1024, 2048, 4096)
    assert 0.0 < t["ms_best"] <= t["ms_default"], t
    x1, it1, f1, _ = bt.solve(b, tol=1e-10, maxit=20000)
    assert (f0 == 0).all() and (f1 == 0).all()
    assert np.abs(it1 - it0).max() <= 1, (it0, it1)
    assert float(torch.linalg.norm(x1 - x0) / torch.linalg.norm(x0)) < 1e-8
    xs, _, fs, rs = bt.solve(b, tol=1e-10, maxit=20000, precision=2)
    assert (fs == 0).all() and rs["rel_true_res"] < 1e-10 * 1.01
    bt2 = gb.Batch(mats, "line_jacobi")
    t2 = bt2.autotune(b, iters=12)
    assert (t2["rows_per_bundle"], t2["chunk_rows"]) == (t["rows_per_bundle"], t["chunk_rows"])
    assert t2["ms_default"] == 0.0 and t2["ms_best"] == 0.0  # from the cache
    x2, *_ = bt2.solve(b, tol=1e-10, maxit=20000)
    assert torch.equal(x2, x1)  # the same plan: bitwise the same result
    bt.close()
    bt2.close()


def test_multi_rhs_autotune_same_results_no_slower():
    A, _ = gen.grid3d_lognormal(16, seed=5)
    B = dev(gen.multi_rhs(A.n, 40, seed=1005))
    s = gb.System.from_csr(A, "line_jacobi")
    X0, it0, r0 = gb.solve_multi(s, B, tol=1e-10, maxit=5000)
    t = gb.autotune_multi(s, B, iters=12)
    assert t["width"] in (32, 16, 8) and 0.0 < t["ms_best"] <= t["ms_default"], t
    X1, it1, r1 = gb.solve_multi(s, B, tol=1e-10, maxit=5000)
    assert r0["flag"] == 0 and r1["flag"] == 0
    assert np.abs(it1 - it0).max() <= 1
    assert float(torch.linalg.norm(X1 - X0) / torch.linalg.norm(X0)) < 1e-8
    s.close()
