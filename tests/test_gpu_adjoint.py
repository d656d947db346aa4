"""Adjoint gradient through the C ABI (gb_adjoint_grad / gb_adjoint_scatter).

x = (L(w) + 1e-2 I)^{-1} b on an anisotropic lognormal grid, loss
L = 0.5 ||x - x*||^2.  The adjoint solves A lambda = x - x* with the same PCG
(A is SPD) and scatters dL/dw_ij = -(lambda_i - lambda_j)(x_i - x_j),
dL/db = lambda.  Checked against
  * the scatter formula on every stored entry (exact),
  * a gradient from the reference's CPU PCG (the oracle) used for both the
    forward and the adjoint solve,
  * central finite differences (h = 1e-6, FP64) on 64 random edges, with the
    solver wrapped in a torch.autograd.Function (test harness only).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a GPU", allow_module_level=True)

import lap_gb300 as gb  # noqa: E402
import oracle  # noqa: E402
from lap_gb300 import gen  # noqa: E402

SHIFT = 1e-2


class GridModel:
    """The anisotropic grid's CSR pattern, with values rebuilt from edge weights."""

    def __init__(self, nside, prec="ichol", **kw):
        ei, ej, w = gen.grid2d_aniso_edges(nside, seed=1006)
        self.A = gen.laplacian_from_edges(nside * nside, ei, ej, w, shift=SHIFT)
        A = self.A
        rows = np.repeat(np.arange(A.n), np.diff(A.ia))
        key = rows.astype(np.int64) * A.n + A.ja
        lo, hi = np.minimum(ei, ej), np.maximum(ei, ej)
        pos_lo_hi = np.searchsorted(key, lo * A.n + hi)
        pos_hi_lo = np.searchsorted(key, hi * A.n + lo)
        diag = np.searchsorted(key, np.arange(A.n, dtype=np.int64) * (A.n + 1))
        # the library lists dL/dw for strict-lower entries in row-major order
        strict_lower = np.nonzero(A.ja < rows)[0]
        self.edge_t = torch.from_numpy(np.searchsorted(strict_lower, pos_hi_lo)).cuda()
        self.pos = [torch.from_numpy(p).cuda() for p in (pos_lo_hi, pos_hi_lo, diag)]
        self.ei, self.ej = torch.from_numpy(lo).cuda(), torch.from_numpy(hi).cuda()
        self.w0 = torch.from_numpy(w).cuda()
        self.sysm = gb.System.from_csr(A, prec)
        self.kw = kw

    def values(self, w):
        a = torch.zeros(self.A.nnz, dtype=torch.float64, device="cuda")
        a[self.pos[0]] = -w
        a[self.pos[1]] = -w
        deg = torch.zeros(self.A.n, dtype=torch.float64, device="cuda")
        deg.index_add_(0, self.ei, w)
        deg.index_add_(0, self.ej, w)
        a[self.pos[2]] = deg + SHIFT
        return a

    def set_weights(self, w):
        self.sysm.set_values(self.values(w))


class LaplacianSolve(torch.autograd.Function):
    """x = A(w)^{-1} b through gb_pcg_solve; backward through gb_adjoint_grad."""

    @staticmethod
    def forward(ctx, w, b, model):
        model.set_weights(w.detach())
        x, r = model.sysm.solve(b.detach(), **model.kw)
        assert r["flag"] == 0
        ctx.model = model
        ctx.save_for_backward(x)
        return x

    @staticmethod
    def backward(ctx, gx):
        (x,) = ctx.saved_tensors
        m = ctx.model
        lam, G, eg, r = m.sysm.adjoint(x, gx.contiguous(), **m.kw)
        assert r["flag"] == 0
        return eg[m.edge_t], lam, None


def test_scatter_matches_formula():
    A, b, _ = gen.grid2d_aniso(12, seed=1006)
    sysm = gb.System.from_csr(A, "line_jacobi")
    rng = np.random.default_rng(0)
    x, lam = rng.standard_normal(A.n), rng.standard_normal(A.n)
    G = torch.empty(A.nnz, dtype=torch.float64, device="cuda")
    ne = (A.nnz - A.n) // 2
    eg = torch.empty(ne, dtype=torch.float64, device="cuda")
    dx, dl = torch.from_numpy(x).cuda(), torch.from_numpy(lam).cuda()
    gb.check(gb.lib().gb_adjoint_scatter(sysm.h, gb.ptr(dx), gb.ptr(dl), gb.ptr(G), gb.ptr(eg)), "scatter")
    rows = np.repeat(np.arange(A.n), np.diff(A.ia))
    assert np.array_equal(G.cpu().numpy(), -lam[rows] * x[A.ja])
    sl = A.ja < rows
    want = -(lam[rows[sl]] - lam[A.ja[sl]]) * (x[rows[sl]] - x[A.ja[sl]])
    assert np.array_equal(eg.cpu().numpy(), want)
    sysm.close()


@pytest.mark.parametrize("precision", [0, 2])
def test_gradient_vs_reference_cpu_adjoint(precision):
    """dL/dw and dL/db from the GPU adjoint against the same quantities built
    from the reference's CPU PCG (FP64 IC(0), the oracle) on 48^2."""
    m = GridModel(48, "ichol", tol=1e-11, maxit=5000, precision=precision)
    A = m.A
    rng = np.random.default_rng(1007)
    b, xs = rng.uniform(-1, 1, A.n), rng.standard_normal(A.n)
    w = m.w0.clone().requires_grad_(True)
    bt = torch.from_numpy(b).cuda().requires_grad_(True)
    x = LaplacianSolve.apply(w, bt, m)
    loss = 0.5 * torch.sum((x - torch.from_numpy(xs).cuda()) ** 2)
    loss.backward()
    ref_x = oracle.solve(A.n, A.ia, A.ja, A.a, b, "ichol", 1e-13, 10000)["x"]
    ref_l = oracle.solve(A.n, A.ia, A.ja, A.a, ref_x - xs, "ichol", 1e-13, 10000)["x"]
    ei, ej = m.ei.cpu().numpy(), m.ej.cpu().numpy()
    ref_gw = -(ref_l[ei] - ref_l[ej]) * (ref_x[ei] - ref_x[ej])
    gw, gb_ = w.grad.cpu().numpy(), bt.grad.cpu().numpy()
    assert np.linalg.norm(gw - ref_gw) / np.linalg.norm(ref_gw) < 1e-6
    assert np.linalg.norm(gb_ - ref_l) / np.linalg.norm(ref_l) < 1e-6
    m.sysm.close()


def test_gradient_vs_central_differences():
    """64 random edges, h = 1e-6, FP64 solves to 1e-13: the adjoint gradient
    (split precision, tol 1e-10) matches the central differences."""
    m = GridModel(96, "ichol", tol=1e-10, maxit=5000, precision=2)
    A = m.A
    rng = np.random.default_rng(1007)
    b = torch.from_numpy(rng.uniform(-1, 1, A.n)).cuda()
    xs = torch.from_numpy(rng.standard_normal(A.n)).cuda()
    w = m.w0.clone().requires_grad_(True)
    loss = 0.5 * torch.sum((LaplacianSolve.apply(w, b, m) - xs) ** 2)
    loss.backward()
    g = w.grad.clone()
    fd_kw = dict(tol=1e-13, maxit=20000, precision=0)
    h = 1e-6
    edges = rng.choice(m.w0.numel(), 64, replace=False)
    fd = []
    for e in edges:
        vals = []
        for sgn in (1.0, -1.0):
            wp = m.w0.clone()
            wp[e] += sgn * h
            m.set_weights(wp)
            x, r = m.sysm.solve(b, **fd_kw)
            assert r["flag"] == 0
            vals.append(0.5 * float(torch.sum((x - xs) ** 2)))
        fd.append((vals[0] - vals[1]) / (2 * h))
    fd = np.array(fd)
    ad = g[torch.from_numpy(edges).cuda()].cpu().numpy()
    scale = np.abs(ad).max()
    assert np.all(np.abs(fd - ad) <= 1e-4 * scale + 1e-4 * np.abs(ad)), np.c_[fd, ad]
    m.sysm.close()
