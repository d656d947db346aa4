"""Seeded synthetic graph Laplacians for the five PCG workloads.

Every generator returns a :class:`CSR` holding the FULL symmetric matrix with
0-based int32 indices, columns ascending in each row, no duplicate entries and
every diagonal entry stored -- the layout LAP's ``coo_to_csr`` produces from a
symmetric lower-triangle Matrix Market file (io_utils.c:141-235), and the one
its ``split`` needs (io_utils.c:268-363 sizes L/U from ``nnz - n``, so a row
without a stored diagonal corrupts memory there).

Workloads (seeds are fixed; the reference's SuiteSparse matrices are not used):

* ``grid2d_unit``   256x256 5-point unit-weight Laplacian + 1e-2 I; b ~ U[-1,1],
                     mean removed (seed 1001).
* ``grid3d_lognormal`` 128^3 7-point Laplacian, edge weights lognormal(0, 0.5),
                     + 1e-3 I; b ~ U[-1,1] (seed 1002).
* ``chung_lu``      power-law graph (expected-degree model, exponent 2.5, mean
                     degree 16), isolated vertices removed, random relabelling,
                     weights U(0,1]; A = 1.001 D - W; b ~ N(0,1) (seed 1003).
* ``knn_batch``     random-geometric symmetric kNN (k=8) graphs, Gaussian
                     weights exp(-d^2/sigma^2), sigma = mean kNN distance,
                     + 1e-2 I; sizes log-uniform (seed 1004).
* ``grid2d_aniso``  1024x1024 5-point, horizontal weights lognormal(0,1),
                     vertical 0.1 x lognormal(0,1), + 1e-2 I; x* ~ N(0,1),
                     b ~ U[-1,1] (seed 1006).
"""
from __future__ import annotations

import dataclasses

import numpy as np


@dataclasses.dataclass
class CSR:
    n: int
    ia: np.ndarray  # int32 [n+1]
    ja: np.ndarray  # int32 [nnz]
    a: np.ndarray   # float64 [nnz]
    name: str = ""

    @property
    def nnz(self) -> int:
        return int(self.ja.shape[0])

    def to_dense(self) -> np.ndarray:
        d = np.zeros((self.n, self.n))
        rows = np.repeat(np.arange(self.n), np.diff(self.ia))
        d[rows, self.ja] = self.a
        return d

    def matvec(self, x: np.ndarray) -> np.ndarray:
        rows = np.repeat(np.arange(self.n), np.diff(self.ia))
        return np.bincount(rows, weights=self.a * x[self.ja], minlength=self.n)


def laplacian_from_edges(n: int, ei: np.ndarray, ej: np.ndarray, w: np.ndarray,
                         shift: float = 0.0, shift_rel: float = 0.0, name: str = "") -> CSR:
    """A = D_w - W + shift*I + shift_rel*D_w for the undirected edges (ei, ej, w).

    Edges must be unique with ei != ej.  The diagonal is stored in every row.
    """
    ei = np.asarray(ei, dtype=np.int64)
    ej = np.asarray(ej, dtype=np.int64)
    w = np.asarray(w, dtype=np.float64)
    deg = np.bincount(ei, weights=w, minlength=n) + np.bincount(ej, weights=w, minlength=n)
    diag = deg * (1.0 + shift_rel) + shift
    rows = np.concatenate([ei, ej, np.arange(n, dtype=np.int64)])
    cols = np.concatenate([ej, ei, np.arange(n, dtype=np.int64)])
    vals = np.concatenate([-w, -w, diag])
    order = np.argsort(rows * n + cols, kind="stable")
    rows, cols, vals = rows[order], cols[order], vals[order]
    ia = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(np.bincount(rows, minlength=n), out=ia[1:])
    return CSR(n, ia.astype(np.int32), cols.astype(np.int32), vals, name)


def grid2d(nx: int, ny: int, wx: np.ndarray | None = None, wy: np.ndarray | None = None,
           shift: float = 0.0, name: str = "") -> CSR:
    """5-point Laplacian on an nx-by-ny grid, vertex (x, y) -> x + nx*y."""
    idx = np.arange(nx * ny, dtype=np.int64).reshape(ny, nx)
    hx_i, hx_j = idx[:, :-1].ravel(), idx[:, 1:].ravel()
    vy_i, vy_j = idx[:-1, :].ravel(), idx[1:, :].ravel()
    if wx is None:
        wx = np.ones(hx_i.shape[0])
    if wy is None:
        wy = np.ones(vy_i.shape[0])
    return laplacian_from_edges(nx * ny, np.concatenate([hx_i, vy_i]),
                                np.concatenate([hx_j, vy_j]), np.concatenate([wx, wy]),
                                shift=shift, name=name)


def grid3d(nd: int, weights: np.ndarray | None = None, shift: float = 0.0, name: str = "") -> CSR:
    """7-point Laplacian on an nd^3 grid, vertex (x, y, z) -> x + nd*y + nd^2*z.

    ``weights`` lists x-edges, then y-edges, then z-edges (C order of each).
    """
    idx = np.arange(nd ** 3, dtype=np.int64).reshape(nd, nd, nd)  # [z, y, x]
    e = [(idx[:, :, :-1], idx[:, :, 1:]), (idx[:, :-1, :], idx[:, 1:, :]),
         (idx[:-1, :, :], idx[1:, :, :])]
    ei = np.concatenate([p.ravel() for p, _ in e])
    ej = np.concatenate([q.ravel() for _, q in e])
    if weights is None:
        weights = np.ones(ei.shape[0])
    return laplacian_from_edges(nd ** 3, ei, ej, weights, shift=shift, name=name)


# ---------------------------------------------------------------- workloads

def grid2d_unit(nside: int = 256, seed: int = 1001):
    """Config 1: unit 5-point Laplacian + 1e-2 I, b ~ U[-1,1] with its mean removed."""
    A = grid2d(nside, nside, shift=1e-2, name=f"grid2d_unit_{nside}")
    rng = np.random.default_rng(seed)
    b = rng.uniform(-1.0, 1.0, A.n)
    b -= b.mean()
    return A, b


def grid3d_lognormal(nside: int = 128, seed: int = 1002):
    """Config 2: 7-point Laplacian, weights lognormal(0, 0.5), + 1e-3 I, b ~ U[-1,1]."""
    rng = np.random.default_rng(seed)
    ne = 3 * nside * nside * (nside - 1)
    w = rng.lognormal(0.0, 0.5, ne)
    A = grid3d(nside, w, shift=1e-3, name=f"grid3d_lognormal_{nside}")
    b = rng.uniform(-1.0, 1.0, A.n)
    return A, b


def grid2d_aniso(nside: int = 1024, seed: int = 1006):
    """Config 5: horizontal weights lognormal(0,1), vertical 0.1*lognormal(0,1), + 1e-2 I.

    Returns (A, b, x_star)."""
    rng = np.random.default_rng(seed)
    nh = nside * (nside - 1)
    wx = rng.lognormal(0.0, 1.0, nh)
    wy = 0.1 * rng.lognormal(0.0, 1.0, nh)
    A = grid2d(nside, nside, wx, wy, shift=1e-2, name=f"grid2d_aniso_{nside}")
    x_star = rng.standard_normal(A.n)
    b = rng.uniform(-1.0, 1.0, A.n)
    return A, b, x_star


def grid2d_aniso_edges(nside: int, seed: int = 1006):
    """Edge list (i, j, w) of :func:`grid2d_aniso` in the order its weights were drawn."""
    rng = np.random.default_rng(seed)
    nh = nside * (nside - 1)
    wx = rng.lognormal(0.0, 1.0, nh)
    wy = 0.1 * rng.lognormal(0.0, 1.0, nh)
    idx = np.arange(nside * nside, dtype=np.int64).reshape(nside, nside)
    ei = np.concatenate([idx[:, :-1].ravel(), idx[:-1, :].ravel()])
    ej = np.concatenate([idx[:, 1:].ravel(), idx[1:, :].ravel()])
    return ei, ej, np.concatenate([wx, wy])


def chung_lu(n_target: int = 1 << 22, mean_deg: float = 16.0, gamma: float = 2.5,
             seed: int = 1003):
    """Config 3: Chung-Lu power-law Laplacian, A = 1.001*D - W, b ~ N(0,1).

    Expected degrees w_i ~ (i+1)^(-1/(gamma-1)) scaled to ``mean_deg``;
    n*mean_deg/2 endpoint pairs are drawn proportionally to w, self loops
    dropped and duplicates merged; isolated vertices are removed and the rest
    relabelled by a random permutation.  Edge weights ~ U(0,1]."""
    rng = np.random.default_rng(seed)
    w = (np.arange(n_target, dtype=np.float64) + 1.0) ** (-1.0 / (gamma - 1.0))
    w *= mean_deg * n_target / w.sum()
    m = int(n_target * mean_deg / 2)
    cdf = np.cumsum(w)
    cdf /= cdf[-1]
    ei = np.searchsorted(cdf, rng.random(m), side="right")
    ej = np.searchsorted(cdf, rng.random(m), side="right")
    keep = ei != ej
    ei, ej = ei[keep], ej[keep]
    lo, hi = np.minimum(ei, ej), np.maximum(ei, ej)
    key = np.unique(lo.astype(np.int64) * n_target + hi)
    lo, hi = key // n_target, key % n_target
    used = np.zeros(n_target, dtype=bool)
    used[lo] = True
    used[hi] = True
    n = int(used.sum())
    perm = rng.permutation(n)
    newid = np.full(n_target, -1, dtype=np.int64)
    newid[np.flatnonzero(used)] = perm
    lo, hi = newid[lo], newid[hi]
    wts = 1.0 - rng.random(lo.shape[0])  # (0, 1]
    A = laplacian_from_edges(n, lo, hi, wts, shift_rel=1e-3, name=f"chung_lu_{n}")
    b = rng.standard_normal(n)
    return A, b


def knn_graph(n: int, k: int = 8, rng=None, seed: int | None = None) -> CSR:
    """Symmetric (union) kNN graph of n uniform points in [0,1]^2, Gaussian weights
    exp(-d^2/sigma^2) with sigma the mean kNN distance, A = L + 1e-2 I."""
    from scipy.spatial import cKDTree

    if rng is None:
        rng = np.random.default_rng(seed)
    pts = rng.random((n, 2))
    dist, nbr = cKDTree(pts).query(pts, k + 1)
    dist, nbr = dist[:, 1:], nbr[:, 1:]
    sigma = float(dist.mean())
    src = np.repeat(np.arange(n, dtype=np.int64), k)
    dst = nbr.ravel().astype(np.int64)
    lo, hi = np.minimum(src, dst), np.maximum(src, dst)
    key = np.unique(lo * n + hi)
    lo, hi = key // n, key % n
    d2 = ((pts[lo] - pts[hi]) ** 2).sum(axis=1)
    return laplacian_from_edges(n, lo, hi, np.exp(-d2 / sigma ** 2), shift=1e-2,
                                name=f"knn_{n}")


def knn_batch(count: int = 512, nmin: int = 1000, nmax: int = 200_000, seed: int = 1004,
              k: int = 8):
    """Config 4: ``count`` kNN Laplacians with sizes log-uniform in [nmin, nmax],
    one rhs ~ U[-1,1] each.  Returns (list of CSR, list of b)."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(nmin), np.log(nmax), count)).astype(np.int64)
    mats, rhs = [], []
    for s in sizes:
        mats.append(knn_graph(int(s), k, rng=rng))
        rhs.append(rng.uniform(-1.0, 1.0, int(s)))
    return mats, rhs


def multi_rhs(n: int, nrhs: int = 32, seed: int = 1005) -> np.ndarray:
    """32 right-hand sides ~ U[-1,1] for the 128^3 matrix, row-major [nrhs, n]."""
    return np.random.default_rng(seed).uniform(-1.0, 1.0, (nrhs, n))


# ---------------------------------------------------------------- Matrix Market

def write_mm(path: str, A: CSR) -> None:
    """Symmetric lower triangle (diagonal included) as 'coordinate real symmetric'."""
    rows = np.repeat(np.arange(A.n, dtype=np.int64), np.diff(A.ia))
    low = A.ja <= rows
    r, c, v = rows[low] + 1, A.ja[low].astype(np.int64) + 1, A.a[low]
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix coordinate real symmetric\n")
        f.write(f"{A.n} {A.n} {r.shape[0]}\n")
        np.savetxt(f, np.column_stack([r, c, v]), fmt=["%d", "%d", "%.17g"])


def write_rhs(path: str, b: np.ndarray) -> None:
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix array real general\n")
        f.write(f"{b.shape[0]} 1\n")
        np.savetxt(f, b, fmt="%.17g")


def write_adjacency(path: str, n: int, ei: np.ndarray, ej: np.ndarray,
                    w: np.ndarray | None = None) -> None:
    """Adjacency (one triangle) as 'coordinate pattern|real symmetric'."""
    lo, hi = np.maximum(ei, ej) + 1, np.minimum(ei, ej) + 1
    with open(path, "w") as f:
        kind = "pattern" if w is None else "real"
        f.write(f"%%MatrixMarket matrix coordinate {kind} symmetric\n")
        f.write(f"{n} {n} {lo.shape[0]}\n")
        if w is None:
            np.savetxt(f, np.column_stack([lo, hi]), fmt="%d")
        else:
            np.savetxt(f, np.column_stack([lo, hi, w]), fmt=["%d", "%d", "%.17g"])
