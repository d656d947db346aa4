"""The seeded synthetic workloads against their definitions: sizes and
non-zero counts by the grid formulas (n + 2·(edges)), symmetry, the
Laplacian structure A = D_w - W + shift (rows sum to the shift), stored
diagonals, sorted columns, value ranges, and determinism per seed.  The
full-size configurations follow from the same formulas: 256^2 gives
326,656 entries, 128^3 14,581,760 and 1024^2 5,238,784."""
import numpy as np
import pytest

from lap_gb300 import gen


def _check_laplacian(A, shift=0.0, shift_rel=0.0):
    n = A.n
    assert A.ia.shape == (n + 1,) and A.ia[0] == 0 and A.ia[-1] == A.ja.shape[0] == A.a.shape[0]
    rows = np.repeat(np.arange(n), np.diff(A.ia))
    # sorted, unique columns with the diagonal stored in every row
    key = rows.astype(np.int64) * n + A.ja
    assert np.all(np.diff(key) > 0)
    diag = A.a[rows == A.ja]
    assert diag.shape == (n,)
    # symmetric values
    import scipy.sparse as sp
    M = sp.csr_matrix((A.a, A.ja, A.ia), shape=(n, n))
    assert abs(M - M.T).max() == 0.0
    off = A.a[rows != A.ja]
    assert np.all(off < 0.0)
    # rows sum to the shift: D_w (1 + shift_rel) + shift - W
    deg = -np.bincount(rows[rows != A.ja], weights=off, minlength=n)
    np.testing.assert_allclose(M.sum(axis=1).A1, shift + shift_rel * deg, rtol=1e-12, atol=1e-12)
    return M


def _formula_nnz(n, edges):
    return n + 2 * edges


@pytest.mark.parametrize("side", [4, 16])
def test_grid2d_unit(side):
    A, b = gen.grid2d_unit(side, seed=1001)
    assert A.n == side * side
    assert A.ja.shape[0] == _formula_nnz(A.n, 2 * side * (side - 1))
    M = _check_laplacian(A, shift=1e-2)
    assert set(np.unique(M.data[M.data < 0])) == {-1.0}
    assert abs(b.mean()) < 1e-14 and np.all(np.abs(b) <= 2.0)  # U[-1,1] less its mean
    assert _formula_nnz(256 * 256, 2 * 256 * 255) == 326_656


@pytest.mark.parametrize("side", [3, 8])
def test_grid3d_lognormal(side):
    A, b = gen.grid3d_lognormal(side, seed=1002)
    assert A.n == side ** 3
    assert A.ja.shape[0] == _formula_nnz(A.n, 3 * side * side * (side - 1))
    _check_laplacian(A, shift=1e-3)
    A2, b2 = gen.grid3d_lognormal(side, seed=1002)
    assert np.array_equal(A.a, A2.a) and np.array_equal(b, b2)
    assert _formula_nnz(128 ** 3, 3 * 128 * 128 * 127) == 14_581_760


def test_grid2d_aniso_and_its_edge_list():
    side = 12
    A, b, xs = gen.grid2d_aniso(side, seed=1006)
    assert A.ja.shape[0] == _formula_nnz(A.n, 2 * side * (side - 1))
    M = _check_laplacian(A, shift=1e-2)
    ei, ej, w = gen.grid2d_aniso_edges(side, seed=1006)
    # the edge list is the same matrix, weights drawn in the same order
    B = gen.laplacian_from_edges(A.n, ei, ej, w, shift=1e-2)
    assert np.array_equal(A.ia, B.ia) and np.array_equal(A.ja, B.ja)
    np.testing.assert_allclose(A.a, B.a, rtol=1e-15)
    # vertical weights are a tenth of a lognormal(0,1) draw: their median sits
    # well below the horizontal ones'
    nh = side * (side - 1)
    assert np.median(w[nh:]) < 0.3 * np.median(w[:nh])
    assert _formula_nnz(1024 * 1024, 2 * 1024 * 1023) == 5_238_784


def test_chung_lu_small():
    A, b = gen.chung_lu(1 << 12, seed=1003)
    M = _check_laplacian(A, shift_rel=1e-3)
    deg = np.diff(A.ia) - 1
    assert deg.min() >= 1  # isolated vertices were removed
    assert A.n <= 1 << 12
    assert deg.max() > 20 * np.median(deg)  # power-law hubs
    # a random labelling: a hub's neighbours are spread over the index range
    hub = int(np.argmax(deg))
    cols = A.ja[A.ia[hub]:A.ia[hub + 1]]
    assert np.ptp(cols) > 0.8 * A.n
    assert np.all(M.data[M.data < 0] >= -1.0)
    A2, b2 = gen.chung_lu(1 << 12, seed=1003)
    assert np.array_equal(A.ja, A2.ja) and np.array_equal(b, b2)


def test_knn_batch_sizes():
    mats, rhs = gen.knn_batch(count=4, nmin=50, nmax=400, seed=1004)
    assert len(mats) == len(rhs) == 4
    for A, b in zip(mats, rhs):
        assert 50 <= A.n <= 400 and b.shape == (A.n,)
        _check_laplacian(A, shift=1e-2)
        assert np.diff(A.ia).min() >= 1 + 8  # at least k neighbours (union of kNN)


def test_multi_rhs_layout():
    B = gen.multi_rhs(100, 7, seed=1005)
    assert B.shape == (7, 100) and np.all(np.abs(B) <= 1.0)
    assert np.array_equal(B, gen.multi_rhs(100, 7, seed=1005))
