"""GPU parity of the individual kernels through the C ABI (LAP's cuda_* surface
and the gb_* API) against fixtures produced by the reference.

SpMV, the triangular solves and the IC(0) factor keep the reference's
operation order, so they are compared bit-exactly; reductions (dot) are
compared at 1e-14 relative.
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


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


# Matrices whose rows exceed the staging sizes (SpMV rows > 512 entries in a
# 32-row bundle, triangular rows > 32 dependencies) are reduced by a warp tree:
# same value up to summation order.  Everything else must be bit-identical.
LONG_ROW_CASES = {"chunglu"}


def same(got, want, name):
    if name in LONG_ROW_CASES:
        np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-14 * np.abs(want).max())
    else:
        assert np.array_equal(got, want)


@pytest.fixture(scope="module")
def L():
    return gb.lib()


def test_kat_spmv_fixture(L):
    a = dev(np.array([1.0, 2.0, 3.0, 7.0, 4.0, 1.0, 2.0, 3.0, 1.0, 9.0]))
    ja = dev(np.array([0, 1, 2, 1, 2, 3, 4, 3, 4, 4], dtype=np.int32))
    ia = dev(np.array([0, 3, 4, 7, 9, 10], dtype=np.int32))
    x = dev(np.arange(1.0, 6.0))
    y = dev(np.ones(5))
    L.cuda_csr_matvec(5, 10, gb.ptr(ia), gb.ptr(ja), gb.ptr(a), gb.ptr(x), gb.ptr(y),
                      C.byref(C.c_double(-2.0)), C.byref(C.c_double(1.5)))
    assert np.array_equal(host(y), [-26.5, -26.5, -50.5, -32.5, -88.5])


def test_kat_trisolve_fixture(L):
    # test_tri_solve_omp.c fixture with the diagonal embedded first in each U row
    ua = np.array([1.0, 2.0, 3.0, 7.0, 4.0, 1.0, 2.0, 3.0, 1.0, 9.0])
    uja = np.array([0, 1, 2, 1, 2, 3, 4, 3, 4, 4], dtype=np.int32)
    uia = np.array([0, 3, 4, 7, 9, 10], dtype=np.int32)
    x, y = dev(np.full(5, 8.0)), dev(np.zeros(5))
    d_uia, d_uja, d_ua = dev(uia), dev(uja), dev(ua)
    L.cuda_upper_triangular_solve(5, 10, gb.ptr(d_uia), gb.ptr(d_uja), gb.ptr(d_ua), 0, gb.ptr(x), gb.ptr(y))
    np.testing.assert_array_equal(host(y), oracle.upper_solve(
        5, np.array([0, 2, 2, 4, 5, 5], dtype=np.int32), np.array([1, 2, 3, 4, 4], dtype=np.int32),
        np.array([2.0, 3.0, 1.0, 2.0, 1.0]), np.array([1.0, 7.0, 4.0, 3.0, 9.0]), np.full(5, 8.0)))


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_spmv_bit_exact(golden, L, name):
    n, ia, ja, a, _ = golden_matrix(golden, name)
    xs, y0 = golden[f"{name}_spmv_x"], golden[f"{name}_spmv_y0"]
    dia, dja, da, dx = dev(ia), dev(ja), dev(a), dev(xs)
    sysm = gb.System(dia, dja, da, "line_jacobi")
    for tag, (al, be) in {"spmv": (1.0, 0.0), "spmv_ab": (-1.0, 1.0), "spmv_odd": (0.37, -2.5)}.items():
        y = dev(y0.copy())
        L.cuda_csr_matvec(n, len(ja), gb.ptr(dia), gb.ptr(dja), gb.ptr(da), gb.ptr(dx), gb.ptr(y),
                          C.byref(C.c_double(al)), C.byref(C.c_double(be)))
        same(host(y), golden[f"{name}_{tag}_y"], name)
        y2 = sysm.spmv(dx, dev(y0.copy()), al, be)
        same(host(y2), golden[f"{name}_{tag}_y"], name)
    sysm.close()


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_trisolve_bit_exact(golden, L, name):
    n, ia, ja, a, _ = golden_matrix(golden, name)
    Lp, Up, d = oracle.split(n, ia, ja, a)
    (lia, lja, la), (uia, uja, ua) = oracle.embed_diagonal(n, Lp, Up, d)
    xs = dev(golden[f"{name}_spmv_x"])
    for (p, j, v, fn, key) in ((lia, lja, la, L.cuda_lower_triangular_solve, "lsolve"),
                               (uia, uja, ua, L.cuda_upper_triangular_solve, "usolve")):
        dp, dj, dv, y = dev(p), dev(j), dev(v), dev(np.zeros(n))
        fn(n, len(j), gb.ptr(dp), gb.ptr(dj), gb.ptr(dv), 0, gb.ptr(xs), gb.ptr(y))
        same(host(y), golden[f"{name}_{key}"], name)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_ichol_factor_bit_exact(golden, name):
    n, ia, ja, a, _ = golden_matrix(golden, name)
    sysm = gb.System(dev(ia), dev(ja), dev(a), "ichol")
    lv, uv = sysm.ichol_factor_values()
    assert np.array_equal(host(lv), golden[f"{name}_ichol_L"])
    assert np.array_equal(host(uv), golden[f"{name}_ichol_U"])
    sysm.close()


@pytest.mark.parametrize("name", ["grid2d", "chunglu"])
def test_initialize_ichol_dropin(golden, L, name):
    """LAP's 5-argument GPU initialize_ichol: L lands in A's lower triangle in place."""
    n, ia, ja, a, _ = golden_matrix(golden, name)
    dia, dja, da = dev(ia), dev(ja), dev(a.copy())
    L.initialize_ichol(n, len(ja), gb.ptr(dia), gb.ptr(dja), gb.ptr(da))
    f = host(da)
    rows = np.repeat(np.arange(n), np.diff(ia))
    low = ja <= rows
    assert np.array_equal(f[low], golden[f"{name}_ichol_L"])
    assert np.array_equal(f[~low], a[~low])  # upper triangle untouched (csric02 contract)
    # cuda_ichol applies (L L^T)^{-1} from ichol_vals on A's pattern
    x = golden[f"{name}_spmv_x"]
    p = gb.PData()
    p.n = n
    aux = dev(np.zeros(n))
    p.aux_vec1 = gb.ptr(aux)
    p.ichol_vals = gb.ptr(da)
    dx, dy = dev(x), dev(np.zeros(n))
    L.cuda_ichol(gb.ptr(dia), gb.ptr(dja), gb.ptr(da), len(ja), C.byref(p), gb.ptr(dx), gb.ptr(dy))
    (lia, lja, la), (uia, uja, ua) = oracle.ichol_factor(n, ia, ja, a)
    op = oracle.lib()
    t = np.zeros(n)
    pd = oracle_pdata(n, lia, lja, la, uia, uja, ua, t)
    yref = np.zeros(n)
    op.orc_ichol_apply(C.byref(pd), x.ctypes.data_as(C.c_void_p), yref.ctypes.data_as(C.c_void_p))
    same(host(dy), yref, name)


def oracle_pdata(n, lia, lja, la, uia, uja, ua, aux):
    class OP(C.Structure):
        _fields_ = [("lia", C.c_void_p), ("lja", C.c_void_p), ("la", C.c_void_p), ("lnnz", C.c_int),
                    ("uia", C.c_void_p), ("uja", C.c_void_p), ("ua", C.c_void_p), ("unnz", C.c_int),
                    ("ichol_vals", C.c_void_p), ("d", C.c_void_p), ("d_r", C.c_void_p), ("n", C.c_int),
                    ("aux_vec1", C.c_void_p), ("aux_vec2", C.c_void_p), ("aux_vec3", C.c_void_p),
                    ("prec_op", C.c_char_p), ("m", C.c_int), ("k", C.c_int)]
    p = OP()
    p.n = n
    p.lia, p.lja, p.la = lia.ctypes.data, lja.ctypes.data, la.ctypes.data
    p.uia, p.uja, p.ua = uia.ctypes.data, uja.ctypes.data, ua.ctypes.data
    p.aux_vec1 = aux.ctypes.data
    oracle_pdata.keep = (lia, lja, la, uia, uja, ua, aux)
    return p


def test_blas1_against_numpy(L):
    rng = np.random.default_rng(3)
    n = 100_003
    v, w = rng.standard_normal(n), rng.standard_normal(n)
    dv, dw = dev(v), dev(w)
    d = L.cuda_dot(n, gb.ptr(dv), gb.ptr(dw))
    assert abs(d - v @ w) <= 1e-13 * np.abs(v * w).sum()
    y = dev(w.copy())
    L.cuda_axpy(n, 0.3, gb.ptr(dv), gb.ptr(y))
    assert np.array_equal(host(y), w + 0.3 * v)
    L.cuda_scal(n, -1.7, gb.ptr(y))
    assert np.array_equal(host(y), (w + 0.3 * v) * -1.7)
    r = dev(np.zeros(n))
    vv = v.copy()
    vv[::7] = 0.0
    L.cuda_vector_reciprocal(n, gb.ptr(dev(vv)), gb.ptr(r))
    ref = np.zeros(n)
    oracle.lib().orc_vector_reciprocal(n, vv, ref)
    assert np.array_equal(host(r), ref)
    L.cuda_vector_sqrt(n, gb.ptr(dv), gb.ptr(r))
    ref2 = np.zeros(n)
    oracle.lib().orc_vector_sqrt(n, v, ref2)
    assert np.array_equal(host(r), ref2)
    L.cuda_vec_vec(n, gb.ptr(dv), gb.ptr(dw), gb.ptr(r))
    assert np.array_equal(host(r), v * w)
    L.cuda_vec_copy(n, gb.ptr(dv), gb.ptr(r))
    assert np.array_equal(host(r), v)
    L.cuda_vec_zero(n, gb.ptr(r))
    assert not host(r).any()
    assert L.cuda_dot(0, gb.ptr(dv), gb.ptr(dw)) == 0.0


def test_devmem_roundtrip(L):
    n = 1000
    p = L.mallocForDevice(None, n, 8)
    assert p
    src = np.arange(n, dtype=np.float64)
    out = np.zeros(n)
    L.memcpyDevice(p, src.ctypes.data, n, 8, b"H2D")
    q = L.mallocForDevice(None, n, 8)
    L.memcpyDevice(q, p, n, 8, b"D2D")  # a real device-to-device copy
    L.memcpyDevice(out.ctypes.data, q, n, 8, b"D2H")
    assert np.array_equal(out, src)
    L.freeDevice(p)
    L.freeDevice(q)
