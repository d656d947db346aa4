"""ctypes bindings for the CPU oracle (TEST INFRASTRUCTURE ONLY).

``liboracle.so`` is our C restatement of LAP's serial PCG path (oracle.c);
``liboracle_omp.so`` the same with the SpMV and dot multithreaded as LAP's
OpenMP backend does; ``_ref/libref.so`` (present only where the LAP sources
were available to compile) is the reference's own code.  Only tests/,
``__graft_entry__.smoke()`` and bench.py's CPU-baseline legs use this module;
the product never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIBS: dict[str, C.CDLL] = {}

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def reference_dir() -> str | None:
    """Where LAP's sources are mounted: $LAP_REFERENCE_DIR, else the default
    mount point of this build's container; None where neither exists (the
    GPU hosts, which only run the prebuilt oracle)."""
    d = os.environ.get("LAP_REFERENCE_DIR") or "/root/reference"
    return d if os.path.isdir(d) else None


def build(ref_dir: str | None = None, quiet: bool = True) -> None:
    """Compile liboracle*.so (always) and _ref/libref.so (when ``ref_dir`` exists)."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.run(["make", "-C", HERE, "oracle"], check=True, stdout=out)
    if ref_dir and os.path.isdir(ref_dir):
        subprocess.run(["make", "-C", HERE, "ref", f"REF_DIR={ref_dir}"], check=True, stdout=out)


def _bind(lib: C.CDLL) -> C.CDLL:
    lib.orc_dot.restype = C.c_double
    lib.orc_dot.argtypes = [C.c_int, _dp, _dp]
    lib.orc_csr_matvec.argtypes = [C.c_int, C.c_int, _ip, _ip, _dp, _dp, _dp,
                                   C.POINTER(C.c_double), C.POINTER(C.c_double)]
    for nm in ("orc_lower_solve", "orc_upper_solve"):
        getattr(lib, nm).argtypes = [C.c_int, C.c_int, _ip, _ip, _dp, _dp, _dp, _dp]
    lib.orc_ichol_factor.argtypes = [C.c_int, C.c_int, _ip, _ip, _dp, _ip, _ip, _dp]
    lib.orc_vector_reciprocal.argtypes = [C.c_int, _dp, _dp]
    lib.orc_vector_sqrt.argtypes = [C.c_int, _dp, _dp]
    lib.orc_solve_csr.restype = C.c_int
    lib.orc_solve_csr.argtypes = [C.c_int, C.c_int, _ip, _ip, _dp, _dp, _dp, C.c_char_p,
                                  C.c_double, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int),
                                  _dp, C.POINTER(C.c_double), C.c_int,
                                  C.POINTER(C.c_double), C.POINTER(C.c_double)]
    lib.orc_num_threads.restype = C.c_int
    lib.orc_spmv_threads.restype = C.c_int
    lib.orc_prec_apply_csr.argtypes = [C.c_int, C.c_int, _ip, _ip, _dp, C.c_char_p, C.c_int,
                                       C.c_int, _dp, _dp]
    return lib


def lib(kind: str = "serial") -> C.CDLL:
    """Load the oracle: ``serial`` (default) or ``omp`` (multicore mirror)."""
    if kind not in _LIBS:
        name = {"serial": "liboracle.so", "omp": "liboracle_omp.so"}[kind]
        path = os.path.join(HERE, name)
        if not os.path.exists(path):
            build()
        _LIBS[kind] = _bind(C.CDLL(path))
    return _LIBS[kind]


def ref_lib() -> C.CDLL | None:
    """The reference's own NOACC code, or None when it was not built here."""
    if "ref" not in _LIBS:
        path = os.path.join(HERE, "_ref", "libref.so")
        if not os.path.exists(path):
            return None
        L = C.CDLL(path)
        L.ref_solve_csr.restype = C.c_int
        L.ref_solve_csr.argtypes = [C.c_int, C.c_int, _ip, _ip, _dp, _dp, _dp, C.c_char_p,
                                    C.c_double, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int),
                                    _dp, C.c_void_p, C.c_void_p]
        L.simple_csr_matvec.argtypes = [C.c_int, C.c_int, _ip, _ip, _dp, _dp, _dp,
                                        C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.simple_upper_triangular_solve.argtypes = [C.c_int, C.c_int, _ip, _ip, _dp, _dp, _dp, _dp]
        L.simple_lower_triangular_solve.argtypes = [C.c_int, C.c_int, _ip, _ip, _dp, _dp, _dp, _dp]
        _LIBS["ref"] = L
    return _LIBS["ref"]


# ------------------------------------------------------------------ helpers

def csr_matvec(n, ia, ja, a, x, y, alpha=1.0, beta=0.0, kind="serial"):
    """y = beta*y + alpha*A*x in the reference's operation order (in place on y)."""
    lib(kind).orc_csr_matvec(n, len(ja), ia, ja, a, x, y, C.byref(C.c_double(alpha)),
                             C.byref(C.c_double(beta)))
    return y


def split(n, ia, ja, a):
    """Strict lower, strict upper (CSR) and the diagonal (io_utils.c:268-363)."""
    rows = np.repeat(np.arange(n), np.diff(ia))
    lo, up, dg = ja < rows, ja > rows, ja == rows
    d = np.zeros(n)
    d[rows[dg]] = a[dg]

    def part(mask):
        cnt = np.bincount(rows[mask], minlength=n)
        p = np.zeros(n + 1, dtype=np.int32)
        np.cumsum(cnt, out=p[1:])
        return p, np.ascontiguousarray(ja[mask], dtype=np.int32), np.ascontiguousarray(a[mask])

    return part(lo), part(up), d


def lower_solve(n, lia, lja, la, diag, x):
    out = np.zeros(n)
    lib().orc_lower_solve(n, len(lja), lia, lja, la, diag, x, out)
    return out


def upper_solve(n, uia, uja, ua, diag, x):
    out = np.zeros(n)
    lib().orc_upper_solve(n, len(uja), uia, uja, ua, diag, x, out)
    return out


def embed_diagonal(n, L, U, d):
    """Diagonal last in each L row, first in each U row (cg_driver2.c:95-196)."""
    (lia, lja, la), (uia, uja, ua) = L, U
    rows_l = np.repeat(np.arange(n), np.diff(lia))
    rows_u = np.repeat(np.arange(n), np.diff(uia))
    # stable sort by (row, is_diag) puts the diagonal last for L
    rl = np.concatenate([rows_l, np.arange(n)])
    cl = np.concatenate([lja, np.arange(n, dtype=np.int32)])
    vl = np.concatenate([la, d])
    ol = np.lexsort((np.concatenate([np.zeros_like(rows_l), np.ones(n, dtype=np.int64)]), rl))
    ru = np.concatenate([np.arange(n), rows_u])
    cu = np.concatenate([np.arange(n, dtype=np.int32), uja])
    vu = np.concatenate([d, ua])
    ou = np.lexsort((np.concatenate([np.zeros(n, dtype=np.int64), np.ones_like(rows_u)]), ru))
    lia2 = (lia + np.arange(n + 1)).astype(np.int32)
    uia2 = (uia + np.arange(n + 1)).astype(np.int32)
    return ((lia2, np.ascontiguousarray(cl[ol], dtype=np.int32), np.ascontiguousarray(vl[ol])),
            (uia2, np.ascontiguousarray(cu[ou], dtype=np.int32), np.ascontiguousarray(vu[ou])))


def ichol_factor(n, ia, ja, a):
    """IC(0) factor of A in the reference's layout: (L with diagonal last, U=L^T
    with diagonal first), via simple_blas.c:139-182 restated."""
    L, U, d = split(n, ia, ja, a)
    (lia, lja, la), (uia, uja, ua) = embed_diagonal(n, L, U, d)
    ua = ua.copy()
    la = la.copy()
    lib().orc_ichol_factor(n, len(uja), uia, uja, ua, lia, lja, la)
    return (lia, lja, la), (uia, uja, ua)


def solve(n, ia, ja, a, b, prec="line_jacobi", tol=1e-8, maxit=10000, M=1, K=1,
          x0=None, kind="serial", max_iters_run=0):
    """CPU PCG exactly as LAP's NOACC cg_driver2 path runs it.

    Returns dict(x, iters, flag, res_hist, true_res, setup_s, solve_s)."""
    x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64)
    hist = np.zeros(maxit + 3)
    flag, tr, su, so = C.c_int(0), C.c_double(0.0), C.c_double(0.0), C.c_double(0.0)
    it = lib(kind).orc_solve_csr(n, len(ja), np.ascontiguousarray(ia, dtype=np.int32),
                                 np.ascontiguousarray(ja, dtype=np.int32),
                                 np.ascontiguousarray(a, dtype=np.float64),
                                 np.ascontiguousarray(b, dtype=np.float64), x,
                                 prec.encode(), tol, maxit, M, K, C.byref(flag), hist,
                                 C.byref(tr), max_iters_run, C.byref(su), C.byref(so))
    return dict(x=x, iters=it, flag=flag.value, res_hist=hist[: it + 1].copy(),
                true_res=tr.value, setup_s=su.value, solve_s=so.value)


def prec_apply(n, ia, ja, a, x, prec, M=1, K=1):
    """y = M^{-1} x: one prec_function call after the NOACC driver's setup."""
    y = np.zeros(n)
    lib().orc_prec_apply_csr(n, len(ja), np.ascontiguousarray(ia, dtype=np.int32),
                             np.ascontiguousarray(ja, dtype=np.int32),
                             np.ascontiguousarray(a, dtype=np.float64), prec.encode(), M, K,
                             np.ascontiguousarray(x, dtype=np.float64), y)
    return y


def ref_solve(n, ia, ja, a, b, prec="line_jacobi", tol=1e-8, maxit=10000, M=1, K=1):
    """Same as :func:`solve` but through the reference's own compiled cg()."""
    L = ref_lib()
    if L is None:
        raise RuntimeError("reference library not built (oracle/_ref/libref.so)")
    x = np.zeros(n)
    hist = np.zeros(maxit + 3)
    flag = C.c_int(0)
    ia = np.ascontiguousarray(ia, dtype=np.int32).copy()
    ja = np.ascontiguousarray(ja, dtype=np.int32).copy()
    a = np.ascontiguousarray(a, dtype=np.float64).copy()
    bb = np.ascontiguousarray(b, dtype=np.float64).copy()
    it = L.ref_solve_csr(n, len(ja), ia, ja, a, bb, x, prec.encode(), tol, maxit, M, K,
                         C.byref(flag), hist, None, None)
    return dict(x=x, iters=it, flag=flag.value, res_hist=hist[: it + 1].copy())


# ---------------------------------------------------------------- Matrix Market
_NUM_PREFIX = None


def _strtod_prefix(tok: str) -> float:
    """The value strtod reads from the start of ``tok`` (sscanf's %lf): the
    longest decimal (or inf / nan) prefix, correctly rounded as glibc does --
    Python's float() rounds decimals the same way."""
    global _NUM_PREFIX
    import re

    if _NUM_PREFIX is None:
        _NUM_PREFIX = re.compile(r"[+-]?(?:inf(?:inity)?|nan|(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?)", re.I)
    m = _NUM_PREFIX.match(tok)
    if not m:
        raise ValueError(f"no number in {tok!r}")
    return float(m.group(0))


def mm_csr(data: bytes, adjacency: bool = False):
    """read_mm_file (io_utils.c:15-74) + coo_to_csr (io_utils.c:141-235) on
    the bytes of a Matrix Market coordinate file, restated in Python/numpy.

    Banner flags 'pattern' / 'symmetric' (io_utils.c:24-35), '%' comment
    lines and the size line (:37-44); one entry per data line "r c [v]",
    1-based (:55-70), where this restatement skips '%' and blank lines and
    stops at the announced count; a symmetric file's off-diagonal entries
    mirrored (:150-157, :177-194); rows bucketed in encounter order, then each
    row sorted by column with equal columns kept in that order (:199-210, the
    reference's qsort being glibc's merge sort here).
    adjacency=True follows read_adjacency_file (io_utils.c:82-138) instead:
    symmetric whatever the banner says, and one unit diagonal entry per
    vertex after the file's entries.
    Returns (n, m, symmetric, ia, ja, a)."""
    text = data.decode("ascii", errors="replace")
    lines = text.split("\n")
    banner = lines[0]
    pattern = "pattern" in banner
    symmetric = "symmetric" in banner or adjacency
    k = 1
    while k < len(lines) and lines[k].startswith("%"):
        k += 1
    n, m, nnz = (int(t) for t in lines[k].split()[:3])
    rows, cols, vals = [], [], []
    for line in lines[k + 1:]:
        if len(rows) == nnz:
            break
        s = line.strip(" \t\r")
        if not s or s.startswith("%"):
            continue
        parts = s.split()
        r, c = int(parts[0]), int(parts[1])
        if not (1 <= r <= n and 1 <= c <= m):
            raise ValueError(f"entry out of range: {s!r}")
        rows.append(r - 1)
        cols.append(c - 1)
        vals.append(1.0 if pattern else _strtod_prefix(parts[2]))
    if len(rows) < nnz:
        raise ValueError(f"file ended after {len(rows)} of {nnz} entries")
    if adjacency:
        rows += list(range(n))
        cols += list(range(n))
        vals += [1.0] * n
    r = np.array(rows, dtype=np.int64)
    c = np.array(cols, dtype=np.int64)
    v = np.array(vals, dtype=np.float64)
    if symmetric:
        off = r != c
        # encounter order: each entry, then its mirror
        er = np.empty(2 * len(r), dtype=np.int64)
        ec = np.empty_like(er)
        ev = np.empty(2 * len(r))
        keep = np.ones(2 * len(r), dtype=bool)
        er[0::2], ec[0::2], ev[0::2] = r, c, v
        er[1::2], ec[1::2], ev[1::2] = c, r, v
        keep[1::2] = off
        r, c, v = er[keep], ec[keep], ev[keep]
    order = np.lexsort((c, r))  # stable: ties keep encounter order
    r, c, v = r[order], c[order], v[order]
    ia = np.zeros(n + 1, dtype=np.int32)
    np.cumsum(np.bincount(r, minlength=n), out=ia[1:])
    return n, m, symmetric, ia, c.astype(np.int32), v


def laplacian_csr(data: bytes, weighted: int = 0, exact_degrees: int = 0):
    """The Laplacian driver's matrix (cg_driver.c:38-45): read_adjacency_file
    + coo_to_csr (mm_csr(adjacency=True)), then create_L_and_split's
    in-place Laplacian (io_utils.c:367-491).  Degrees are summed into an int
    as the reference does, every partial sum truncated toward zero
    (io_utils.c:387-395), unless exact_degrees.  Returns (n, ia, ja, a)."""
    n, _, _, ia, ja, a = mm_csr(data, adjacency=True)
    a = a.copy()
    deg = np.zeros(n)
    for i in range(n):
        if exact_degrees:
            d = -1.0
            for k in range(ia[i], ia[i + 1]):
                d += a[k]
        else:
            d = -1
            for k in range(ia[i], ia[i + 1]):
                d = int(d + a[k])  # C: int += double truncates toward zero
        deg[i] = d
    out = a.copy()
    one = np.float64(1.0)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):  # IEEE results, as C gives
        for i in range(n):
            dsq = one / np.sqrt(np.float64(deg[i])) if weighted else 0.0
            for k in range(ia[i], ia[i + 1]):
                c = ja[k]
                if c == i:
                    out[k] = 1.0 if weighted else deg[i]
                elif not weighted:
                    out[k] = -1.0 * a[k]
                else:
                    out[k] = (np.float64(-1.0) * a[k]) * dsq * (one / np.sqrt(np.float64(deg[c])))
    return n, ia, ja, out


def laplacian_rhs(n, diag, weighted=0):
    """cg_driver.c:159-230: b_i = (-1)^i minus its component along e/sqrt(n)
    (unweighted) or sqrt(d)/||sqrt(d)|| (weighted); numpy sums, so the last
    bits may differ from a device dot."""
    b = np.where(np.arange(n) % 2, -1.0, 1.0)
    if not weighted:
        e = np.ones(n) * (1.0 / np.sqrt(n))
    else:
        e = np.sqrt(np.asarray(diag, dtype=np.float64))
        e = e * (1.0 / np.sqrt(np.dot(e, e)))
    return b - np.dot(e, b) * e
