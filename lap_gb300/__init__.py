"""lap_gb300 -- GB300-native PCG for graph Laplacians behind LAP's C call surface.

The product is the C-ABI shared library ``lap_gb300/libgblap.so`` (built by
``python -m lap_gb300.build``; headers in ``include/``).  This module is a
thin ctypes binding over it, used by the tests, ``bench.py`` and Python
callers.  PyTorch only supplies device memory: every compute call goes
through libgblap's kernels, and there is no CPU or library fallback -- if the
shared library is missing the import of :func:`lib` raises.

Reference surface mirrored (LAP): ``cg`` (cg.c:5-140) with its ``pdata``
(common.h:29-50), the preconditioner names of prec.c:6-45, the cuda_*
backend of cuda_blas.h and devMem.h.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgblap.so")

PRECONDITIONERS = ("none", "line_jacobi", "it_jacobi", "GS_std", "GS_it", "GS_it2", "ichol")
STATUS = {0: "ok", 1: "maxit", 2: "breakdown", 3: "zero_pivot", 4: "timeout", 5: "bad_input",
          6: "cuda_error", 7: "no_memory", 8: "not_supported", 9: "internal"}

_lib: C.CDLL | None = None


class GbError(RuntimeError):
    def __init__(self, status: int, where: str = ""):
        self.status = status
        super().__init__(f"{where}: {STATUS.get(status, status)}")


class PcgOpts(C.Structure):
    _fields_ = [("tol", C.c_double), ("maxit", C.c_int), ("precision", C.c_int),
                ("inner_tol", C.c_double), ("max_outer", C.c_int), ("use_graph", C.c_int),
                ("verbose", C.c_int)]


class PcgResult(C.Structure):
    _fields_ = [("iters", C.c_int), ("outer", C.c_int), ("flag", C.c_int), ("status", C.c_int),
                ("res0", C.c_double), ("res", C.c_double), ("true_res", C.c_double),
                ("rel_true_res", C.c_double), ("device_ms", C.c_double)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class PData(C.Structure):
    """Layout-identical mirror of LAP's ``pdata`` (common.h:29-50)."""
    _fields_ = [("lia", C.c_void_p), ("lja", C.c_void_p), ("la", C.c_void_p), ("lnnz", C.c_int),
                ("uia", C.c_void_p), ("uja", C.c_void_p), ("ua", C.c_void_p), ("unnz", C.c_int),
                ("ichol_vals", C.c_void_p), ("d", C.c_void_p), ("d_r", C.c_void_p),
                ("n", C.c_int), ("aux_vec1", C.c_void_p), ("aux_vec2", C.c_void_p),
                ("aux_vec3", C.c_void_p), ("prec_op", C.c_char_p), ("m", C.c_int),
                ("k", C.c_int)]


class MMatrix(C.Structure):
    """Layout-identical mirror of LAP's ``mmatrix`` (io_utils.h:26-42)."""
    _fields_ = [("coo_rows", C.POINTER(C.c_int)), ("coo_cols", C.POINTER(C.c_int)),
                ("coo_vals", C.POINTER(C.c_double)), ("csr_ia", C.POINTER(C.c_int)),
                ("csr_ja", C.POINTER(C.c_int)), ("csr_vals", C.POINTER(C.c_double)),
                ("n", C.c_int), ("m", C.c_int), ("nnz", C.c_int), ("nnz_unpacked", C.c_int),
                ("symmetric", C.c_int)]


class MmCsr(C.Structure):
    """gb_mm_csr (include/gblap.h): a CSR matrix built on the device from a
    Matrix Market file."""
    _fields_ = [("n", C.c_int), ("m", C.c_int), ("nnz_file", C.c_longlong), ("nnz", C.c_int),
                ("symmetric", C.c_int), ("pattern", C.c_int),
                ("ia", C.c_void_p), ("ja", C.c_void_p), ("a", C.c_void_p),
                ("host_parsed", C.c_int), ("read_ms", C.c_double), ("h2d_ms", C.c_double),
                ("device_ms", C.c_double)]


def _proto(L: C.CDLL) -> None:
    vp, i, d = C.c_void_p, C.c_int, C.c_double
    sig = {
        "gb_status_str": (C.c_char_p, [i]),
        "gb_prec_from_name": (i, [C.c_char_p]),
        "gb_version": (C.c_char_p, []),
        "gb_system_create": (i, [i, i, vp, vp, vp, C.c_char_p, i, i, C.POINTER(vp)]),
        "gb_system_destroy": (i, [vp]),
        "gb_system_update_values": (i, [vp]),
        "gb_system_refresh_matrix": (i, [vp]),
        "gb_system_set_prec_values": (i, [vp, vp, vp, vp, i, vp, vp, vp, i, vp, vp]),
        "gb_system_pattern_hash": (i, [vp, i, i, vp, vp, C.POINTER(C.c_ulonglong)]),
        "gb_system_info": (i, [vp, C.POINTER(i), C.POINTER(i), C.POINTER(i)]),
        "gb_pcg_opts_default": (None, [C.POINTER(PcgOpts)]),
        "gb_pcg_solve": (i, [vp, vp, vp, C.POINTER(PcgOpts), vp, i, C.POINTER(PcgResult)]),
        "gb_pcg_solve_host": (i, [vp, vp, vp, C.POINTER(PcgOpts), C.POINTER(PcgResult)]),
        "gb_spmv": (i, [vp, d, vp, d, vp]),
        "gb_precond_apply": (i, [vp, vp, vp]),
        "gb_ichol_factor_values": (i, [vp, vp, vp]),
        "gb_adjoint_scatter": (i, [vp, vp, vp, vp, vp]),
        "gb_adjoint_grad": (i, [vp, vp, vp, vp, vp, vp, C.POINTER(PcgOpts), C.POINTER(PcgResult)]),
        "gb_batch_create": (i, [i, vp, vp, vp, vp, vp, C.c_char_p, C.POINTER(vp)]),
        "gb_batch_destroy": (i, [vp]),
        "gb_batch_solve": (i, [vp, vp, vp, C.POINTER(PcgOpts), vp, vp, C.POINTER(PcgResult)]),
        "gb_pcg_solve_multi": (i, [vp, i, vp, vp, C.POINTER(PcgOpts), vp, C.POINTER(PcgResult)]),
        "gb_autotune_spmv": (i, [vp, C.POINTER(i)]),
        "gb_batch_autotune": (i, [vp, vp, i, C.POINTER(i), C.POINTER(i), C.POINTER(d), C.POINTER(d)]),
        "gb_pcg_autotune_multi": (i, [vp, i, vp, i, C.POINTER(i), C.POINTER(d), C.POINTER(d)]),
        "gb_pcg_autotune_precision": (i, [vp, vp, vp, C.POINTER(i), vp]),
        "gb_debug_set_spin_budget": (i, [vp, C.c_ulonglong]),
        "gb_dot_noalloc": (i, [i, vp, vp, C.POINTER(C.c_double), vp]),
        "gb_mm_read_csr": (i, [C.c_char_p, C.POINTER(MmCsr)]),
        "gb_mm_parse_csr": (i, [C.c_char_p, C.c_longlong, C.POINTER(MmCsr)]),
        "gb_mm_csr_free": (i, [C.POINTER(MmCsr)]),
        "gb_mm_read_laplacian": (i, [C.c_char_p, i, i, C.POINTER(MmCsr)]),
        "gb_mm_parse_laplacian": (i, [C.c_char_p, C.c_longlong, i, i, C.POINTER(MmCsr)]),
        "gb_laplacian_rhs": (i, [i, vp, vp, vp, i, vp, vp]),
        "gb_profile_iteration": (i, [vp, vp, vp, i, i, C.c_char_p, i, vp, vp, i, C.POINTER(i)]),
        # LAP surface
        "cuda_dot": (d, [i, vp, vp]),
        "cuda_scal": (None, [i, d, vp]),
        "cuda_axpy": (None, [i, d, vp, vp]),
        "cuda_csr_matvec": (None, [i, i, vp, vp, vp, vp, vp, C.POINTER(d), C.POINTER(d)]),
        "cuda_lower_triangular_solve": (None, [i, i, vp, vp, vp, vp, vp, vp]),
        "cuda_upper_triangular_solve": (None, [i, i, vp, vp, vp, vp, vp, vp]),
        "cuda_vec_vec": (None, [i, vp, vp, vp]),
        "cuda_vector_sqrt": (None, [i, vp, vp]),
        "cuda_vector_reciprocal": (None, [i, vp, vp]),
        "cuda_vec_copy": (None, [i, vp, vp]),
        "cuda_vec_zero": (None, [i, vp]),
        "initialize_handles": (None, []),
        "initialize_ichol": (None, [i, i, vp, vp, vp]),
        "initialize_and_analyze_L_and_U_solve": (None, [i, i, vp, vp, vp, i, vp, vp, vp]),
        "initialize_spmv_buffer": (None, [i, i, vp, vp, vp, vp, vp, C.POINTER(d), C.POINTER(d)]),
        "initialize_L_and_U_descriptors": (None, [i, i, vp, vp, vp, i, vp, vp, vp]),
        "cuda_ichol": (None, [vp, vp, vp, i, C.POINTER(PData), vp, vp]),
        "mallocForDevice": (vp, [vp, i, i]),
        "memcpyDevice": (None, [vp, vp, i, i, C.c_char_p]),
        "freeDevice": (None, [vp]),
        "cg": (None, [i, d, vp, vp, vp, vp, vp, d, C.POINTER(PData), i, C.POINTER(i), C.POINTER(i), vp]),
        "prec_function": (None, [vp, vp, vp, i, C.POINTER(PData), vp, vp]),
        "read_mm_file": (None, [C.c_char_p, C.POINTER(MMatrix)]),
        "read_adjacency_file": (None, [C.c_char_p, C.POINTER(MMatrix)]),
        "coo_to_csr": (None, [C.POINTER(MMatrix)]),
        "read_rhs": (None, [C.c_char_p, vp]),
        "split": (None, [C.POINTER(MMatrix)] * 4),
        "create_L_and_split": (None, [C.POINTER(MMatrix)] * 4 + [i]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args


def lib() -> C.CDLL:
    """The loaded libgblap.so.  Raises if it has not been built: there is no fallback."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing; build it with `python -m lap_gb300.build`")
        L = C.CDLL(LIB_PATH)
        _proto(L)
        _lib = L
    return _lib


def check(rc: int, where: str) -> None:
    if rc != 0:
        raise GbError(rc, where)


def ptr(t) -> int:
    """Device address of a torch tensor (or 0 for None)."""
    return 0 if t is None else int(t.data_ptr())


def opts(tol=1e-8, maxit=10000, precision=0, inner_tol=0.0, max_outer=50, use_graph=True,
         verbose=False) -> PcgOpts:
    o = PcgOpts()
    lib().gb_pcg_opts_default(C.byref(o))
    o.tol, o.maxit, o.precision = tol, maxit, precision
    o.inner_tol, o.max_outer = inner_tol, max_outer
    o.use_graph, o.verbose = int(bool(use_graph)), int(bool(verbose))
    return o


class System:
    """A gb_system over a device CSR (torch int32 / float64 CUDA tensors)."""

    def __init__(self, ia, ja, a, prec: str = "line_jacobi", m: int = 1, k: int = 1):
        import torch

        self.ia = ia.to(device="cuda", dtype=torch.int32).contiguous()
        self.ja = ja.to(device="cuda", dtype=torch.int32).contiguous()
        self.a = a.to(device="cuda", dtype=torch.float64).contiguous()
        self.n = self.ia.numel() - 1
        self.nnz = self.ja.numel()
        self.prec = prec
        torch.cuda.synchronize()
        h = C.c_void_p()
        check(lib().gb_system_create(self.n, self.nnz, ptr(self.ia), ptr(self.ja), ptr(self.a),
                                     prec.encode(), m, k, C.byref(h)), "gb_system_create")
        self.h = h

    @classmethod
    def from_csr(cls, csr, prec="line_jacobi", m=1, k=1):
        import torch

        return cls(torch.from_numpy(csr.ia), torch.from_numpy(csr.ja), torch.from_numpy(csr.a),
                   prec, m, k)

    def close(self) -> None:
        if getattr(self, "h", None):
            lib().gb_system_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self) -> dict:
        lo, up, t = C.c_int(), C.c_int(), C.c_int()
        rc = lib().gb_system_info(self.h, C.byref(lo), C.byref(up), C.byref(t))
        return dict(lower_levels=lo.value, upper_levels=up.value, spmv_bundles=t.value, status=rc)

    def solve(self, b, x=None, hist_len: int = 0, **kw):
        """Solves A x = b on the device; returns (x, result dict[, history])."""
        import torch

        b = b.to(device="cuda", dtype=torch.float64).contiguous()
        x = torch.zeros_like(b) if x is None else x.to(device="cuda", dtype=torch.float64).contiguous().clone()
        o = opts(**kw)
        r = PcgResult()
        hist = np.zeros(max(hist_len, 1))
        torch.cuda.synchronize()
        rc = lib().gb_pcg_solve(self.h, ptr(b), ptr(x), C.byref(o),
                                hist.ctypes.data if hist_len else None, hist_len, C.byref(r))
        if rc not in (0, 4):
            raise GbError(rc, "gb_pcg_solve")
        out = r.as_dict()
        if hist_len:
            return x, out, hist[: min(hist_len, r.iters + 1)]
        return x, out

    def autotune_precision(self, b, **kw) -> dict:
        """gb_pcg_autotune_precision: the fastest converging precision mode
        for b, kept on the system (solve(..., precision=-1) uses it)."""
        import torch

        b = b.to(device="cuda", dtype=torch.float64).contiguous()
        o = opts(**kw)
        best = C.c_int(-1)
        ms = np.zeros(3)
        torch.cuda.synchronize()
        check(lib().gb_pcg_autotune_precision(self.h, ptr(b), C.byref(o), C.byref(best), ms.ctypes.data),
              "gb_pcg_autotune_precision")
        return dict(best=best.value, ms=[float(v) for v in ms])

    def solve_host(self, b: np.ndarray, x0: np.ndarray | None = None, **kw):
        """Same solve from/to host numpy arrays (copies inside the call)."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=np.float64)
        o = opts(**kw)
        r = PcgResult()
        rc = lib().gb_pcg_solve_host(self.h, b.ctypes.data, x.ctypes.data, C.byref(o), C.byref(r))
        if rc not in (0, 4):
            raise GbError(rc, "gb_pcg_solve_host")
        return x, r.as_dict()

    def spmv(self, x, y=None, alpha=1.0, beta=0.0):
        import torch

        y = torch.zeros_like(x) if y is None else y
        torch.cuda.synchronize()
        check(lib().gb_spmv(self.h, alpha, ptr(x), beta, ptr(y)), "gb_spmv")
        return y

    def precond(self, x):
        import torch

        y = torch.empty_like(x)
        torch.cuda.synchronize()
        check(lib().gb_precond_apply(self.h, ptr(x), ptr(y)), "gb_precond_apply")
        return y

    def ichol_factor_values(self):
        """(L values, U values) in LAP's CPU layout (diag last in L rows, first in U rows)."""
        import torch

        m = (self.nnz - self.n) // 2 + self.n
        lv = torch.empty(m, dtype=torch.float64, device="cuda")
        uv = torch.empty_like(lv)
        torch.cuda.synchronize()
        check(lib().gb_ichol_factor_values(self.h, ptr(lv), ptr(uv)), "gb_ichol_factor_values")
        return lv, uv

    def adjoint(self, x, g, edges: bool = True, **kw):
        """lambda = A^{-1} g, G = -lambda x^T on A's pattern, dL/dw per strict-lower entry."""
        import torch

        lam = torch.zeros_like(x)
        G = torch.empty(self.nnz, dtype=torch.float64, device="cuda")
        eg = torch.empty((self.nnz - self.n) // 2, dtype=torch.float64, device="cuda") if edges else None
        o = opts(**kw)
        r = PcgResult()
        torch.cuda.synchronize()
        check(lib().gb_adjoint_grad(self.h, ptr(x), ptr(g), ptr(lam), ptr(G), ptr(eg), C.byref(o),
                                    C.byref(r)), "gb_adjoint_grad")
        return lam, G, eg, r.as_dict()

    def set_values(self, a) -> None:
        """New matrix values on the same pattern (device tensor [nnz]); refactors
        the preconditioner (gb_system_update_values)."""
        import torch

        self.a.copy_(a.to(device="cuda", dtype=torch.float64))
        torch.cuda.synchronize()
        check(lib().gb_system_update_values(self.h), "gb_system_update_values")

    def autotune(self) -> int:
        best = C.c_int()
        check(lib().gb_autotune_spmv(self.h, C.byref(best)), "gb_autotune_spmv")
        return best.value

    def profile(self, b, precision=0, iters=20):
        """Per-kernel average device time (ms) and algorithmic bytes of one iteration."""
        import torch

        x = torch.zeros_like(b)
        names = C.create_string_buffer(1024)
        ms = np.zeros(32)
        by = np.zeros(32)
        cnt = C.c_int()
        torch.cuda.synchronize()
        check(lib().gb_profile_iteration(self.h, ptr(b), ptr(x), precision, iters, names, 1024,
                                         ms.ctypes.data, by.ctypes.data, 32, C.byref(cnt)),
              "gb_profile_iteration")
        k = cnt.value
        return [dict(name=nm, ms=float(ms[i]), bytes=float(by[i]))
                for i, nm in enumerate(names.value.decode().split(";")[:k])]


class Batch:
    """Many independent CSR systems solved together (gb_batch_*): the
    matrices are concatenated block-diagonally with system-local columns."""

    def __init__(self, mats, prec="line_jacobi"):
        import torch

        row_off = np.zeros(len(mats) + 1, dtype=np.int64)
        nnz_off = np.zeros(len(mats) + 1, dtype=np.int64)
        for s, A in enumerate(mats):
            row_off[s + 1] = row_off[s] + A.n
            nnz_off[s + 1] = nnz_off[s] + A.nnz
        ia = np.concatenate([A.ia[:-1] + nnz_off[s] for s, A in enumerate(mats)] + [nnz_off[-1:]])
        self.ia = torch.from_numpy(ia.astype(np.int32)).cuda()
        self.ja = torch.from_numpy(np.concatenate([A.ja for A in mats]).astype(np.int32)).cuda()
        self.a = torch.from_numpy(np.concatenate([A.a for A in mats]).astype(np.float64)).cuda()
        self.row_off, self.nnz_off = row_off, nnz_off
        self.count, self.N = len(mats), int(row_off[-1])
        h = C.c_void_p()
        check(lib().gb_batch_create(self.count, row_off.ctypes.data, nnz_off.ctypes.data, ptr(self.ia),
                                    ptr(self.ja), ptr(self.a), prec.encode(), C.byref(h)), "gb_batch_create")
        self.h = h

    def solve(self, b, x=None, **kw):
        """b, x: concatenated device vectors [N].  Returns (x, per-system
        iterations, per-system flags, aggregate result dict)."""
        import torch

        b = b.to(device="cuda", dtype=torch.float64).contiguous()
        x = torch.zeros_like(b) if x is None else x.to(device="cuda", dtype=torch.float64).contiguous().clone()
        o = opts(**kw)
        r = PcgResult()
        it = np.zeros(self.count, dtype=np.int32)
        fl = np.zeros(self.count, dtype=np.int32)
        torch.cuda.synchronize()
        check(lib().gb_batch_solve(self.h, ptr(b), ptr(x), C.byref(o), it.ctypes.data, fl.ctypes.data,
                                   C.byref(r)), "gb_batch_solve")
        return x, it, fl, r.as_dict()

    def autotune(self, b, iters: int = 16) -> dict:
        """gb_batch_autotune: times the row-bundle / chunk choices on this
        batch (right-hand side b) and applies the fastest."""
        import torch

        b = b.to(device="cuda", dtype=torch.float64).contiguous()
        rpb, cr, t0, t1 = C.c_int(), C.c_int(), C.c_double(), C.c_double()
        torch.cuda.synchronize()
        check(lib().gb_batch_autotune(self.h, ptr(b), iters, C.byref(rpb), C.byref(cr), C.byref(t0), C.byref(t1)),
              "gb_batch_autotune")
        return dict(rows_per_bundle=rpb.value, chunk_rows=cr.value, ms_default=t0.value, ms_best=t1.value)

    def split(self, v):
        """Per-system views of a concatenated vector."""
        return [v[self.row_off[s]:self.row_off[s + 1]] for s in range(self.count)]

    def close(self) -> None:
        if getattr(self, "h", None):
            lib().gb_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def read_mm_device(path=None, data: bytes | None = None, laplacian: dict | None = None):
    """A Matrix Market coordinate file (``path``, or its bytes ``data``) parsed
    into CSR on the device (gb_mm_read_csr / gb_mm_parse_csr).  With
    ``laplacian=dict(weighted=0|1, exact_degrees=0|1)`` the file is an
    adjacency matrix turned into its graph Laplacian (gb_mm_read_laplacian).
    Returns (ia, ja, a) as CUDA tensors and an info dict (sizes, flags,
    timings)."""
    import torch

    out = MmCsr()
    if laplacian is not None:
        w, ex = int(laplacian.get("weighted", 0)), int(laplacian.get("exact_degrees", 0))
        if data is not None:
            rc = lib().gb_mm_parse_laplacian(data, len(data), w, ex, C.byref(out))
        else:
            rc = lib().gb_mm_read_laplacian(os.fsencode(path), w, ex, C.byref(out))
    elif data is not None:
        rc = lib().gb_mm_parse_csr(data, len(data), C.byref(out))
    else:
        rc = lib().gb_mm_read_csr(os.fsencode(path), C.byref(out))
    check(rc, "gb_mm_read_csr")
    try:
        ia = torch.empty(out.n + 1, dtype=torch.int32, device="cuda")
        ja = torch.empty(max(out.nnz, 0), dtype=torch.int32, device="cuda")
        a = torch.empty(max(out.nnz, 0), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        _copy_dev(ia, out.ia, out.n + 1, 4)
        if out.nnz:
            _copy_dev(ja, out.ja, out.nnz, 4)
            _copy_dev(a, out.a, out.nnz, 8)
    finally:
        lib().gb_mm_csr_free(C.byref(out))
    info = {k: getattr(out, k) for k in ("n", "m", "nnz_file", "nnz", "symmetric", "pattern", "host_parsed",
                                         "read_ms", "h2d_ms", "device_ms")}
    return ia, ja, a, info


def laplacian_rhs(ia, ja, a, weighted=0):
    """The Laplacian driver's projected right-hand side (gb_laplacian_rhs)."""
    import torch

    n = ia.numel() - 1
    b = torch.empty(n, dtype=torch.float64, device="cuda")
    work = torch.empty(n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    check(lib().gb_laplacian_rhs(n, ptr(ia), ptr(ja), ptr(a), int(weighted), ptr(b), ptr(work)),
          "gb_laplacian_rhs")
    return b


def _copy_dev(dst, src_ptr, count, size):
    """Device-to-device copy of count elements of size bytes from a raw device
    pointer into a tensor (devMem's memcpyDevice)."""
    lib().memcpyDevice(C.c_void_p(dst.data_ptr()), C.c_void_p(src_ptr), count, size, b"D2D")


def solve_multi(system, B, X=None, **kw):
    """nrhs right-hand sides on one System (gb_pcg_solve_multi); B [nrhs, n]
    on the device.  Returns (X, per-column iterations, aggregate result)."""
    import torch

    B = B.to(device="cuda", dtype=torch.float64).contiguous()
    X = torch.zeros_like(B) if X is None else X.to(device="cuda", dtype=torch.float64).contiguous().clone()
    o = opts(**kw)
    r = PcgResult()
    it = np.zeros(B.shape[0], dtype=np.int32)
    torch.cuda.synchronize()
    check(lib().gb_pcg_solve_multi(system.h, B.shape[0], ptr(B), ptr(X), C.byref(o), it.ctypes.data,
                                   C.byref(r)), "gb_pcg_solve_multi")
    return X, it, r.as_dict()


def autotune_multi(system, B, iters: int = 16) -> dict:
    """gb_pcg_autotune_multi: columns per interleaved chunk for B [nrhs, n]
    on this System, chosen by timing and kept on the system."""
    import torch

    B = B.to(device="cuda", dtype=torch.float64).contiguous()
    w, t0, t1 = C.c_int(), C.c_double(), C.c_double()
    torch.cuda.synchronize()
    check(lib().gb_pcg_autotune_multi(system.h, B.shape[0], ptr(B), iters, C.byref(w), C.byref(t0), C.byref(t1)),
          "gb_pcg_autotune_multi")
    return dict(width=w.value, ms_default=t0.value, ms_best=t1.value)
