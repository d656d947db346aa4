"""Matrix Market -> CSR on the device (gb_mm_read_csr / gb_mm_parse_csr)
against the oracle's restatement of read_mm_file + coo_to_csr, itself pinned
to the reference's reader (tests/test_oracle.py): ia, ja and the values'
bit patterns must be identical."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a GPU", allow_module_level=True)

import lap_gb300 as gb  # noqa: E402
import mm_cases  # noqa: E402
import oracle  # noqa: E402
from conftest import ROOT  # noqa: E402
from lap_gb300 import gen  # noqa: E402


def _same(text_or_bytes, **kw):
    data = text_or_bytes if isinstance(text_or_bytes, bytes) else text_or_bytes.encode()
    ia, ja, a, info = gb.read_mm_device(data=data)
    n, m, sym, oia, oja, oa = oracle.mm_csr(data)
    assert (info["n"], info["m"], bool(info["symmetric"])) == (n, m, sym)
    assert np.array_equal(ia.cpu().numpy(), oia)
    assert np.array_equal(ja.cpu().numpy(), oja)
    got = a.cpu().numpy()
    bad = np.nonzero(got.view(np.int64) != oa.view(np.int64))[0]
    assert bad.size == 0, (bad[:5], got[bad[:5]], oa[bad[:5]])
    return info


def test_reference_fixture(golden):
    """grid6.mtx against the CSR the reference's own reader produced."""
    path = f"{ROOT}/tests/golden/grid6.mtx"
    ia, ja, a, info = gb.read_mm_device(path)
    assert info["symmetric"] == 1 and info["n"] == 36 and info["host_parsed"] == 0
    assert np.array_equal(ia.cpu().numpy(), golden["mm_ia"])
    assert np.array_equal(ja.cpu().numpy(), golden["mm_ja"])
    assert np.array_equal(a.cpu().numpy().view(np.int64), golden["mm_a"].view(np.int64))


@pytest.mark.parametrize("kind", ["general", "symmetric", "pattern", "comments"])
def test_stress_texts(kind):
    text = {"general": mm_cases.general_text(), "symmetric": mm_cases.symmetric_text(),
            "pattern": mm_cases.pattern_text(),
            "comments": mm_cases.with_comments_and_blanks(mm_cases.general_text(seed=5))}[kind]
    info = _same(text)
    if kind == "general":
        assert info["host_parsed"] > 0  # the spellings outside the exact path went to strtod


def test_values_round_like_strtod():
    """200k random spellings (repr, %.17g, %.6e, %g, integers, 1-19 digit
    mantissas with exponents in [-40, 40]): every value's bits equal
    Python's correctly rounded float(), which is what strtod returns."""
    rng = np.random.default_rng(7)
    vals = mm_cases.value_strings(rng, 200_000)
    n = 1000
    lines = ["%%MatrixMarket matrix coordinate real general", f"{n} {n} {len(vals)}"]
    r = rng.integers(1, n + 1, len(vals))
    c = rng.integers(1, n + 1, len(vals))
    lines += [f"{r[i]} {c[i]} {v}" for i, v in enumerate(vals)]
    info = _same("\n".join(lines) + "\n")
    assert info["host_parsed"] < 0.2 * len(vals)


def test_generated_laplacian_file(tmp_path):
    """A 12^3 lognormal Laplacian written as the benchmark writes its files."""
    A, _ = gen.grid3d_lognormal(12, seed=1002)
    p = tmp_path / "g12.mtx"
    gen.write_mm(str(p), A)
    ia, ja, a, info = gb.read_mm_device(str(p))
    assert info["host_parsed"] == 0 and info["nnz"] == len(A.ja)
    assert np.array_equal(ia.cpu().numpy(), A.ia) and np.array_equal(ja.cpu().numpy(), A.ja)
    assert np.array_equal(a.cpu().numpy(), A.a)  # %.17g round-trips exactly
    _same(p.read_bytes())


def _same_file(tmp_path, data, name="t.mtx"):
    """The file path (header read, chunked reader threads) against the
    oracle on the same bytes."""
    p = tmp_path / name
    p.write_bytes(data)
    ia, ja, a, info = gb.read_mm_device(str(p))
    n, m, sym, oia, oja, oa = oracle.mm_csr(data)
    assert (info["n"], info["m"], bool(info["symmetric"])) == (n, m, sym)
    assert np.array_equal(ia.cpu().numpy(), oia) and np.array_equal(ja.cpu().numpy(), oja)
    assert np.array_equal(a.cpu().numpy().view(np.int64), oa.view(np.int64))
    return info


@pytest.fixture(scope="module")
def g64_file(tmp_path_factory):
    A, _ = gen.grid3d_lognormal(64, seed=1011)
    p = tmp_path_factory.mktemp("mm") / "g64.mtx"
    gen.write_mm(str(p), A)
    return A, p


@pytest.mark.parametrize("threads", ["1", "2", "8"])
def test_file_reader_chunks(g64_file, monkeypatch, threads):
    """A 34 MB file (nine 4 MB chunks; with 2 threads each reuses its two
    staging chunks) gives the same CSR with 1, 2 or 8 reader threads."""
    monkeypatch.setenv("GBLAP_MM_READ_THREADS", threads)
    A, p = g64_file
    assert p.stat().st_size > 8 * (4 << 20)
    ia, ja, a, info = gb.read_mm_device(str(p))
    assert info["host_parsed"] == 0 and info["nnz"] == len(A.ja)
    assert np.array_equal(ia.cpu().numpy(), A.ia) and np.array_equal(ja.cpu().numpy(), A.ja)
    assert np.array_equal(a.cpu().numpy(), A.a)


def test_file_reader_host_parsed_and_headers(tmp_path):
    """From a file: lines left to strtod (their bytes come back from the
    device copy), a comment block longer than the first header read, and a
    file that ends on its size line."""
    info = _same_file(tmp_path, mm_cases.general_text().encode(), "g.mtx")
    assert info["host_parsed"] > 0
    long_comments = "%%MatrixMarket matrix coordinate real general\n" + \
        "".join(f"% comment line {i:06d} " + "x" * 80 + "\n" for i in range(1500)) + \
        mm_cases.general_text(seed=9).split("\n", 1)[1]
    assert len(long_comments) > 2 * (1 << 16)
    _same_file(tmp_path, long_comments.encode(), "c.mtx")
    ia, ja, a, info = gb.read_mm_device(str(_write(tmp_path / "e.mtx",
                                                   b"%%MatrixMarket matrix coordinate real general\n3 3 0")))
    assert info["nnz"] == 0 and ia.cpu().tolist() == [0, 0, 0, 0]


def _write(p, data):
    p.write_bytes(data)
    return p


def test_edge_cases():
    # no entries
    ia, ja, a, info = gb.read_mm_device(data=b"%%MatrixMarket matrix coordinate real general\n3 3 0\n")
    assert info["nnz"] == 0 and ia.cpu().tolist() == [0, 0, 0, 0]
    # extra lines past the announced count are ignored
    _same("%%MatrixMarket matrix coordinate real general\n2 2 1\n1 2 3.5\n2 1 4.5\n")
    # a single entry with no newline at the end; a diagonal-only symmetric file
    _same("%%MatrixMarket matrix coordinate real symmetric\n1 1 1\n1 1 -2.5")
    # empty rows
    _same("%%MatrixMarket matrix coordinate real general\n5 5 2\n5 1 1\n1 5 2\n")


@pytest.mark.parametrize("text", [
    "%%MatrixMarket matrix coordinate real general\n",                       # no size line
    "%%MatrixMarket matrix coordinate real general\n2 2 2\n1 1 1.0\n",       # fewer entries
    "%%MatrixMarket matrix coordinate real general\n2 2 1\n3 1 1.0\n",       # row out of range
    "%%MatrixMarket matrix coordinate real general\n2 2 1\n1 0 1.0\n",       # column 0
    "%%MatrixMarket matrix coordinate real general\n2 2 1\n1 x 1.0\n",       # not a number
])
def test_rejects_bad_files(text):
    with pytest.raises(gb.GbError):
        gb.read_mm_device(data=text.encode())


def _adjacency_bytes(weights, seed=5, n=300, m=1500, unique=False):
    """A random graph's adjacency, lower triangle; repeated edges unless
    unique (the solver takes no duplicate entries)."""
    rng = np.random.default_rng(seed)
    ei, ej = rng.integers(0, n, m), rng.integers(0, n, m)
    keep = ei != ej
    ei, ej = ei[keep], ej[keep]
    lo, hi = np.maximum(ei, ej) + 1, np.minimum(ei, ej) + 1
    if unique:
        pairs = np.unique(np.stack([lo, hi], 1), axis=0)
        lo, hi = pairs[:, 0], pairs[:, 1]
    kind = "real" if weights else "pattern"
    lines = [f"%%MatrixMarket matrix coordinate {kind} symmetric", f"{n} {n} {lo.shape[0]}"]
    if weights:
        w = rng.uniform(0.1, 3.0, lo.shape[0])
        lines += [f"{lo[i]} {hi[i]} {float(w[i])!r}" for i in range(lo.shape[0])]
    else:
        lines += [f"{lo[i]} {hi[i]}" for i in range(lo.shape[0])]
    return ("\n".join(lines) + "\n").encode()


@pytest.mark.parametrize("weights", [False, True])
@pytest.mark.parametrize("weighted", [0, 1])
@pytest.mark.parametrize("exact", [0, 1])
def test_laplacian_from_adjacency(weights, weighted, exact):
    """gb_mm_parse_laplacian against oracle.laplacian_csr (pinned to the
    reference's builder): int-truncated degrees by default, exact ones with
    the flag -- the two differ once weights are not integers."""
    data = _adjacency_bytes(weights)
    ia, ja, a, info = gb.read_mm_device(data=data, laplacian=dict(weighted=weighted, exact_degrees=exact))
    n, oia, oja, oa = oracle.laplacian_csr(data, weighted, exact)
    assert info["symmetric"] == 1 and info["n"] == n
    assert np.array_equal(ia.cpu().numpy(), oia) and np.array_equal(ja.cpu().numpy(), oja)
    assert np.array_equal(a.cpu().numpy().view(np.int64), oa.view(np.int64))
    if weights and not weighted:
        _, _, _, trunc = oracle.laplacian_csr(data, 0, 0)
        _, _, _, full = oracle.laplacian_csr(data, 0, 1)
        assert not np.array_equal(trunc, full)  # the flag matters here


def test_laplacian_reference_fixture(golden):
    ia, ja, a, _ = gb.read_mm_device(f"{ROOT}/tests/golden/adj5.mtx", laplacian=dict(weighted=0))
    assert np.array_equal(ia.cpu().numpy(), golden["adj_ia"]) and np.array_equal(ja.cpu().numpy(), golden["adj_ja"])
    assert np.array_equal(a.cpu().numpy(), golden["adj_a"])


@pytest.mark.parametrize("weighted", [0, 1])
def test_laplacian_rhs_and_solve(weighted):
    """The driver's projected right-hand side is orthogonal to the vector it
    projects out and matches the oracle's to rounding; the singular
    unweighted Laplacian system then solves (cg_driver.c's flow, on the
    device).  The weighted driver projects out sqrt(diag) = e as well, while
    I - D^-1/2 W D^-1/2 has null vector D^1/2 e, so that system is left
    unsolved here, as the reference leaves it inconsistent."""
    data = _adjacency_bytes(False, n=400, m=4000, unique=True)
    ia, ja, a, _ = gb.read_mm_device(data=data, laplacian=dict(weighted=weighted))
    b = gb.laplacian_rhs(ia, ja, a, weighted)
    n = ia.numel() - 1
    A = gen.CSR(n, ia.cpu().numpy(), ja.cpu().numpy(), a.cpu().numpy())
    rows = np.repeat(np.arange(n), np.diff(A.ia))
    diag = A.a[A.ja == rows]
    ref = oracle.laplacian_rhs(n, diag, weighted)
    assert np.abs(b.cpu().numpy() - ref).max() <= 1e-14 * np.abs(ref).max() + 1e-15
    null = np.sqrt(diag) if weighted else np.ones(n)
    assert abs(float(np.dot(b.cpu().numpy(), null))) < 1e-10 * np.linalg.norm(null)
    if not weighted:
        sysm = gb.System.from_csr(A, "line_jacobi")
        x, r = sysm.solve(b, tol=1e-8, maxit=5000)
        assert r["flag"] == 0
        sysm.close()


def test_spmv_driver_report_matches_reference():
    """lap_mm_driver (mm_driver.c on the library) prints the reference
    program's report line for line: tests/golden/mm_driver_grid6.txt is the
    reference's own output on grid6.mtx with 3 trials.  The two time lines
    carry this run's times, and ||A x|| may differ from the reference's serial
    dot in the last bits."""
    import os
    import re
    import subprocess

    drv = os.path.join(ROOT, "lap_gb300", "lap_mm_driver")
    out = subprocess.run([drv, f"{ROOT}/tests/golden/grid6.mtx", "3"], capture_output=True, text=True,
                         check=True).stdout.split("\n")
    ref = open(f"{ROOT}/tests/golden/mm_driver_grid6.txt").read().split("\n")
    assert len(out) == len(ref)
    for got, want in zip(out, ref):
        if "Time (" in want:
            pat = re.escape(want[: want.index(":") + 2]) + r"\d+\.\d{16}  $"
            assert re.match(pat, got), (got, want)
        elif "Norm of A*x" in want:
            head = want[: want.index(":") + 2]
            assert got.startswith(head) and re.match(re.escape(head) + r"-?\d\.\d{16}e[+-]\d\d  $", got)
            g, w = float(got[len(head):]), float(want[len(head):])
            assert abs(g - w) <= 1e-14 * abs(w)
        else:
            assert got == want
