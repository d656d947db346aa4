"""gb_pcg_autotune_precision: the precision mode chosen by timing each
mode's converged solve, and precision = -1 solving in that mode."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a GPU", allow_module_level=True)

import lap_gb300 as gb  # noqa: E402
from lap_gb300 import gen  # noqa: E402


def _system(prec, n=24):
    A, b = gen.grid3d_lognormal(n, seed=1002)
    return gb.System.from_csr(A, prec), torch.from_numpy(b).cuda()


def test_choice_is_the_fastest_converged_mode_and_minus_one_uses_it():
    s, b = _system("ichol")
    out = s.autotune_precision(b, tol=1e-8, maxit=2000)
    ms = out["ms"]
    assert out["best"] in (0, 1, 2)
    assert all(v > 0.0 for v in ms)  # IC(0) runs every mode
    assert ms[out["best"]] == min(ms)
    x_auto, r_auto = s.solve(b, tol=1e-8, maxit=2000, precision=-1)
    x_best, r_best = s.solve(b, tol=1e-8, maxit=2000, precision=out["best"])
    assert r_auto["iters"] == r_best["iters"] and r_auto["flag"] == 0
    assert np.array_equal(x_auto.cpu().numpy(), x_best.cpu().numpy())


def test_unsupported_mode_is_skipped():
    s, b = _system("line_jacobi", n=16)
    out = s.autotune_precision(b, tol=1e-8, maxit=2000)
    assert out["ms"][2] == -1.0  # the split recurrence needs a triangular-solve preconditioner
    assert out["best"] in (0, 1)


def test_before_autotuning_minus_one_is_fp64():
    s, b = _system("ichol", n=12)
    x_auto, r_auto = s.solve(b, tol=1e-8, maxit=2000, precision=-1)
    x_64, r_64 = s.solve(b, tol=1e-8, maxit=2000, precision=0)
    assert r_auto["iters"] == r_64["iters"]
    assert np.array_equal(x_auto.cpu().numpy(), x_64.cpu().numpy())
