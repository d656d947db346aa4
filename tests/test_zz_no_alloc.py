"""gb_dot_noalloc (allocation-free dot product) through the C ABI, against
the library's cuda_dot on the same device vectors.

The file name sorts last so that pytest collects it after the other tests: the
entry point must also work in a process whose earlier tests have already
initialised the library and its allocating paths.  Reductions are compared at
1e-14 relative, as the other dot tests are.
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a GPU", allow_module_level=True)

import lap_gb300 as gb  # noqa: E402

GB_OK, GB_BAD_INPUT = 0, 5
MAX_N = 8192 * 4096  # GB_DOT_NOALLOC_MAX_N in include/gblap.h


def _noalloc(n, v, w):
    out = C.c_double(np.nan)
    rc = gb.lib().gb_dot_noalloc(n, gb.ptr(v), gb.ptr(w), C.byref(out), None)
    return rc, out.value


@pytest.mark.parametrize("n", [1, 1000, 4096, 4097, 1_000_003, 8_000_000])
def test_noalloc_dot_matches_cuda_dot_twice(n):
    rng = np.random.default_rng(20_000 + n)
    v = torch.from_numpy(rng.standard_normal(n)).cuda()
    w = torch.from_numpy(rng.standard_normal(n)).cuda()
    torch.cuda.synchronize()
    ref = gb.lib().cuda_dot(n, gb.ptr(v), gb.ptr(w))
    scale = float(torch.dot(v.abs(), w.abs()).item())
    for _ in range(2):  # two calls in a row: the scratch is reused
        rc, got = _noalloc(n, v, w)
        assert rc == GB_OK
        assert abs(got - ref) <= 1e-14 * scale + 1e-300


def test_noalloc_dot_empty_and_rejections(capfd):
    v = torch.ones(16, dtype=torch.float64, device="cuda")
    assert _noalloc(0, v, v) == (GB_OK, 0.0)
    assert _noalloc(-1, v, v)[0] == GB_BAD_INPUT
    # over the static limit: rejected on the host before any device access
    rc, _ = _noalloc(MAX_N + 1, v, v)
    assert rc == GB_BAD_INPUT
    assert "exceeds the static scratch limit" in capfd.readouterr().err
    # the scratch is still usable afterwards
    assert _noalloc(16, v, v) == (GB_OK, 16.0)


_NO_GROWTH_CHILD = r"""
import ctypes as C, sys
import torch
sys.path.insert(0, sys.argv[1])
import lap_gb300 as gb
L = gb.lib()
n = 3_000_001
v = torch.ones(n, dtype=torch.float64, device="cuda")
out = C.c_double()
torch.cuda.synchronize()
assert L.gb_dot_noalloc(n, gb.ptr(v), gb.ptr(v), C.byref(out), None) == 0  # first call: set-up
free0, _ = torch.cuda.mem_get_info()
for _ in range(50):
    assert L.gb_dot_noalloc(n, gb.ptr(v), gb.ptr(v), C.byref(out), None) == 0
    assert out.value == float(n)
torch.cuda.synchronize()
free1, _ = torch.cuda.mem_get_info()
print("free-before", free0, "free-after", free1)
assert free1 == free0, (free0, free1)
"""


def test_noalloc_dot_takes_no_device_memory():
    """The property the entry point exists for, in a fresh process: after the
    first call (which only looks the scratch array up), fifty more calls
    leave the device's free memory exactly where it was."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", _NO_GROWTH_CHILD, root], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
