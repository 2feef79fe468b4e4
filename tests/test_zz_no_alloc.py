"""qsf_norm_noalloc: the norm for callers that cannot allocate device memory.

Such a caller -- one whose device memory all comes from its own pool, or a runtime
that may only pass buffers it already owns across its foreign-function boundary --
holds psi and a one-double result buffer on the device itself.  The entry point keeps
its per-block partial sums in a fixed array inside the library instead of allocating.
Here it must agree with the handle-based qsf_average (same tolerance as the other
single-primitive checks, 1e-12 relative) on two calls in a row, and it must refuse a
size larger than its fixed array can reduce.  This file is collected last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12
MAX_POINTS = 8192 * 16384


def _entry():
    from qsf_gb300._lib import lib
    f = lib().qsf_norm_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


@pytest.mark.parametrize("dim,n,seed", [(1, 4096, 3), (2, 384, 1), (3, 48, 2)])
def test_norm_noalloc_matches_average_on_two_calls(dim, n, seed):
    torch = pytest.importorskip("torch")
    import qsf_gb300 as Q
    f = _entry()
    dx = 0.3
    g = Q.Grid(dim, n, dx)
    rng = np.random.default_rng(seed)
    shape = (n,) * dim
    g.upload(rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
    expected = g.average(Q.REP_X, Q.OP_IDENTITY)
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    for _ in range(2):
        out.fill_(-1.0)
        torch.cuda.synchronize()
        rc = f(g.device_ptr(), g.m, dx ** dim, out.data_ptr(), None)
        assert rc == 0, Q.lib().qsf_last_error()
        torch.cuda.synchronize()
        assert float(out[0].item()) == pytest.approx(expected, rel=TOL)
        assert float(out[1].item()) == -1.0  # nothing written past the one output double


def test_norm_noalloc_rejects_sizes_beyond_its_scratch():
    import qsf_gb300 as Q
    f = _entry()
    # rejected on the host before anything is launched, so placeholder addresses suffice
    rc = f(ctypes.c_void_p(256), MAX_POINTS + 1, 1.0, ctypes.c_void_p(256), None)
    assert rc == 1
    assert b"exceeds the maximum" in Q.lib().qsf_last_error()
