"""The allocation-free direct-sum entry point, through the C ABI.

gsgpu_pairwise_acceleration_noalloc serves callers that cannot allocate
device memory while they run (fixed recorded/replayed GPU work, caller-owned
memory pools, real-time loops): it takes caller-owned device arrays and keeps
its scratch in a fixed device array of the library.  This file runs last so
that a failure here cannot hide the other tests, and it passes both alone in
a fresh process and after the rest of the suite.

Checks, for a Plummer sphere at the origin and the same sphere moved 100
units away (the entry point centres positions on their bounding box on the
device, as acceleration() does on the host), two calls in a row each:
  * against the FP64 direct sum of the oracle, with the tolerance of the
    direct-sum tests -- every particle |a - a_ref| <= 3e-5 * A_i (A_i the
    sum of pair-term magnitudes), median relative error <= 1e-6, 99th
    percentile <= 1e-5;
  * against the existing entry point (acceleration() with GRAV_GPU_PAIRWISE)
    with the same per-particle bound, doubled because both sides carry FP32
    rounding;
  * the two calls agree exactly.
A particle count beyond the fixed capacity, or below one, is rejected with
GRAV_VALUE_ERROR.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_ABS_SUM = 3e-5
TOL_MEDIAN = 1e-6
TOL_P99 = 1e-5


def _noalloc(lib):
    f = lib.gsgpu_pairwise_acceleration_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_double,
                  ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]
    return f


@pytest.mark.parametrize("offset", [0.0, 100.0])
def test_noalloc_matches_oracle_and_existing_entry_point_twice(lib, g, orc, wl, offset):
    torch = pytest.importorskip("torch")
    f = _noalloc(lib)
    n, G, eps = 20000, 1.0, 0.01
    x, v, m = wl.plummer(n, 4242)
    x = np.ascontiguousarray(x + np.array([offset, -0.5 * offset, 0.25 * offset]))
    exact = orc.pairwise(x, m, G, eps)
    A = orc.abs_sum_rows(x, m, G, eps)
    engine = g.acceleration(lib, x, m, G, g.METHOD_GPU_PAIRWISE, softening_length=eps)
    dx = torch.from_numpy(x).cuda()
    dm = torch.from_numpy(np.ascontiguousarray(m)).cuda()
    da = torch.empty((n, 3), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    results = []
    for call in range(2):
        da.fill_(float("nan"))
        rc = f(dx.data_ptr(), dm.data_ptr(), n, G, eps, da.data_ptr(),
               ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, rc
        torch.cuda.synchronize()
        a = da.cpu().numpy()
        assert np.all(np.isfinite(a)), call
        diff = np.linalg.norm(a - exact, axis=1)
        assert np.all(diff <= TOL_ABS_SUM * A), (call, float(np.max(diff / A)))
        rel = diff / np.linalg.norm(exact, axis=1)
        assert np.median(rel) <= TOL_MEDIAN, (call, float(np.median(rel)))
        assert np.quantile(rel, 0.99) <= TOL_P99, (call, float(np.quantile(rel, 0.99)))
        d_engine = np.linalg.norm(a - engine, axis=1)
        assert np.all(d_engine <= 2 * TOL_ABS_SUM * A), call
        results.append(a)
    assert np.array_equal(results[0], results[1])


def test_noalloc_rejects_counts_beyond_capacity(lib, g):
    torch = pytest.importorskip("torch")
    f = _noalloc(lib)
    d = torch.zeros(3, dtype=torch.float64, device="cuda")
    assert f(d.data_ptr(), d.data_ptr(), 32769, 1.0, 0.01, d.data_ptr(), None) == g.GRAV_VALUE_ERROR
    assert f(d.data_ptr(), d.data_ptr(), 0, 1.0, 0.01, d.data_ptr(), None) == g.GRAV_VALUE_ERROR
