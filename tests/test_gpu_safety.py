"""Failure paths that must not hang or fault the GPU.

Every wait in the library's kernels is bounded: after its limit the kernel
sets a bit in a device status word and returns, and the host turns the word
into an ErrorStatus.  The test runs a wait on an mbarrier that nothing
completes, with a short limit, and checks that the status comes back and the
context still computes."""
import ctypes
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ST_WAIT_TIMEOUT = 1


def test_expired_wait_reports_status_and_context_survives(lib, g, orc, wl):
    f = lib.gsgpu_wait_timeout_selftest
    f.argtypes = [ctypes.c_double, ctypes.POINTER(ctypes.c_uint)]
    status = ctypes.c_uint(0)
    t0 = time.perf_counter()
    assert f(50.0, ctypes.byref(status)) == 0
    elapsed = time.perf_counter() - t0
    assert status.value == ST_WAIT_TIMEOUT
    assert elapsed < 5.0
    # the context is still usable: a direct sum matches the oracle
    x, v, m = wl.plummer(300, 3)
    a = g.acceleration(lib, x, m, 1.0, g.METHOD_GPU_PAIRWISE_FP64, 1.0, 0.01, -1)
    assert np.array_equal(a, orc.pairwise(x, m, 1.0, 0.01))


def test_selftest_rejects_bad_limits(lib):
    f = lib.gsgpu_wait_timeout_selftest
    f.argtypes = [ctypes.c_double, ctypes.POINTER(ctypes.c_uint)]
    status = ctypes.c_uint(0)
    assert f(0.0, ctypes.byref(status)) != 0
    assert f(5000.0, ctypes.byref(status)) != 0


@pytest.mark.parametrize("method,k", [(101, 1), (101, 3), (106, 1), (106, 5), (102, 2)])
def test_allocation_failure_is_reported_and_recovered(lib, g, orc, wl, method, k):
    """Host-side fault injection: the k-th device allocation of a fresh
    engine fails as an out-of-memory cudaMalloc would.  The call returns
    GRAV_MEMORY_ERROR with a traceback, nothing crashes, and the next call
    (no injection) computes the right forces."""
    lib.gsgpu_test_fail_allocation.argtypes = [ctypes.c_int]
    lib.gsgpu_test_fail_allocation.restype = None
    n = 700 + 10 * k + method % 7      # a size no earlier test built an engine for
    x, v, m = wl.plummer(n, 40 + k)
    lib.gsgpu_test_fail_allocation(k)
    try:
        with pytest.raises(g.GravError) as e:
            g.acceleration(lib, x, m, 1.0, method, 0.5, 0.01, -1)
        assert e.value.code == g.GRAV_MEMORY_ERROR
        assert "cudaMalloc" in e.value.traceback
    finally:
        lib.gsgpu_test_fail_allocation(0)
    a = g.acceleration(lib, x, m, 1.0, method, 0.5, 0.01, -1)
    ref = orc.pairwise(x, m, 1.0, 0.01)
    assert np.isfinite(a).all()
    err = np.linalg.norm(a - ref, axis=1) / np.linalg.norm(ref, axis=1)
    assert np.median(err) < (1e-3 if method == 106 else 1e-6)


def test_allocation_failure_in_launch_simulation(lib, g, orc, wl):
    lib.gsgpu_test_fail_allocation.argtypes = [ctypes.c_int]
    x, v, m = wl.plummer(300, 77)
    lib.gsgpu_test_fail_allocation(2)
    try:
        with pytest.raises(RuntimeError):
            g.launch_simulation(lib, x.copy(), v.copy(), m, 1.0, integrator=4, dt=1e-3, tf=5e-3,
                                method=g.METHOD_GPU_PAIRWISE_FP64, softening_length=0.01)
    finally:
        lib.gsgpu_test_fail_allocation(0)
    _, xo, vo, _ = g.launch_simulation(lib, x.copy(), v.copy(), m, 1.0, integrator=4, dt=1e-3,
                                       tf=5e-3, method=g.METHOD_GPU_PAIRWISE_FP64,
                                       softening_length=0.01)
    xr, vr = orc.fixed_step_run(4, 1, x, v, m, 1.0, 0.01, 1e-3, 5e-3)
    assert np.array_equal(xo, xr) and np.array_equal(vo, vr)
