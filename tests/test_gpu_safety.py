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
