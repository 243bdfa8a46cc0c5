"""Direct-sum accelerations on the GPU against the oracle.

GRAV_GPU_PAIRWISE_FP64 (111) must equal grav_sim's acceleration_pairwise bit
for bit.  GRAV_GPU_PAIRWISE (101, compensated FP32) is held to these
tolerances against the FP64 reference:
  * every particle: |a_i - a_ref,i| <= 3e-5 * A_i, where
    A_i = G sum_j m_j |r_ij| / (r_ij^2 + eps^2)^1.5 is the sum of the pair
    terms' magnitudes -- the scale that the rounding of FP32 pair terms is
    proportional to (a particle whose force nearly cancels keeps this
    absolute accuracy, not the same relative one).  The floor of this bound
    is set by rounding positions to FP32 for the closest pairs, about
    ulp(|x|) / |r_ij|;
  * per-particle relative error |a_i - a_ref,i| / |a_ref,i|: median <= 1e-6
    and 99th percentile <= 1e-5, over populations of at least 4096 particles.
"""
import ctypes

import numpy as np
import pytest

from conftest import cases, golden

pytestmark = pytest.mark.gpu

TOL_ABS_SUM = 3e-5
TOL_MEDIAN = 1e-6
TOL_P99 = 1e-5


def check_fp32(a, ref, abs_sum):
    a = np.asarray(a)
    ref = np.asarray(ref)
    diff = np.linalg.norm(a - ref, axis=1)
    assert np.all(diff <= TOL_ABS_SUM * abs_sum + 1e-300), float(np.max(diff / (abs_sum + 1e-300)))
    mag = np.linalg.norm(ref, axis=1)
    nz = mag > 0
    if nz.sum() < 4096:
        # the relative-error statistics need a population; tiny cases are
        # held to the per-particle bound above
        return 0.0, 0.0
    rel = diff[nz] / mag[nz]
    med = float(np.median(rel))
    p99 = float(np.quantile(rel, 0.99))
    assert med <= TOL_MEDIAN, med
    assert p99 <= TOL_P99, p99
    return med, p99


def test_fp64_reference_order_bitexact_golden(lib, g):
    for name, c in cases(golden("pairwise")).items():
        a = g.acceleration(lib, c["x"], c["m"], float(c["G"]), g.METHOD_GPU_PAIRWISE_FP64,
                           softening_length=float(c["eps"]))
        assert np.array_equal(a, c["a"]), name


def test_fp32_golden_cases(lib, g, orc):
    for name, c in cases(golden("pairwise")).items():
        G, eps = float(c["G"]), float(c["eps"])
        a = g.acceleration(lib, c["x"], c["m"], G, g.METHOD_GPU_PAIRWISE, softening_length=eps)
        check_fp32(a, c["a"], orc.abs_sum_rows(c["x"], c["m"], G, eps))


@pytest.mark.parametrize("n", [1000, 1023, 1025, 3000, 20000])
def test_fp32_sizes(lib, g, orc, wl, n):
    x, v, m = wl.plummer(n, 300 + n)
    a = g.acceleration(lib, x, m, 1.0, g.METHOD_GPU_PAIRWISE, softening_length=0.01)
    check_fp32(a, orc.pairwise(x, m, 1.0, 0.01), orc.abs_sum_rows(x, m, 1.0, 0.01))


def test_fp32_unsoftened_and_offset_frame(lib, g, orc, wl):
    x, v, m = wl.plummer(5000, 77)
    x = x + np.array([100.0, -50.0, 25.0])    # far from the origin
    a = g.acceleration(lib, x, m, 2.5, g.METHOD_GPU_PAIRWISE, softening_length=0.0)
    check_fp32(a, orc.pairwise(x, m, 2.5, 0.0), orc.abs_sum_rows(x, m, 2.5, 0.0))


def test_fp32_repeat_calls_and_resize(lib, g, orc, wl):
    for n in (4096, 100, 4096, 7):
        x, v, m = wl.plummer(n, n)
        a1 = g.acceleration(lib, x, m, 1.0, g.METHOD_GPU_PAIRWISE, softening_length=0.01)
        a2 = g.acceleration(lib, x, m, 1.0, g.METHOD_GPU_PAIRWISE, softening_length=0.01)
        assert np.array_equal(a1, a2)     # deterministic
        check_fp32(a1, orc.pairwise(x, m, 1.0, 0.01), orc.abs_sum_rows(x, m, 1.0, 0.01))


def test_fp32_full_size_plummer_262144(lib, g, orc, wl):
    """The mixed-precision workload at full size: median relative error
    against an FP64 direct sum (4096 sampled particles) <= 1e-6."""
    x, v, m = wl.plummer(262144, 2)
    a = g.acceleration(lib, x, m, 1.0, g.METHOD_GPU_PAIRWISE, softening_length=0.01)
    rows = np.random.default_rng(0).choice(262144, 4096, replace=False).astype(np.int32)
    ref = orc.direct_rows(x, m, 1.0, 0.01, rows)
    med, p99 = check_fp32(a[rows], ref, orc.abs_sum_rows(x, m, 1.0, 0.01, rows))
    print(f"N=262144 median {med:.3g} p99 {p99:.3g}")


def test_cpu_method_code_rejected(lib, g, wl):
    x, v, m = wl.plummer(16, 1)
    with pytest.raises(g.GravError) as e:
        g.acceleration(lib, x, m, 1.0, 1)
    assert e.value.code == g.GRAV_VALUE_ERROR


def test_fp64_reference_order_bitexact_large(lib, g, orc, wl):
    """Above 32,768 particles the FP64 reference-order sum runs ten particles
    per warp; still the reference's operations in the reference's order."""
    x, v, m = wl.plummer(33000, 17)
    a = g.acceleration(lib, x, m, 1.0, g.METHOD_GPU_PAIRWISE_FP64, 1.0, 0.01, -1)
    assert np.array_equal(a, orc.pairwise(x, m, 1.0, 0.01))


def _softened_energy_fp64(x, v, m, G, eps):
    ke = 0.5 * np.sum(m * np.sum(v * v, axis=1))
    pe = 0.0
    for i0 in range(0, len(m), 512):
        d = x[i0:i0 + 512, None, :] - x[None, :, :]
        r = np.sqrt(np.sum(d * d, axis=2) + eps * eps)
        w = m[i0:i0 + 512, None] * m[None, :] / r
        idx = np.arange(i0, min(i0 + 512, len(m)))
        w[idx - i0, idx] = 0.0
        pe += w.sum()
    return ke - 0.5 * G * pe


@pytest.mark.parametrize("n", [0, 1, 2, 4097])
def test_softened_energy_against_fp64(lib, n):
    """gsgpu_softened_energy (compensated FP32 pair terms on double-float
    coordinates) against the FP64 sum, within 1e-6 relative; at n = 4097 the
    system sits 100 units off the origin."""
    lib.gsgpu_softened_energy.restype = ctypes.c_int
    dp = ctypes.POINTER(ctypes.c_double)
    lib.gsgpu_softened_energy.argtypes = [dp, dp, dp, ctypes.c_int, ctypes.c_double,
                                          ctypes.c_double, dp]
    rng = np.random.default_rng(n)
    x = rng.normal(size=(n, 3)) + 100.0
    v = rng.normal(size=(n, 3))
    m = rng.uniform(0.5, 1.5, n) / max(n, 1)
    e = ctypes.c_double()
    assert lib.gsgpu_softened_energy(x.ctypes.data_as(dp), v.ctypes.data_as(dp),
                                     m.ctypes.data_as(dp), n, 1.0, 0.01, ctypes.byref(e)) == 0
    want = _softened_energy_fp64(x, v, m, 1.0, 0.01) if n else 0.0
    assert abs(e.value - want) <= 1e-6 * max(abs(want), 1e-300), (e.value, want)
