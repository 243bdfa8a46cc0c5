"""GRAV_GPU_MASSLESS against grav_sim's acceleration_massless: FP64 in the
reference's operation order, bit-exact (tolerance 0), including the
reference's loop-index mass read when massive and massless particles are
interleaved."""
import numpy as np
import pytest

from conftest import cases, golden

pytestmark = pytest.mark.gpu


def test_massless_bitexact_golden(lib, g):
    for name, c in cases(golden("massless")).items():
        a = g.acceleration(lib, c["x"], c["m"], 1.0, g.METHOD_GPU_MASSLESS,
                           softening_length=0.01)
        assert np.array_equal(a, c["a"]), name


@pytest.mark.parametrize("n,frac", [(1, 0.0), (2, 0.5), (5000, 0.9), (20000, 0.999)])
def test_massless_bitexact_fresh(lib, g, orc, wl, n, frac):
    x, v, m = wl.plummer(n, 40 + n)
    rng = np.random.default_rng(n)
    m = m.copy()
    m[rng.random(n) < frac] = 0.0
    a = g.acceleration(lib, x, m, 1.3, g.METHOD_GPU_MASSLESS, softening_length=0.02)
    assert np.array_equal(a, orc.massless(x, m, 1.3, 0.02))


@pytest.mark.parametrize("integ", [1, 2, 3, 4])
def test_massless_integrators_bitexact(lib, g, orc, wl, integ):
    systems = wl.planetary_ensemble(1, 7, max_test=300)
    x, v, m = systems[0]
    dt, tf = 1.0, 50.0
    _, xo, vo, _ = g.launch_simulation(lib, x.copy(), v.copy(), m.copy(), wl.G_AU_MSUN_DAY,
                                       integrator=integ, dt=dt, tf=tf,
                                       method=g.METHOD_GPU_MASSLESS)
    xr, vr = orc.fixed_step_run(integ, 2, x, v, m, wl.G_AU_MSUN_DAY, 0.0, dt, tf)
    assert np.array_equal(xo, xr) and np.array_equal(vo, vr)
