"""Tiny systems and empty runs through the GPU path.

One and two particles through every integrator of launch_simulation, for no
time (tf = 0) and for three steps, equal bit for bit to grav_sim's own runs
(tests/golden/edges.npz; FP64 reference-order forces 111, massless 102 for
WHFast).  Every GPU acceleration method on one, two and three particles.
"""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

D = golden("edges")
CASES = sorted({k.split("/")[0] for k in D if "/" in k})


@pytest.mark.parametrize("key", CASES)
def test_tiny_runs_match_reference(lib, g, key):
    n = int(key.split("_")[0][1:])
    integ = int(key.split("_")[1][3:])
    tf = float(key.split("_")[2][2:])
    x, v, m = D["x"][:n].copy(), D["v"][:n].copy(), D["m"][:n].copy()
    kw = dict(tolerance=1e-8) if 5 <= integ <= 9 else {}
    method = g.METHOD_GPU_MASSLESS if integ == 10 else g.METHOD_GPU_PAIRWISE_FP64
    ids, xo, vo, _ = g.launch_simulation(lib, x, v, m, 1.0, integrator=integ, dt=1e-3, tf=tf,
                                         method=method, softening_length=0.01, **kw)
    assert np.array_equal(ids, D[f"{key}/ids"])
    assert np.array_equal(xo, D[f"{key}/x"]) and np.array_equal(vo, D[f"{key}/v"])


def test_ias15_single_particle_stops_with_error(lib, g):
    """The reference's IAS15 loop never ends for one particle (0/0 error
    estimate); this library stops with an error."""
    x, v, m = D["x"][:1].copy(), D["v"][:1].copy(), D["m"][:1].copy()
    with pytest.raises(RuntimeError):
        g.launch_simulation(lib, x, v, m, 1.0, integrator=9, dt=1e-3, tf=3e-3,
                            method=g.METHOD_GPU_PAIRWISE_FP64, softening_length=0.01,
                            tolerance=1e-8)


@pytest.mark.parametrize("method", [101, 102, 103, 105, 106, 107, 111, 113])
@pytest.mark.parametrize("n", [1, 2, 3])
def test_every_method_on_tiny_systems(lib, g, orc, method, n):
    x, m = D["x"][:n].copy(), D["m"][:n].copy()
    a = g.acceleration(lib, x, m, 1.0, method, 0.5, 0.01, -1)
    assert a.shape == (n, 3) and np.isfinite(a).all()
    if n == 1:
        assert (a == 0).all()
        return
    if method in (101, 102, 111):
        ref = orc.pairwise(x, m, 1.0, 0.01)
    elif method in (103, 113):
        ref = orc.barnes_hut(x, m, 1.0, 0.01, 0.5, 1, method == 113)
    else:
        return   # quadrupole / group walks: finite, checked above
    assert np.allclose(a, ref, rtol=1e-5, atol=1e-6 * np.abs(ref).max())
