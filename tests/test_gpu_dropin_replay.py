"""grav_sim's own Simulator call, replayed through this library on the GPU.

tests/golden/make_dropin_calls.py ran grav_sim's unchanged Python package
(GravitySimulatorAPI with this library and the GPU method codes registered,
Simulator.launch_simulation) and recorded the one call it makes,
launch_simulation_python (src/python_interface.c:94-192), argument by
argument with grav_sim's ctypes types; the expected results are the same
call into the reference C library with the CPU method.  Here the recorded
call goes to this library as grav_sim would make it, and the state that
comes back through grav_sim's output pointers must be the reference's: bit
for bit for the FP64 pairwise sum (111) and the massless WHFast (102), to
the group walk (106) against the exact pairwise force through the velocity
change over the run: its median relative error within the recorded bound
(1e-3, a few times the walk's median force error), its 99th percentile
within 10 times that, positions to 1e-6 of their extent.
"""
import numpy as np
import pytest

from conftest import cases, golden
from dropin_replay import replay

pytestmark = pytest.mark.gpu

CASES = cases(golden("dropin_calls"))


@pytest.mark.parametrize("name", sorted(CASES))
def test_grav_sim_call_replayed(lib, name):
    c = CASES[name]
    arrays = {k: c[k] for k in ("ids", "x", "v", "m")}
    rc, ids, x, v, m = replay(lib, c["spec.json"], arrays)
    assert rc == 0
    # (WHFast returns the particles sorted by distance, as the reference does)
    assert np.array_equal(ids, c["ids_expected"]) and np.array_equal(m, c["m_expected"])
    tol = float(c["tolerance"])
    if tol == 0.0:
        assert np.array_equal(x, c["x_expected"]) and np.array_equal(v, c["v_expected"])
    else:
        dv_ref = c["v_expected"] - c["v"]
        err = np.linalg.norm((v - c["v"]) - dv_ref, axis=1) / np.linalg.norm(dv_ref, axis=1)
        print(f"{name}: velocity change median error {np.median(err):.3g}, "
              f"p99 {np.percentile(err, 99):.3g}")
        assert np.median(err) <= tol and np.percentile(err, 99) <= 10 * tol
        assert np.abs(x - c["x_expected"]).max() <= 1e-6 * np.abs(c["x_expected"]).max()
