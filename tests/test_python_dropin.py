"""grav_sim's own Python package driving this library, unchanged.

GravitySimulatorAPI(c_lib_path=...) loads the library and sets the restypes
of every symbol grav_sim/utils.py:38-58 names; the Simulator then calls
launch_simulation_python with its own argument marshalling
(grav_sim/simulator.py:22-143).  The only change a maintainer makes is to
register the GPU method codes (grav_sim/parameters.py:21-35), which the test
does as the integration guide shows.  The package is imported from the
reference's directory where it is present (it is not installed; matplotlib,
which only its plotting module needs, is stubbed).  Without a GPU the run
stops at the device check with the library's traceback; with one it must
equal the oracle bit for bit.
"""
import ctypes
import sys
import types

import numpy as np
import pytest

from oracle.reference import REF_DIR as REF
pytestmark = pytest.mark.skipif(not (REF / "grav_sim" / "api.py").exists(),
                                reason="grav_sim's Python package not present")

GPU_CODES = {"gpu_pairwise": 101, "gpu_massless": 102, "gpu_barnes_hut": 103,
             "gpu_barnes_hut_learned": 104, "gpu_barnes_hut_quadrupole": 105,
             "gpu_barnes_hut_group": 106, "gpu_barnes_hut_group_mono": 107,
             "gpu_pairwise_fp64": 111, "gpu_barnes_hut_compat": 113}


@pytest.fixture(scope="module")
def grav_sim():
    if "matplotlib" not in sys.modules:
        mpl = types.ModuleType("matplotlib")
        plt = types.ModuleType("matplotlib.pyplot")
        def attr(name):
            if name.startswith("__"):
                raise AttributeError(name)
            return lambda *a, **k: None
        plt.__getattr__ = attr
        mpl.pyplot = plt
        sys.modules["matplotlib"] = mpl
        sys.modules["matplotlib.pyplot"] = plt
    sys.path.insert(0, str(REF))
    import grav_sim
    from grav_sim import parameters
    P = parameters.AccelerationParam
    for name, code in GPU_CODES.items():
        if name not in P.AVAILABLE_ACCELERATION_METHODS:
            P.AVAILABLE_ACCELERATION_METHODS.append(name)
        P.ACCELERATION_METHODS_TO_ENCODING[name] = code
        P.ACCELERATION_ENCODING_TO_METHODS[code] = name
    return grav_sim


def test_api_loads_this_library(grav_sim, g):
    api = grav_sim.GravitySimulatorAPI(c_lib_path=str(g.library_path()))
    assert api.c_lib._name == str(g.library_path())
    assert "gpu_pairwise" in api.AVAILABLE_ACCELERATION_METHODS


def test_simulator_launch_through_grav_sim(grav_sim, g, orc, wl, capfd):
    from grav_sim import parameters
    from grav_sim.system import System
    api = grav_sim.GravitySimulatorAPI(c_lib_path=str(g.library_path()))
    x, v, m = wl.plummer(200, 8)
    system = System(api.c_lib)
    system.add(x, v, m)
    system.G = 1.0
    ap = parameters.AccelerationParam()
    ap.method = "gpu_pairwise_fp64"
    ap.softening_length = 0.01
    ip = parameters.IntegratorParam()
    ip.integrator = "leapfrog"
    ip.dt = 1e-3
    op = parameters.OutputParam()
    op.method = "disabled"
    st = parameters.Settings()
    st.verbose = "ignore_all"
    st.enable_progress_bar = False
    try:
        import torch
        have_gpu = torch.cuda.is_available()
    except ImportError:
        have_gpu = False
    if not have_gpu:
        capfd.readouterr()
        with pytest.raises(RuntimeError):
            api.launch_simulation(system, ap, ip, op, st, 0.01)
        assert "CUDA" in capfd.readouterr().err
        return
    api.launch_simulation(system, ap, ip, op, st, 0.01)
    xr, vr = orc.fixed_step_run(4, 1, x, v, m, 1.0, 0.01, 1e-3, 0.01)
    assert np.array_equal(system.x, xr) and np.array_equal(system.v, vr)
