"""Record the call grav_sim's own Python Simulator makes into the library, for
replay on a GPU (tests/test_gpu_dropin_replay.py).

grav_sim's package cannot travel to a machine without the reference sources,
and a machine with them here has no GPU.  So this script runs grav_sim's
unchanged ``GravitySimulatorAPI`` / ``Simulator.launch_simulation``
(grav_sim/api.py, grav_sim/simulator.py:22-143) with this library loaded and
the GPU method codes registered in grav_sim's method tables
(grav_sim/parameters.py:21-35), and intercepts the
one call it makes, ``launch_simulation_python`` (src/python_interface.c
:94-192): every argument is recorded with the ctypes type grav_sim gave it,
and the input arrays with their values.  The expected results come from the
same call into the reference C library itself (oracle/_ref), with the CPU
method the GPU code reproduces.  Run where the reference is present:

    python tests/golden/make_dropin_calls.py

Output: tests/golden/dropin_calls.npz
"""
from __future__ import annotations

import ctypes
import importlib.util
import json
import sys
import types
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
OUT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

from dropin_replay import replay  # noqa: E402
from oracle import reference as ref  # noqa: E402

spec = importlib.util.spec_from_file_location("wl", ROOT / "gravity-simulator_gb300" / "workloads.py")
wl = importlib.util.module_from_spec(spec)
spec.loader.exec_module(wl)

GPU_CODES = {"gpu_pairwise": 101, "gpu_massless": 102, "gpu_barnes_hut": 103,
             "gpu_barnes_hut_learned": 104, "gpu_barnes_hut_quadrupole": 105,
             "gpu_barnes_hut_group": 106, "gpu_barnes_hut_group_mono": 107,
             "gpu_pairwise_fp64": 111, "gpu_barnes_hut_compat": 113}


def import_grav_sim():
    if "matplotlib" not in sys.modules:   # only grav_sim's plotting module needs it
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
    sys.path.insert(0, str(ref.REF_DIR))
    import grav_sim
    from grav_sim import parameters
    P = parameters.AccelerationParam
    for name, code in GPU_CODES.items():
        if name not in P.AVAILABLE_ACCELERATION_METHODS:
            P.AVAILABLE_ACCELERATION_METHODS.append(name)
        P.ACCELERATION_METHODS_TO_ENCODING[name] = code
        P.ACCELERATION_ENCODING_TO_METHODS[code] = name
    return grav_sim


class Recorder:
    """Stands in for the loaded library in grav_sim's Simulator: records the
    arguments of launch_simulation_python and reports a failure, so that
    nothing runs here."""

    def __init__(self):
        self.args = None

    def launch_simulation_python(self, *args):
        self.args = args
        return 1


def describe(args):
    """(spec, arrays): per argument its kind and ctypes type name (and value
    for scalars); the arrays behind the four input pointers."""
    n = args[0]._obj.value
    shapes = {1: (n,), 2: (n, 3), 3: (n, 3), 4: (n,)}
    spec, arrays = [], {}
    for k, a in enumerate(args):
        tname = type(a).__name__
        if tname == "CArgObject":
            obj = a._obj
            if isinstance(obj, ctypes._Pointer):
                spec.append({"kind": "out_pointer", "type": type(obj._type_()).__name__})
            else:
                spec.append({"kind": "byref", "type": type(obj).__name__, "value": obj.value})
        elif isinstance(a, ctypes._Pointer):
            base = type(a._type_()).__name__
            arr = np.ctypeslib.as_array(a, shape=shapes[k]).copy()
            name = {1: "ids", 2: "x", 3: "v", 4: "m"}[k]
            arrays[name] = arr
            spec.append({"kind": "array", "type": base, "name": name})
        elif isinstance(a, bytes):
            spec.append({"kind": "bytes", "value": a.decode()})
        elif isinstance(a, ctypes._SimpleCData):
            spec.append({"kind": "scalar", "type": tname, "value": a.value})
        else:
            raise TypeError(f"argument {k}: {tname}")
    return spec, arrays


def record(grav_sim, x, v, m, G, method, integrator, dt, tf, eps=0.0, theta=None, leaf=None,
           tolerance=None):
    from grav_sim import parameters
    from grav_sim.system import System
    lib_path = ROOT / "gravity-simulator_gb300" / "libgrav_sim_gb300.so"
    api = grav_sim.GravitySimulatorAPI(c_lib_path=str(lib_path))
    rec = Recorder()
    api.simulator.c_lib = rec
    system = System(api.c_lib)
    system.add(x, v, m)
    system.G = G
    ap = parameters.AccelerationParam()
    ap.method = method
    ap.softening_length = eps
    if theta is not None:   # otherwise grav_sim's defaults
        ap.opening_angle = theta
    if leaf is not None:
        ap.max_num_particles_per_leaf = leaf
    ip = parameters.IntegratorParam()
    ip.integrator = integrator
    ip.dt = dt
    if tolerance is not None:
        ip.tolerance = tolerance
    op = parameters.OutputParam()
    op.method = "disabled"
    st = parameters.Settings()
    st.verbose = "ignore_all"
    st.enable_progress_bar = False
    try:
        api.launch_simulation(system, ap, ip, op, st, tf)
    except RuntimeError:
        pass
    assert rec.args is not None, "grav_sim did not call launch_simulation_python"
    return describe(rec.args)


def main():
    grav_sim = import_grav_sim()
    # grav_sim resolves its default output folder "tmp/" against the working
    # directory (output is disabled in these calls): record it as "/tmp/"
    import os
    os.chdir("/")
    out = {}
    cases = []
    # leapfrog, FP64 pairwise in the reference's order: bit-exact to method 1
    x, v, m = wl.plummer(200, 8)
    cases.append(("leapfrog_fp64", x, v, m, 1.0, "gpu_pairwise_fp64", "leapfrog", 1e-3, 0.02,
                  dict(eps=0.01), 1, 0.0))
    # WHFast with the massless acceleration on a planetary system: bit-exact to method 2
    sys_ = wl.planetary_ensemble(1, 31, max_test=300)[0]   # 181 particles
    cases.append(("whfast_massless", sys_[0], sys_[1], sys_[2], wl.G_AU_MSUN_DAY,
                  "gpu_massless", "whfast", 1.0, 60.0, {}, 2, 0.0))
    # RK4 with the group walk on a galaxy pair against the reference's pairwise
    # sum: the tolerance bounds the median relative error of the velocity
    # change over the run (the force error's footprint)
    x, v, m = wl.galaxy_pair(4096, 31)
    cases.append(("rk4_group", x, v, m, 1.0, "gpu_barnes_hut_group", "rk4", 1e-3, 0.005,
                  dict(eps=0.01, theta=0.5, leaf=16), 1, 1e-3))
    names = []
    for name, x, v, m, G, method, integ, dt, tf, kw, ref_method, tol in cases:
        spec, arrays = record(grav_sim, x, v, m, G, method, integ, dt, tf, **kw)
        # the same call into the reference library, with its CPU method
        rc, idr, xr, vr, mr = replay(ref.load(), spec, arrays, method=ref_method)
        assert rc == 0, name
        if integ == "whfast":
            # grav_sim's WHFast reads its aux sums uninitialised
            # (src/integrator_whfast.c:1026/1063, undefined behaviour); the
            # policy is zeroed sums, which the oracle's restatement uses and
            # which a fresh reference process reproduces -- required here
            from oracle import restatement as orc
            G_ = spec[9]["value"]
            _, xo, vo, _ = orc.whfast_run(x, v, m, G_, 0.0, dt, tf, ids=arrays["ids"])
            assert np.array_equal(xo, xr) and np.array_equal(vo, vr), \
                "reference WHFast differs from the zeroed-aux restatement; rerun in a fresh process"
        out[f"{name}/spec.json"] = np.frombuffer(json.dumps(spec).encode(), dtype=np.uint8)
        for k, a in arrays.items():
            out[f"{name}/{k}"] = a
        out[f"{name}/ids_expected"] = idr
        out[f"{name}/m_expected"] = mr
        out[f"{name}/x_expected"] = xr
        out[f"{name}/v_expected"] = vr
        out[f"{name}/tolerance"] = np.float64(tol)
        names.append(name)
    np.savez_compressed(OUT / "dropin_calls.npz", **out)
    print("wrote", OUT / "dropin_calls.npz", names)


if __name__ == "__main__":
    main()
