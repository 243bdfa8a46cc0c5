"""ctypes wrapper of grav_sim itself, compiled from its own sources.

TEST INFRASTRUCTURE ONLY.  ``oracle/Makefile`` target ``ref`` compiles the
unmodified reference C sources (read in place, never copied) into
oracle/_ref/libgrav_sim_ref.so (serial) and libgrav_sim_ref_omp.so (OpenMP).
Those files exist only where the reference sources were present at build
time; ``available()`` says whether they are here.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REF_DIR = Path(os.environ.get("GRAV_SIM_REFERENCE_DIR", "/root/reference"))
SERIAL = HERE / "_ref" / "libgrav_sim_ref.so"
OPENMP = HERE / "_ref" / "libgrav_sim_ref_omp.so"
# the reference with its particle-mesh sources, FFTW calls served by the
# oracle's direct DFT (oracle/fftw_compat)
PM = HERE / "_ref" / "libgrav_sim_ref_pm.so"

_PKG = HERE.parent / "gravity-simulator_gb300"


def _gsgpu():
    import importlib.util
    spec = importlib.util.spec_from_file_location("gsgpu_abi", _PKG / "gsgpu.py")
    mod = sys.modules.get("gsgpu_abi")
    if mod is None:
        mod = importlib.util.module_from_spec(spec)
        sys.modules["gsgpu_abi"] = mod
        spec.loader.exec_module(mod)
    return mod


def build() -> bool:
    """Compile oracle/_ref from the reference sources, if they are present."""
    if not (REF_DIR / "src" / "acceleration.c").exists():
        return False
    subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF_DIR={REF_DIR}"], check=True)
    return SERIAL.exists()


def _loadable(path: Path) -> bool:
    if not path.exists():
        return False
    try:
        ctypes.CDLL(str(path))
        return True
    except OSError:
        return False


def available(openmp: bool = False) -> bool:
    return _loadable(OPENMP if openmp else SERIAL)


_cache = {}


def load(openmp: bool = False) -> ctypes.CDLL:
    key = bool(openmp)
    if key not in _cache:
        g = _gsgpu()
        lib = ctypes.CDLL(str(OPENMP if openmp else SERIAL))
        lib.acceleration.restype = g.ErrorStatus
        lib.acceleration.argtypes = [g.c_double_p, ctypes.POINTER(g.System),
                                     ctypes.POINTER(g.AccelerationParam)]
        lib.construct_octree.restype = g.ErrorStatus
        lib.construct_octree.argtypes = [ctypes.POINTER(g.LinearOctree), ctypes.POINTER(g.System),
                                         ctypes.POINTER(g.AccelerationParam), g.c_double_p,
                                         ctypes.c_double]
        lib.get_new_linear_octree.restype = g.LinearOctree
        lib.free_linear_octree.restype = None
        lib.free_linear_octree.argtypes = [ctypes.POINTER(g.LinearOctree)]
        lib.launch_simulation_python.restype = ctypes.c_int
        lib.compute_energy_python.restype = None
        lib.compute_linear_momentum_python.restype = None
        lib.compute_angular_momentum_python.restype = None
        lib.free_traceback.restype = None
        lib.free_traceback.argtypes = [ctypes.POINTER(g.ErrorStatus)]
        _cache[key] = lib
    return _cache[key]


def acceleration(x, m, G, method, theta=1.0, eps=0.0, leaf=-1, openmp=False):
    g = _gsgpu()
    return g.acceleration(load(openmp), x, m, G, method, theta, eps, leaf)


def octree(x, m, leaf_max):
    """construct_octree (src/linear_octree.c:825-962): keys, sorted ids and
    the node arrays, copied out (only fields the reference defines)."""
    g = _gsgpu()
    lib = load()
    system, keep = g.make_system(x, m, 1.0)
    t = lib.get_new_linear_octree()
    p = g.AccelerationParam(3, 1.0, 0.0, int(leaf_max))
    st = lib.construct_octree(ctypes.byref(t), ctypes.byref(system), ctypes.byref(p), None, -1.0)
    assert st.return_code == 0, g.take_traceback(lib, st)
    n, nn = system.num_particles, t.num_internal_nodes
    nic = np.ctypeslib.as_array(t.tree_num_internal_children, (nn,)).copy()
    fic = np.ctypeslib.as_array(t.tree_first_internal_children_idx, (nn,)).copy()
    fic = np.where(nic > 0, fic, -1)
    out = dict(
        box_width=t.box_width, num_nodes=nn,
        keys=np.ctypeslib.as_array(t.particle_morton_indices_deepest_level, (n,)).copy(),
        sorted_indices=np.ctypeslib.as_array(t.sorted_indices, (n,)).copy(),
        num_particles=np.ctypeslib.as_array(t.tree_num_particles, (nn,)).copy(),
        num_children=nic,
        first_particle=np.ctypeslib.as_array(t.tree_first_particle_sorted_idx, (nn,)).copy(),
        first_child=fic,
        mass=np.ctypeslib.as_array(t.tree_mass, (nn,)).copy(),
        com=np.stack([np.ctypeslib.as_array(t.tree_center_of_mass_x, (nn,)).copy(),
                      np.ctypeslib.as_array(t.tree_center_of_mass_y, (nn,)).copy(),
                      np.ctypeslib.as_array(t.tree_center_of_mass_z, (nn,)).copy()], 1),
    )
    lib.free_linear_octree(ctypes.byref(t))
    del keep
    return out


def launch(x, v, m, G, integrator, dt, tf, method, theta=1.0, eps=0.0, leaf=-1,
           tolerance=-1.0, initial_dt=-1.0, openmp=False, **output):
    g = _gsgpu()
    x = np.ascontiguousarray(x, dtype=np.float64).copy()
    v = np.ascontiguousarray(v, dtype=np.float64).copy()
    m = np.ascontiguousarray(m, dtype=np.float64).copy()
    ids, xo, vo, mo = g.launch_simulation(
        load(openmp), x, v, m, G, integrator=integrator, dt=dt, tf=tf, method=method,
        opening_angle=theta, softening_length=eps, max_num_particles_per_leaf=leaf,
        tolerance=tolerance, initial_dt=initial_dt, **output)
    return ids.copy(), xo.copy(), vo.copy(), mo.copy()


def load_pm() -> ctypes.CDLL:
    if "pm" not in _cache:
        g = _gsgpu()
        lib = ctypes.CDLL(str(PM))
        lib.free_traceback.restype = None
        lib.free_traceback.argtypes = [ctypes.POINTER(g.ErrorStatus)]
        _cache["pm"] = lib
    return _cache["pm"]


def acceleration_pm(x, m, box_center, box_width, H0, omega_m, mean_bkg_density, grid,
                    scale_factor):
    """acceleration_PM (src/acceleration_PM.c:274-391) of the reference."""
    g = _gsgpu()
    return g.acceleration_pm(load_pm(), x, m, box_center, box_width, H0, omega_m,
                             mean_bkg_density, grid, scale_factor)


def cosmological_run(x, v, m, **kw):
    """launch_cosmological_simulation of the reference; returns (x, status)."""
    g = _gsgpu()
    x = np.ascontiguousarray(x, dtype=np.float64).copy()
    v = np.ascontiguousarray(v, dtype=np.float64).copy()
    st = g.launch_cosmological_simulation(load_pm(), x, v, m, **kw)
    return x, (st.t, st.dt, st.num_steps)


def energy_python(x, v, m, G):
    lib = load()
    n = m.size
    state = np.concatenate([m[:, None], x, v], axis=1).astype(np.float64)
    state = np.ascontiguousarray(state)
    e = np.empty(1)
    lib.compute_energy_python(e.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                              ctypes.c_double(G),
                              state.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                              ctypes.c_int32(1), ctypes.c_int32(n))
    return float(e[0])
