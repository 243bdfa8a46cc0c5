"""ctypes mirror of grav_sim's C interface for the GB300 library.

The product is ``libgrav_sim_gb300.so`` (built in this directory by
``__graft_entry__.build()``).  It exports the same C symbols and struct
layouts as grav_sim's ``libgrav_sim`` (src/acceleration.h:20-26,
src/system.h:12-20, src/error.h:31-36, src/linear_octree.h:20-57,
src/python_interface.c:94-304), so this module mirrors grav_sim's own
ctypes layer (grav_sim/utils.py:12-58, grav_sim/simulator.py:22-143):
the same struct definitions, the same restypes, the same
thread + ``is_exit`` launch and the same ``RuntimeError`` on failure.

The GPU path is chosen through ``AccelerationParam.method`` with the GPU
method codes below; the CPU codes 1-3 of the reference are rejected by this
library with GRAV_VALUE_ERROR (there is no CPU fallback).
"""
from __future__ import annotations

import ctypes
import os
import threading
import time
from pathlib import Path
from queue import Queue
from typing import Optional

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_NAME = "libgrav_sim_gb300.so"

# grav_sim error codes (src/error.h:14-21)
GRAV_SUCCESS = 0
GRAV_VALUE_ERROR = 2
GRAV_POINTER_ERROR = 3
GRAV_MEMORY_ERROR = 4
GRAV_OS_ERROR = 5
GRAV_NOT_IMPLEMENTED_ERROR = 6

# Reference CPU method codes (src/acceleration.h:16-18); rejected here.
ACCELERATION_METHOD_PAIRWISE = 1
ACCELERATION_METHOD_MASSLESS = 2
ACCELERATION_METHOD_BARNES_HUT = 3

# GPU method codes of this library (same AccelerationParam.method field).
METHOD_GPU_PAIRWISE = 101          # compensated-FP32 direct sum
METHOD_GPU_MASSLESS = 102          # FP64 massive/massless direct sum
METHOD_GPU_BARNES_HUT = 103        # FP32 walk, true leaf multipoles
METHOD_GPU_BH_LEARNED = 104        # theta-cheap walk + learned MLP residual
METHOD_GPU_BARNES_HUT_QUAD = 105   # FP32 walk, monopole + quadrupole cell terms
METHOD_GPU_BARNES_HUT_GROUP = 106  # group walk with interaction lists, quadrupole cells
METHOD_GPU_BARNES_HUT_GROUP_MONO = 107  # group walk with interaction lists, monopole cells
METHOD_GPU_PAIRWISE_FP64 = 111     # FP64 direct sum in the reference's order
METHOD_GPU_BARNES_HUT_COMPAT = 113 # FP32 walk reproducing the reference's tree quirks

# Integrator codes (src/integrator.h:17-26)
INTEGRATOR_EULER = 1
INTEGRATOR_EULER_CROMER = 2
INTEGRATOR_RK4 = 3
INTEGRATOR_LEAPFROG = 4
INTEGRATOR_RKF45 = 5
INTEGRATOR_DOPRI = 6
INTEGRATOR_DVERK = 7
INTEGRATOR_RKF78 = 8
INTEGRATOR_IAS15 = 9
INTEGRATOR_WHFAST = 10

# Output codes (src/output.h:13-19)
OUTPUT_METHOD_DISABLED = 1
OUTPUT_METHOD_CSV = 2
OUTPUT_METHOD_HDF5 = 3
OUTPUT_DTYPE_FLOAT = 1
OUTPUT_DTYPE_DOUBLE = 2

c_double_p = ctypes.POINTER(ctypes.c_double)
c_int_p = ctypes.POINTER(ctypes.c_int32)
c_int64_p = ctypes.POINTER(ctypes.c_int64)


class System(ctypes.Structure):
    """src/system.h:12-20"""
    _fields_ = [
        ("num_particles", ctypes.c_int),
        ("particle_ids", c_int_p),
        ("x", c_double_p),
        ("v", c_double_p),
        ("m", c_double_p),
        ("G", ctypes.c_double),
    ]


class AccelerationParam(ctypes.Structure):
    """src/acceleration.h:20-26"""
    _fields_ = [
        ("method", ctypes.c_int),
        ("opening_angle", ctypes.c_double),
        ("softening_length", ctypes.c_double),
        ("max_num_particles_per_leaf", ctypes.c_int),
    ]


class ErrorStatus(ctypes.Structure):
    """src/error.h:31-36 (returned by value)"""
    _fields_ = [
        ("return_code", ctypes.c_int),
        ("traceback", ctypes.c_void_p),
        ("traceback_code_", ctypes.c_int),
    ]


class LinearOctree(ctypes.Structure):
    """src/linear_octree.h:20-57"""
    _fields_ = [
        ("box_width", ctypes.c_double),
        ("num_internal_nodes", ctypes.c_int),
        ("particle_morton_indices_deepest_level", c_int64_p),
        ("sorted_indices", c_int_p),
        ("tree_num_particles", c_int_p),
        ("tree_num_internal_children", c_int_p),
        ("tree_first_particle_sorted_idx", c_int_p),
        ("tree_first_internal_children_idx", c_int_p),
        ("tree_mass", c_double_p),
        ("tree_center_of_mass_x", c_double_p),
        ("tree_center_of_mass_y", c_double_p),
        ("tree_center_of_mass_z", c_double_p),
    ]


class CosmologicalSystem(ctypes.Structure):
    """src/system.h:22-38"""
    _fields_ = [
        ("num_particles", ctypes.c_int),
        ("particle_ids", c_int_p),
        ("x", c_double_p),
        ("v", c_double_p),
        ("m", c_double_p),
        ("h", ctypes.c_double),
        ("omega_m", ctypes.c_double),
        ("omega_lambda", ctypes.c_double),
        ("omega_k", ctypes.c_double),
        ("box_center", ctypes.c_double * 3),
        ("box_width", ctypes.c_double),
        ("unit_mass", ctypes.c_double),
        ("unit_length", ctypes.c_double),
        ("unit_time", ctypes.c_double),
    ]


class OutputParam(ctypes.Structure):
    """src/common.h:38-49"""
    _fields_ = [
        ("method", ctypes.c_int),
        ("output_dir", ctypes.c_char_p),
        ("output_initial", ctypes.c_bool),
        ("output_interval", ctypes.c_double),
        ("coordinate_output_dtype", ctypes.c_int),
        ("velocity_output_dtype", ctypes.c_int),
        ("mass_output_dtype", ctypes.c_int),
        ("output_count_", ctypes.c_int),
    ]


class SimulationStatus(ctypes.Structure):
    """src/common.h:51-56"""
    _fields_ = [("t", ctypes.c_double), ("dt", ctypes.c_double), ("num_steps", ctypes.c_int64)]


class Settings(ctypes.Structure):
    """src/settings.h:11-16"""
    _fields_ = [("verbose", ctypes.c_int), ("enable_progress_bar", ctypes.c_bool),
                ("is_exit_ptr", ctypes.POINTER(ctypes.c_bool))]


def library_path() -> Path:
    return HERE / LIB_NAME


def load_c_lib(c_lib_path: Optional[str | os.PathLike] = None) -> ctypes.CDLL:
    """Load the GB300 library (grav_sim/utils.py:12-35).  Fails loudly when
    the CUDA library has not been built: there is no fallback."""
    path = Path(c_lib_path) if c_lib_path else library_path()
    if not path.exists():
        raise FileNotFoundError(
            f"{path} not found: build it with __graft_entry__.build()")
    lib = ctypes.CDLL(str(path))
    initialize_c_lib(lib)
    return lib


def initialize_c_lib(lib: ctypes.CDLL) -> None:
    """Restypes of grav_sim/utils.py:38-58 plus the entry points used here."""
    lib.launch_simulation_python.restype = ctypes.c_int
    lib.compute_energy_python.restype = None
    lib.compute_linear_momentum_python.restype = None
    lib.compute_angular_momentum_python.restype = None
    lib.load_built_in_system_python.restype = ctypes.c_int
    lib.free_memory_int32.restype = None
    lib.free_memory_double.restype = None
    lib.keplerian_to_cartesian_python.restype = None
    lib.acceleration.restype = ErrorStatus
    lib.acceleration.argtypes = [c_double_p, ctypes.POINTER(System),
                                 ctypes.POINTER(AccelerationParam)]
    lib.free_traceback.restype = None
    lib.free_traceback.argtypes = [ctypes.POINTER(ErrorStatus)]
    if hasattr(lib, "construct_octree"):
        lib.construct_octree.restype = ErrorStatus
        lib.construct_octree.argtypes = [
            ctypes.POINTER(LinearOctree), ctypes.POINTER(System),
            ctypes.POINTER(AccelerationParam), c_double_p, ctypes.c_double]
        lib.free_linear_octree.restype = None
        lib.free_linear_octree.argtypes = [ctypes.POINTER(LinearOctree)]


def _dp(a: np.ndarray):
    return a.ctypes.data_as(c_double_p)


def _ip(a: np.ndarray):
    return a.ctypes.data_as(c_int_p)


def make_system(x: np.ndarray, m: np.ndarray, G: float,
                v: Optional[np.ndarray] = None,
                ids: Optional[np.ndarray] = None):
    """Wrap numpy arrays (C-contiguous float64 / int32) as a System without a
    copy, like src/python_interface.c:127-134.  Returns (system, keepalive)."""
    n = int(m.shape[0])
    x = np.ascontiguousarray(x, dtype=np.float64).reshape(n, 3)
    m = np.ascontiguousarray(m, dtype=np.float64)
    v = np.zeros_like(x) if v is None else np.ascontiguousarray(v, dtype=np.float64).reshape(n, 3)
    ids = np.arange(n, dtype=np.int32) if ids is None else np.ascontiguousarray(ids, dtype=np.int32)
    s = System(n, _ip(ids), _dp(x), _dp(v), _dp(m), float(G))
    return s, (x, v, m, ids)


def acceleration_pm(lib: ctypes.CDLL, x: np.ndarray, m: np.ndarray, box_center, box_width: float,
                    H0: float, omega_m: float, mean_bkg_density: float, pm_grid_size: int,
                    scale_factor: float) -> np.ndarray:
    """acceleration_PM (src/acceleration_PM.c:274-391) on host arrays."""
    lib.acceleration_PM.restype = ErrorStatus
    lib.acceleration_PM.argtypes = [c_double_p, ctypes.c_int, c_double_p, c_double_p, c_double_p,
                                    ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_double, ctypes.c_int, ctypes.c_double]
    x = np.ascontiguousarray(x, dtype=np.float64)
    m = np.ascontiguousarray(m, dtype=np.float64)
    c = np.ascontiguousarray(box_center, dtype=np.float64)
    a = np.empty((m.shape[0], 3))
    st = lib.acceleration_PM(_dp(a), int(m.shape[0]), _dp(x), _dp(m), _dp(c), float(box_width),
                             float(H0), float(omega_m), float(mean_bkg_density), int(pm_grid_size),
                             float(scale_factor))
    if st.return_code != 0:
        raise GravError(st.return_code, take_traceback(lib, st))
    return a


def launch_cosmological_simulation(lib: ctypes.CDLL, x: np.ndarray, v: np.ndarray, m: np.ndarray,
                                   *, h: float, omega_m: float, omega_lambda: float, box_center,
                                   box_width: float, dt: float, a_begin: float, a_final: float,
                                   pm_grid_size: int, output_method: int = OUTPUT_METHOD_DISABLED,
                                   ids: Optional[np.ndarray] = None,
                                   output_dir: Optional[str] = None, output_interval: float = 1.0,
                                   output_initial: bool = False,
                                   output_dtypes=(OUTPUT_DTYPE_DOUBLE,) * 3,
                                   units=(1.0, 1.0, 1.0)):
    """launch_cosmological_simulation (src/grav_sim.c:140-255).  x is advanced
    in place; v changes only at HDF5 snapshots (output_method 3, written to
    output_dir every output_interval of scale factor), where it becomes
    momentum / a^2 as in the reference.  output_dtypes: coordinates,
    velocities, masses; units: mass, length, time in cgs.  Returns the
    status (t = final scale factor, dt, num_steps)."""
    lib.launch_cosmological_simulation.restype = ErrorStatus
    lib.launch_cosmological_simulation.argtypes = [
        ctypes.POINTER(CosmologicalSystem), ctypes.POINTER(OutputParam),
        ctypes.POINTER(SimulationStatus), ctypes.POINTER(Settings), ctypes.c_double,
        ctypes.c_double, ctypes.c_double, ctypes.c_int]
    n = int(m.shape[0])
    assert x.flags.c_contiguous and x.dtype == np.float64 and v.flags.c_contiguous
    ids = np.arange(n, dtype=np.int32) if ids is None else np.ascontiguousarray(ids, np.int32)
    m = np.ascontiguousarray(m, dtype=np.float64)
    sysc = CosmologicalSystem(n, _ip(ids), _dp(x), _dp(v), _dp(m), float(h), float(omega_m),
                              float(omega_lambda), 1.0 - omega_m - omega_lambda,
                              (ctypes.c_double * 3)(*[float(q) for q in box_center]),
                              float(box_width), *[float(u) for u in units])
    out_dir = output_dir.encode() if output_dir is not None else None
    op = OutputParam(int(output_method), out_dir, bool(output_initial), float(output_interval),
                     *[int(d) for d in output_dtypes], 0)
    status = SimulationStatus(0.0, 0.0, 0)
    flag = ctypes.c_bool(False)
    settings = Settings(0, False, ctypes.pointer(flag))
    st = lib.launch_cosmological_simulation(ctypes.byref(sysc), ctypes.byref(op),
                                            ctypes.byref(status), ctypes.byref(settings),
                                            float(dt), float(a_begin), float(a_final),
                                            int(pm_grid_size))
    if st.return_code != 0:
        raise GravError(st.return_code, take_traceback(lib, st))
    return status


def write_snapshot_hdf5(lib: ctypes.CDLL, path, ids, x, v, m, t: float,
                        output_dtypes=(OUTPUT_DTYPE_DOUBLE,) * 3):
    """One HDF5 snapshot file in grav_sim's layout (gsgpu_write_snapshot_hdf5);
    output_dtypes: coordinates, velocities, masses."""
    lib.gsgpu_write_snapshot_hdf5.restype = ctypes.c_int
    lib.gsgpu_write_snapshot_hdf5.argtypes = [ctypes.c_char_p, ctypes.c_int, c_int_p, c_double_p,
                                              c_double_p, c_double_p, ctypes.c_double,
                                              ctypes.c_int, ctypes.c_int, ctypes.c_int]
    ids = np.ascontiguousarray(ids, dtype=np.int32)
    x, v, m = (np.ascontiguousarray(a, dtype=np.float64) for a in (x, v, m))
    n = int(m.shape[0])
    assert ids.shape == (n,) and x.size == 3 * n and v.size == 3 * n
    rc = lib.gsgpu_write_snapshot_hdf5(str(path).encode(), n, _ip(ids), _dp(x), _dp(v), _dp(m),
                                       float(t), *[int(d) for d in output_dtypes])
    if rc != 0:
        raise GravError(rc, f"gsgpu_write_snapshot_hdf5({path})")


def hdf5_read(lib: ctypes.CDLL, path, obj: str, attribute: Optional[str] = None) -> np.ndarray:
    """The values of a dataset (or of one attribute of an object) of an HDF5
    file as float64 (gsgpu_hdf5_read)."""
    lib.gsgpu_hdf5_read.restype = ctypes.c_int
    lib.gsgpu_hdf5_read.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p,
                                    c_double_p, ctypes.c_longlong,
                                    ctypes.POINTER(ctypes.c_longlong)]
    count = ctypes.c_longlong()
    attr = attribute.encode() if attribute is not None else None
    rc = lib.gsgpu_hdf5_read(str(path).encode(), obj.encode(), attr, None, 0, ctypes.byref(count))
    if rc != 0:
        raise GravError(rc, f"gsgpu_hdf5_read({path}, {obj}, {attribute})")
    out = np.empty(count.value, dtype=np.float64)
    rc = lib.gsgpu_hdf5_read(str(path).encode(), obj.encode(), attr, _dp(out), out.size,
                             ctypes.byref(count))
    if rc != 0:
        raise GravError(rc, f"gsgpu_hdf5_read({path}, {obj}, {attribute})")
    return out


def load_gadget2_ic(lib: ctypes.CDLL, path):
    """Gadget-2 HDF5 initial conditions (load_gadget2_ic): returns
    (x, v, m, (unit_length, unit_mass, unit_time)) as numpy copies."""
    lib.load_gadget2_ic.restype = ErrorStatus
    lib.load_gadget2_ic.argtypes = [ctypes.c_char_p, ctypes.POINTER(System), c_double_p,
                                    c_double_p, c_double_p]
    lib.free_system.restype = None
    lib.free_system.argtypes = [ctypes.POINTER(System)]
    s = System()
    units = (ctypes.c_double * 3)()
    st = lib.load_gadget2_ic(str(path).encode(), ctypes.byref(s),
                             ctypes.cast(ctypes.byref(units, 0), c_double_p),
                             ctypes.cast(ctypes.byref(units, 8), c_double_p),
                             ctypes.cast(ctypes.byref(units, 16), c_double_p))
    if st.return_code != 0:
        raise GravError(st.return_code, take_traceback(lib, st))
    n = s.num_particles
    x = np.ctypeslib.as_array(s.x, (n, 3)).copy()
    v = np.ctypeslib.as_array(s.v, (n, 3)).copy()
    m = np.ctypeslib.as_array(s.m, (n,)).copy()
    ids = np.ctypeslib.as_array(s.particle_ids, (n,)).copy()
    lib.free_system(ctypes.byref(s))
    assert (ids == np.arange(n)).all()
    return x, v, m, tuple(units)


def take_traceback(lib: ctypes.CDLL, st: ErrorStatus) -> str:
    text = ""
    if st.traceback:
        text = ctypes.string_at(st.traceback).decode("utf-8", "replace")
        lib.free_traceback(ctypes.byref(st))
    return text


class GravError(RuntimeError):
    def __init__(self, code: int, traceback: str):
        super().__init__(f"grav_sim error {code}: {traceback}")
        self.code = code
        self.traceback = traceback


def acceleration(lib: ctypes.CDLL, x: np.ndarray, m: np.ndarray, G: float,
                 method: int, opening_angle: float = 1.0,
                 softening_length: float = 0.0,
                 max_num_particles_per_leaf: int = -1) -> np.ndarray:
    """Call ``acceleration(a, system, param)`` (src/acceleration.h:53-57)
    with host buffers and return a as an (N, 3) array."""
    system, keep = make_system(x, m, G)
    a = np.empty((system.num_particles, 3), dtype=np.float64)
    p = AccelerationParam(int(method), float(opening_angle),
                          float(softening_length), int(max_num_particles_per_leaf))
    st = lib.acceleration(_dp(a), ctypes.byref(system), ctypes.byref(p))
    if st.return_code != GRAV_SUCCESS:
        raise GravError(st.return_code, take_traceback(lib, st))
    del keep
    return a


def launch_simulation(lib: ctypes.CDLL, x: np.ndarray, v: np.ndarray,
                      m: np.ndarray, G: float, *, integrator: int, dt: float,
                      tf: float, method: int, opening_angle: float = 1.0,
                      softening_length: float = 0.0,
                      max_num_particles_per_leaf: int = -1,
                      tolerance: float = -1.0, initial_dt: float = -1.0,
                      whfast_remove_invalid_particles: bool = True,
                      ids: Optional[np.ndarray] = None, verbose: int = 0,
                      is_exit: Optional[ctypes.c_bool] = None,
                      output_method: int = OUTPUT_METHOD_DISABLED,
                      output_dir: Optional[str] = None, output_initial: bool = False,
                      output_interval: float = 0.0,
                      coordinate_output_dtype: int = OUTPUT_DTYPE_DOUBLE,
                      velocity_output_dtype: int = OUTPUT_DTYPE_DOUBLE,
                      mass_output_dtype: int = OUTPUT_DTYPE_DOUBLE):
    """Mirror of Simulator.launch_simulation (grav_sim/simulator.py:22-143):
    runs ``launch_simulation_python`` on a worker thread, raises
    RuntimeError when it returns non-zero, and returns the (possibly
    shrunk) (ids, x, v, m) arrays.  x and v are updated in place.  The
    output arguments are those of grav_sim/parameters.py's OutputParam
    (``output_dir`` None lets the library name a snapshots_<date>/ folder)."""
    n = int(m.shape[0])
    num = ctypes.c_int32(n)
    ids = np.arange(n, dtype=np.int32) if ids is None else ids
    new_ids = c_int_p()
    new_x = c_double_p()
    new_v = c_double_p()
    new_m = c_double_p()
    flag = ctypes.c_bool(False) if is_exit is None else is_exit
    q: Queue = Queue()

    def run(*args):
        q.put(lib.launch_simulation_python(*args))

    args = (
        ctypes.byref(num), _ip(ids), _dp(x), _dp(v), _dp(m),
        ctypes.byref(new_ids), ctypes.byref(new_x), ctypes.byref(new_v),
        ctypes.byref(new_m), ctypes.c_double(G), ctypes.c_int32(integrator),
        ctypes.c_double(dt), ctypes.c_double(tolerance),
        ctypes.c_double(initial_dt), ctypes.c_bool(whfast_remove_invalid_particles),
        ctypes.c_int32(method), ctypes.c_double(opening_angle),
        ctypes.c_double(softening_length), ctypes.c_int32(max_num_particles_per_leaf),
        ctypes.c_int32(output_method),
        None if output_dir is None else ctypes.c_char_p(str(output_dir).encode()),
        ctypes.c_bool(output_initial), ctypes.c_double(output_interval),
        ctypes.c_int32(coordinate_output_dtype), ctypes.c_int32(velocity_output_dtype),
        ctypes.c_int32(mass_output_dtype),
        ctypes.c_int32(verbose), ctypes.c_bool(False), ctypes.byref(flag),
        ctypes.c_double(tf),
    )
    th = threading.Thread(target=run, args=args)
    th.start()
    while th.is_alive():
        time.sleep(0.002)
    th.join()
    ret = q.get()
    if ret != 0:
        raise RuntimeError("Simulation failed. Please check the C library traceback.")
    k = num.value
    # The C side returns the caller's own buffers (src/python_interface.c:186-190),
    # possibly compacted to k particles; hand back views of the numpy arrays
    # that own that memory so they stay alive with the result.
    assert ctypes.addressof(new_x.contents) == x.ctypes.data
    return (ids[:k], x.reshape(-1, 3)[:k], v.reshape(-1, 3)[:k], m[:k])


class Ensemble:
    """Batched planetary ensembles (``gsgpu_ensemble_*``): many independent
    systems of uneven size advanced together on the GPU by WHFast
    (INTEGRATOR_WHFAST) or leapfrog (INTEGRATOR_LEAPFROG) with the massless or
    pairwise accelerations.  Each system evolves as the reference's
    ``launch_simulation`` evolves it alone (src/integrator_whfast.c:200-407,
    src/integrator.c:894-1121).

    ``counts`` gives the particles per system; ``ids``, ``x``, ``v``, ``m``
    are the systems concatenated, ids system-local with the primary's id 0.
    """

    def __init__(self, lib: ctypes.CDLL, counts, G: float, *, integrator: int,
                 method: int, dt: float, softening_length: float = 0.0,
                 remove_invalid_particles: bool = True):
        self.lib = lib
        _init_ensemble_api(lib)
        self.counts = np.ascontiguousarray(counts, dtype=np.int32)
        self.num_systems = int(self.counts.shape[0])
        self.num_particles = int(self.counts.sum())
        h = ctypes.c_void_p()
        rc = lib.gsgpu_ensemble_create(
            ctypes.byref(h), self.num_systems, _ip(self.counts), float(G), int(integrator),
            int(method), float(softening_length), float(dt), int(bool(remove_invalid_particles)),
            None)
        if rc != 0:
            raise GravError(rc, "gsgpu_ensemble_create failed")
        self.handle = h

    def _check(self, rc: int, what: str) -> None:
        if rc != 0:
            raise GravError(rc, f"{what} failed")

    def upload(self, ids: np.ndarray, x: np.ndarray, v: np.ndarray, m: np.ndarray) -> None:
        P = self.num_particles
        self._keep = (np.ascontiguousarray(ids, dtype=np.int32).reshape(P),
                      np.ascontiguousarray(x, dtype=np.float64).reshape(P, 3),
                      np.ascontiguousarray(v, dtype=np.float64).reshape(P, 3),
                      np.ascontiguousarray(m, dtype=np.float64).reshape(P))
        i, xx, vv, mm = self._keep
        self._check(self.lib.gsgpu_ensemble_upload(self.handle, _ip(i), _dp(xx), _dp(vv), _dp(mm)),
                    "gsgpu_ensemble_upload")

    def run(self, num_steps: int) -> None:
        self._check(self.lib.gsgpu_ensemble_run(self.handle, ctypes.c_int64(int(num_steps))),
                    "gsgpu_ensemble_run")

    def run_until(self, tf: float) -> None:
        self._check(self.lib.gsgpu_ensemble_run_until(self.handle, ctypes.c_double(tf)),
                    "gsgpu_ensemble_run_until")

    def download(self):
        """Returns (counts, ids, x, v, m); system s occupies the first
        counts[s] slots of its block (blocks at the original offsets)."""
        P = self.num_particles
        counts = np.empty(self.num_systems, dtype=np.int32)
        ids = np.empty(P, dtype=np.int32)
        x = np.empty((P, 3))
        v = np.empty((P, 3))
        m = np.empty(P)
        self._check(self.lib.gsgpu_ensemble_download(self.handle, _ip(counts), _ip(ids), _dp(x),
                                                     _dp(v), _dp(m)),
                    "gsgpu_ensemble_download")
        return counts, ids, x, v, m

    def kernels_per_step(self) -> int:
        return int(self.lib.gsgpu_ensemble_kernels_per_step(self.handle))

    def tuning(self):
        """(accel, drift) thread-block sizes chosen by the autotuner."""
        a, d = ctypes.c_int(), ctypes.c_int()
        self._check(self.lib.gsgpu_ensemble_tuning(self.handle, ctypes.byref(a), ctypes.byref(d)),
                    "gsgpu_ensemble_tuning")
        return a.value, d.value

    def sort_tuning(self):
        """[(size-class capacity, threads per system)] of the sort by distance."""
        p2 = np.zeros(8, dtype=np.int32)
        th = np.zeros(8, dtype=np.int32)
        k = self.lib.gsgpu_ensemble_sort_tuning(self.handle, _ip(p2), _ip(th), 8)
        return [(int(p2[i]), int(th[i])) for i in range(max(k, 0))]

    def set_kernel_timing(self, enable: bool) -> None:
        """Direct launches with CUDA events around the drift and the
        accelerations (instead of graph replays) while enabled."""
        self._check(self.lib.gsgpu_ensemble_set_kernel_timing(self.handle, int(bool(enable))),
                    "gsgpu_ensemble_set_kernel_timing")

    def kernel_timing(self):
        """(drift ms, acceleration ms, timed steps) summed since timing was
        enabled."""
        d, a, k = ctypes.c_double(), ctypes.c_double(), ctypes.c_int64()
        self._check(self.lib.gsgpu_ensemble_kernel_timing(self.handle, ctypes.byref(d),
                                                          ctypes.byref(a), ctypes.byref(k)),
                    "gsgpu_ensemble_kernel_timing")
        return d.value, a.value, k.value

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.lib.gsgpu_ensemble_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _init_ensemble_api(lib: ctypes.CDLL) -> None:
    if getattr(lib, "_ensemble_api", False):
        return
    vp = ctypes.c_void_p
    lib.gsgpu_ensemble_create.restype = ctypes.c_int
    lib.gsgpu_ensemble_create.argtypes = [ctypes.POINTER(vp), ctypes.c_int, c_int_p,
                                          ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_double, ctypes.c_double, ctypes.c_int, vp]
    lib.gsgpu_ensemble_upload.restype = ctypes.c_int
    lib.gsgpu_ensemble_upload.argtypes = [vp, c_int_p, c_double_p, c_double_p, c_double_p]
    lib.gsgpu_ensemble_run.restype = ctypes.c_int
    lib.gsgpu_ensemble_run.argtypes = [vp, ctypes.c_int64]
    lib.gsgpu_ensemble_run_until.restype = ctypes.c_int
    lib.gsgpu_ensemble_run_until.argtypes = [vp, ctypes.c_double]
    lib.gsgpu_ensemble_download.restype = ctypes.c_int
    lib.gsgpu_ensemble_download.argtypes = [vp, c_int_p, c_int_p, c_double_p, c_double_p,
                                            c_double_p]
    lib.gsgpu_ensemble_kernels_per_step.restype = ctypes.c_int
    lib.gsgpu_ensemble_kernels_per_step.argtypes = [vp]
    lib.gsgpu_ensemble_tuning.restype = ctypes.c_int
    lib.gsgpu_ensemble_tuning.argtypes = [vp, c_int_p, c_int_p]
    lib.gsgpu_ensemble_sort_tuning.restype = ctypes.c_int
    lib.gsgpu_ensemble_sort_tuning.argtypes = [vp, c_int_p, c_int_p, ctypes.c_int]
    lib.gsgpu_ensemble_set_kernel_timing.restype = ctypes.c_int
    lib.gsgpu_ensemble_set_kernel_timing.argtypes = [vp, ctypes.c_int]
    lib.gsgpu_ensemble_kernel_timing.restype = ctypes.c_int
    lib.gsgpu_ensemble_kernel_timing.argtypes = [vp, c_double_p, c_double_p,
                                                 ctypes.POINTER(ctypes.c_int64)]
    lib.gsgpu_ensemble_destroy.restype = None
    lib.gsgpu_ensemble_destroy.argtypes = [vp]
    lib._ensemble_api = True
