"""C ABI checks that need no GPU: the library loads, exports every symbol
include/grav_sim_gb300.h declares, lays its structs out exactly like
grav_sim, and applies grav_sim's parameter validation on the host."""
import ctypes
import subprocess
import sys
import textwrap
from pathlib import Path

import pytest

from conftest import ROOT

sys.path.insert(0, str(ROOT))
import __graft_entry__ as entry  # noqa: E402

HEADER = ROOT / "include" / "grav_sim_gb300.h"


def test_exports_every_declared_symbol(lib):
    names = entry.declared_symbols()
    assert "acceleration" in names and "launch_simulation_python" in names
    missing = [s for s in names if not hasattr(lib, s)]
    assert not missing, missing


LAYOUT_C = textwrap.dedent("""
    #include <stdio.h>
    #include <stddef.h>
    #include HDR
    #define P(T, f) printf(#T "." #f " %zu\\n", offsetof(T, f));
    int main(void) {
      printf("System %zu\\n", sizeof(System));
      P(System, num_particles) P(System, particle_ids) P(System, x) P(System, v) P(System, m) P(System, G)
      printf("AccelerationParam %zu\\n", sizeof(AccelerationParam));
      P(AccelerationParam, method) P(AccelerationParam, opening_angle)
      P(AccelerationParam, softening_length) P(AccelerationParam, max_num_particles_per_leaf)
      printf("ErrorStatus %zu\\n", sizeof(ErrorStatus));
      P(ErrorStatus, traceback) P(ErrorStatus, traceback_code_)
      printf("IntegratorParam %zu\\n", sizeof(IntegratorParam));
      P(IntegratorParam, dt) P(IntegratorParam, whfast_remove_invalid_particles)
      printf("OutputParam %zu\\n", sizeof(OutputParam));
      P(OutputParam, output_dir) P(OutputParam, output_interval) P(OutputParam, output_count_)
      printf("SimulationStatus %zu\\n", sizeof(SimulationStatus));
      printf("Settings %zu\\n", sizeof(Settings));
      P(Settings, is_exit_ptr)
      printf("LinearOctree %zu\\n", sizeof(LinearOctree));
      P(LinearOctree, num_internal_nodes) P(LinearOctree, sorted_indices)
      P(LinearOctree, tree_center_of_mass_z)
      return 0;
    }
""")


def _layout(tmp_path, include_line: str, extra_flags=()):
    src = tmp_path / "layout.c"
    src.write_text(LAYOUT_C.replace("HDR", include_line))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=gnu99", *extra_flags, "-o", str(exe), str(src)], check=True)
    return subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout


def test_struct_layout_matches_reference(tmp_path):
    ours = _layout(tmp_path, f'"{HEADER}"')
    assert "System 48" in ours and "AccelerationParam 32" in ours and "ErrorStatus 24" in ours
    refsrc = Path("/root/reference/src")
    if not (refsrc / "linear_octree.h").exists():
        pytest.skip("reference headers not present")
    shim = tmp_path / "ref_all.h"
    shim.write_text('#include "common.h"\n#include "error.h"\n#include "system.h"\n'
                    '#include "acceleration.h"\n#include "linear_octree.h"\n'
                    '#include "settings.h"\n')
    theirs = _layout(tmp_path, f'"{shim}"', [f"-I{refsrc}"])
    assert ours == theirs


def test_ctypes_mirror_sizes(g):
    assert ctypes.sizeof(g.System) == 48
    assert ctypes.sizeof(g.AccelerationParam) == 32
    assert ctypes.sizeof(g.ErrorStatus) == 24
    assert ctypes.sizeof(g.LinearOctree) == 96


def test_finalize_acceleration_param_host_logic(lib, g):
    f = lib.finalize_acceleration_param
    f.restype = g.ErrorStatus
    f.argtypes = [ctypes.POINTER(g.AccelerationParam)]
    p = g.AccelerationParam(g.METHOD_GPU_BARNES_HUT, 0.5, 0.01, -1)
    st = f(ctypes.byref(p))
    assert st.return_code == 0 and p.max_num_particles_per_leaf == 1
    p = g.AccelerationParam(g.METHOD_GPU_BARNES_HUT, 0.5, 0.01, 0)
    st = f(ctypes.byref(p))
    assert st.return_code == g.GRAV_VALUE_ERROR
    assert "per leaf" in g.take_traceback(lib, st)
    p = g.AccelerationParam(g.METHOD_GPU_PAIRWISE, 1.0, -0.1, -1)
    st = f(ctypes.byref(p))
    assert st.return_code == g.GRAV_VALUE_ERROR
    assert "Softening" in g.take_traceback(lib, st)
    # the reference's CPU codes are not accepted: no CPU fallback
    for cpu_code in (1, 2, 3):
        p = g.AccelerationParam(cpu_code, 1.0, 0.0, -1)
        st = f(ctypes.byref(p))
        assert st.return_code == g.GRAV_VALUE_ERROR
        g.take_traceback(lib, st)


def test_launch_validation_order_on_host(lib, g):
    """finalize_system runs first (src/grav_sim.c:73-78): a bad G fails before
    any device work and launch_simulation_python returns 1."""
    import numpy as np
    x = np.zeros((4, 3))
    v = np.zeros((4, 3))
    m = np.ones(4)
    with pytest.raises(RuntimeError):
        g.launch_simulation(lib, x, v, m, -1.0, integrator=4, dt=1e-3, tf=0.01,
                            method=g.METHOD_GPU_PAIRWISE)
    with pytest.raises(RuntimeError):     # CPU method code rejected
        g.launch_simulation(lib, x, v, m, 1.0, integrator=4, dt=1e-3, tf=0.01, method=1)
    with pytest.raises(RuntimeError):     # unknown integrator
        g.launch_simulation(lib, x, v, m, 1.0, integrator=42, dt=1e-3, tf=0.01,
                            method=g.METHOD_GPU_PAIRWISE)


def test_check_if_included(lib):
    f = lib.linear_octree_check_if_included
    f.restype = ctypes.c_bool
    f.argtypes = [ctypes.c_int64, ctypes.c_int64, ctypes.c_int]
    assert f(0b111000, 0b111111, 20)
    assert not f(0b111000, 0b111111, 21)
