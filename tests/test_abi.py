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
      printf("CosmologicalSystem %zu\\n", sizeof(CosmologicalSystem));
      P(CosmologicalSystem, m) P(CosmologicalSystem, h) P(CosmologicalSystem, omega_k)
      P(CosmologicalSystem, box_center) P(CosmologicalSystem, box_width)
      P(CosmologicalSystem, unit_time)
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
    from oracle.reference import REF_DIR
    refsrc = REF_DIR / "src"
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
    assert ctypes.sizeof(g.CosmologicalSystem) == 128
    assert ctypes.sizeof(g.OutputParam) == 48


def test_finalize_acceleration_param_host_logic(lib, g):
    f = lib.finalize_acceleration_param
    f.restype = g.ErrorStatus
    f.argtypes = [ctypes.POINTER(g.AccelerationParam)]
    p = g.AccelerationParam(g.METHOD_GPU_BARNES_HUT, 0.5, 0.01, -1)
    st = f(ctypes.byref(p))
    assert st.return_code == 0 and p.max_num_particles_per_leaf == 1
    p = g.AccelerationParam(106, 0.5, 0.01, -1)    # the group walks default to 16 per leaf
    st = f(ctypes.byref(p))
    assert st.return_code == 0 and p.max_num_particles_per_leaf == 16
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


def test_output_param_checks_on_host(lib, g, tmp_path, capfd):
    """finalize_output_param (src/output.c:126-239) runs before any device
    work: each bad output argument fails with the reference's message, and
    a valid snapshot folder is created (the run itself then needs a GPU)."""
    import numpy as np
    x, v, m = np.zeros((4, 3)), np.zeros((4, 3)), np.ones(4)
    bad = [
        (dict(output_method=2, output_dir=str(tmp_path / "a"), output_interval=1.0),
         "must end with a trailing slash"),
        (dict(output_method=2, output_dir=str(tmp_path / "b") + "/", output_interval=0.0),
         "Output interval must be positive"),
        (dict(output_method=3, output_dir=str(tmp_path / "b") + "/", output_interval=-1.0),
         "Output interval must be positive"),
        (dict(output_method=7, output_dir=str(tmp_path / "b") + "/", output_interval=1.0),
         "Unknown output method"),
    ]
    capfd.readouterr()
    for kw, msg in bad:
        with pytest.raises(RuntimeError):
            g.launch_simulation(lib, x.copy(), v.copy(), m, 1.0, integrator=4, dt=1e-3, tf=0.01,
                                method=g.METHOD_GPU_PAIRWISE, **kw)
        assert msg in capfd.readouterr().err
    assert not (tmp_path / "a").exists() and not (tmp_path / "b").exists()
    try:
        g.launch_simulation(lib, x.copy(), v.copy(), m, 1.0, integrator=4, dt=1e-3, tf=0.0,
                            method=g.METHOD_GPU_PAIRWISE, output_method=2,
                            output_dir=str(tmp_path / "c") + "/", output_interval=1.0)
    except RuntimeError:
        pass
    assert (tmp_path / "c").is_dir()
    try:    # HDF5 output (method 3) is accepted as well
        g.launch_simulation(lib, x.copy(), v.copy(), m, 1.0, integrator=4, dt=1e-3, tf=0.0,
                            method=g.METHOD_GPU_PAIRWISE, output_method=3,
                            output_dir=str(tmp_path / "d") + "/", output_interval=1.0)
    except RuntimeError:
        pass
    assert (tmp_path / "d").is_dir()


def test_check_if_included(lib):
    f = lib.linear_octree_check_if_included
    f.restype = ctypes.c_bool
    f.argtypes = [ctypes.c_int64, ctypes.c_int64, ctypes.c_int]
    assert f(0b111000, 0b111111, 20)
    assert not f(0b111000, 0b111111, 21)


def test_cosmological_checks_on_host(lib, g, capfd, tmp_path):
    """launch_cosmological_simulation's checks (src/grav_sim.c:166-229) run
    before any device work, in the reference's order and words."""
    import numpy as np
    x, v, m = np.zeros((4, 3)), np.zeros((4, 3)), np.ones(4)
    good = dict(h=0.7, omega_m=0.3, omega_lambda=0.7, box_center=[0, 0, 0], box_width=1.0,
                dt=0.01, a_begin=0.1, a_final=0.2, pm_grid_size=8)
    bad = [
        (dict(h=-1.0), "Hubble parameter"),
        (dict(box_width=0.0), "Box width must be positive"),
        (dict(output_method=2), "CSV output is not supported"),
        (dict(output_method=3, output_dir=str(tmp_path / "h")), "must end with a trailing slash"),
        (dict(output_method=3, output_dir=str(tmp_path / "h") + "/", output_interval=0.0),
         "Output interval must be positive"),
        (dict(dt=-1.0), "dt must be non=negative"),
        (dict(a_begin=0.0), "a_begin must be positive"),
        (dict(a_final=0.05), "a_final must be greater or equal"),
        (dict(pm_grid_size=0), "pm_grid_size must be positive"),
    ]
    for over, msg in bad:
        kw = dict(good, **over)
        with pytest.raises(g.GravError) as e:
            g.launch_cosmological_simulation(lib, x.copy(), v.copy(), m, **kw)
        assert msg in str(e.value), (msg, str(e.value))


def test_recorded_grav_sim_calls_match_the_abi():
    """The launch_simulation_python calls recorded from grav_sim's Simulator
    (tests/golden/dropin_calls.npz) have the 30 arguments of
    src/python_interface.c:94-125 in grav_sim's types: the particle count and
    exit flag by reference, four input arrays, four output pointers, one
    output folder string and 19 scalars of the declared types."""
    import json
    import numpy as np
    from conftest import cases, golden
    for name, c in cases(golden("dropin_calls")).items():
        spec = json.loads(bytes(c["spec.json"]).decode())
        kinds = [a["kind"] for a in spec]
        assert len(spec) == 30, name
        assert kinds[0] == "byref" and kinds[28] == "byref", name
        assert kinds[1:5] == ["array"] * 4 and kinds[5:9] == ["out_pointer"] * 4, name
        assert kinds[20] == "bytes" and kinds.count("scalar") == 19, name
        n = spec[0]["value"]
        assert c["x"].shape == (n, 3) and c["m"].shape == (n,), name


def test_print_compilation_info(lib, capfd):
    """grav_sim's `python -m grav_sim` calls print_compilation_info
    (grav_sim/__main__.py; src/grav_sim.h:92): it is exported and prints the
    build's facts in the reference's sections, without touching a GPU."""
    lib.print_compilation_info.restype = None
    capfd.readouterr()
    lib.print_compilation_info()
    out = capfd.readouterr().out
    assert "Operating System:" in out and "Compilation Info:" in out and "Build time:" in out
    assert "sm_103a" in out


def test_rk_error_sum_switch(lib, g):
    """gsgpu_set_rk_error_sum takes 0 (the reference's order on the host,
    the default) or 1 (on the device) and rejects other modes; it only sets a
    flag, so it runs without a GPU."""
    lib.gsgpu_set_rk_error_sum.argtypes = [ctypes.c_int]
    assert lib.gsgpu_set_rk_error_sum(2) == g.GRAV_VALUE_ERROR
    assert lib.gsgpu_set_rk_error_sum(-1) == g.GRAV_VALUE_ERROR
    assert lib.gsgpu_set_rk_error_sum(1) == 0
    assert lib.gsgpu_set_rk_error_sum(0) == 0
