"""benchmark_acceleration and the helpers grav_sim's benchmark example links
against (src/acceleration.c:369-506, src/system.c:38-66, src/utils.c:20-82).

CPU: the PCG32 generator behind init_pcg_rng / grav_randrange against a
restatement of the published algorithm (O'Neill 2014) and, where the
reference was built here, against grav_sim's own grav_randrange from the
same generator state; get_initialized_system's arrays and ids; the WRAP_*
helpers (raise_error, traceback) keep a success untouched and prepend frames
to a failure.
GPU: benchmark_acceleration over two GPU methods prints the reference's
report (one block per parameter set, mean and spread of the run times, MAE
of the first call against set 0) and returns success; a CPU method code is
rejected with the library's GRAV_VALUE_ERROR.
"""
import ctypes

import numpy as np
import pytest


class Pcg32(ctypes.Structure):
    _fields_ = [("state", ctypes.c_uint64), ("inc", ctypes.c_uint64)]


M64 = (1 << 64) - 1


def pcg32_step(state, inc):
    """One PCG32 draw: (output, new state)."""
    old = state
    state = (old * 6364136223846793005 + inc) & M64
    xorshifted = (((old >> 18) ^ old) >> 27) & 0xFFFFFFFF
    rot = old >> 59
    out = ((xorshifted >> rot) | (xorshifted << ((-rot) & 31))) & 0xFFFFFFFF
    return out, state


def pcg32_seeded(initstate, initseq):
    inc = ((initseq << 1) | 1) & M64
    _, state = pcg32_step(0, inc)
    state = (state + initstate) & M64
    _, state = pcg32_step(state, inc)
    return state, inc


def _bind(lib):
    lib.grav_randrange.restype = ctypes.c_double
    lib.grav_randrange.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.POINTER(Pcg32)]
    lib.init_pcg_rng.restype = Pcg32
    lib.grav_get_current_time.restype = ctypes.c_double


def test_randrange_is_pcg32(lib):
    _bind(lib)
    state, inc = pcg32_seeded(42, 54)
    rng = Pcg32(state, inc)
    for _ in range(64):
        out, state = pcg32_step(state, inc)
        want = -1.0 + 2.0 * (out / 2.0 ** 32)
        assert lib.grav_randrange(-1.0, 1.0, ctypes.byref(rng)) == want
        assert rng.state == state and rng.inc == inc
    # a clock-seeded generator draws inside [min, max)
    r = lib.init_pcg_rng()
    draws = [lib.grav_randrange(2.0, 3.0, ctypes.byref(r)) for _ in range(1000)]
    assert min(draws) >= 2.0 and max(draws) < 3.0
    t0 = lib.grav_get_current_time()
    assert lib.grav_get_current_time() >= t0


def test_randrange_matches_reference_build(lib):
    from oracle import reference
    if not reference.available():
        pytest.skip("grav_sim was not built from its sources on this machine")
    ref = ctypes.CDLL(str(reference.SERIAL))
    _bind(lib)
    ref.grav_randrange.restype = ctypes.c_double
    ref.grav_randrange.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.POINTER(Pcg32)]
    state, inc = pcg32_seeded(20261204, 7)
    a, b = Pcg32(state, inc), Pcg32(state, inc)
    for _ in range(256):
        assert lib.grav_randrange(-1.0, 1.0, ctypes.byref(a)) == \
            ref.grav_randrange(-1.0, 1.0, ctypes.byref(b))


def test_initialized_system_and_error_helpers(lib, g):
    lib.get_initialized_system.restype = g.ErrorStatus
    lib.get_initialized_system.argtypes = [ctypes.POINTER(g.System), ctypes.c_int]
    lib.free_system.argtypes = [ctypes.POINTER(g.System)]
    lib.free_system.restype = None
    s = g.System()
    st = lib.get_initialized_system(ctypes.byref(s), 17)
    assert st.return_code == g.GRAV_SUCCESS
    assert s.num_particles == 17 and s.G == 0.000295912208284119496676630
    assert [s.particle_ids[i] for i in range(17)] == list(range(17))
    assert all(s.x[i] == 0.0 for i in range(51)) and all(s.m[i] == 0.0 for i in range(17))
    lib.free_system(ctypes.byref(s))
    st = lib.get_initialized_system(None, 3)
    assert st.return_code == g.GRAV_POINTER_ERROR
    lib.free_traceback.argtypes = [ctypes.POINTER(g.ErrorStatus)]
    lib.free_traceback(ctypes.byref(st))

    lib.raise_error.restype = g.ErrorStatus
    lib.raise_error.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_char_p, ctypes.c_int,
                                ctypes.c_char_p]
    lib.traceback.restype = g.ErrorStatus
    lib.traceback.argtypes = [g.ErrorStatus, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int,
                              ctypes.c_char_p]
    e = lib.raise_error(b"a.c", 10, b"f", g.GRAV_VALUE_ERROR, b"bad value")
    assert e.return_code == g.GRAV_VALUE_ERROR
    e = lib.traceback(e, b"f(x)", b"b.c", 20, b"main")
    text = ctypes.string_at(e.traceback).decode()
    assert text.index("b.c") < text.index("a.c") and "bad value" in text
    lib.free_traceback(ctypes.byref(e))
    lib.make_success_error_status.restype = g.ErrorStatus
    okst = lib.make_success_error_status()
    assert lib.traceback(okst, b"g()", b"c.c", 1, b"h").return_code == g.GRAV_SUCCESS


@pytest.mark.gpu
def test_benchmark_acceleration_report(lib, g, wl, capfd):
    lib.benchmark_acceleration.restype = g.ErrorStatus
    lib.benchmark_acceleration.argtypes = [ctypes.POINTER(g.System),
                                           ctypes.POINTER(g.AccelerationParam), ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_int)]
    n = 20000
    x, v, m = wl.plummer(n, 99)
    ids = np.arange(n, dtype=np.int32)
    s = g.System(n, ids.ctypes.data_as(g.c_int_p), x.ctypes.data_as(g.c_double_p),
                 v.ctypes.data_as(g.c_double_p), m.ctypes.data_as(g.c_double_p), 1.0)
    params = (g.AccelerationParam * 3)(
        g.AccelerationParam(g.METHOD_GPU_PAIRWISE_FP64, 1.0, 0.01, -1),
        g.AccelerationParam(g.METHOD_GPU_PAIRWISE, 1.0, 0.01, -1),
        g.AccelerationParam(g.METHOD_GPU_BARNES_HUT_GROUP, 0.5, 0.01, 8))
    times = (ctypes.c_int * 3)(1, 3, 0)
    capfd.readouterr()
    st = lib.benchmark_acceleration(ctypes.byref(s), params, 3, times)
    out = capfd.readouterr().out
    assert st.return_code == g.GRAV_SUCCESS, out
    assert out.startswith("Benchmarking acceleration...\n")
    assert "Test 0:    Method: Pairwise (GPU, FP64 reference order)" in out
    assert "Test 1:    Method: Pairwise (GPU, compensated FP32)" in out
    assert "Test 2:    Skipped since num_times: 0 <= 0" in out
    assert out.count("Number of times: ") == 2
    mae = [float(ln.split(":")[1]) for ln in out.splitlines() if ln.strip().startswith("MAE:")]
    assert mae[0] == 0.0
    # the compensated FP32 sum agrees with the FP64 one to ~1e-6 of |a|
    a_scale = np.abs(g.acceleration(lib, x, m, 1.0, g.METHOD_GPU_PAIRWISE_FP64,
                                    softening_length=0.01)).sum(axis=1).mean()
    assert 0.0 < mae[1] < 1e-5 * a_scale
    # a CPU method code: acceleration()'s error comes back with a traceback
    bad = (g.AccelerationParam * 1)(g.AccelerationParam(1, 1.0, 0.0, -1))
    one = (ctypes.c_int * 1)(1)
    st = lib.benchmark_acceleration(ctypes.byref(s), bad, 1, one)
    assert st.return_code == g.GRAV_VALUE_ERROR
    lib.free_traceback.argtypes = [ctypes.POINTER(g.ErrorStatus)]
    lib.free_traceback(ctypes.byref(st))


def test_reference_benchmark_program_links_and_runs(tmp_path, lib):
    """grav_sim's own examples/benchmark/c/benchmark.c, compiled against the
    reference's headers, links this library and runs: its first set is
    skipped (0 runs) and its second, the CPU Barnes-Hut code 3, is rejected
    with the library's traceback (the program exits 1)."""
    import subprocess
    from oracle.reference import REF_DIR
    src = REF_DIR / "examples" / "benchmark" / "c" / "benchmark.c"
    if not src.exists():
        pytest.skip("grav_sim's sources are not present")
    libdir = str(__import__("pathlib").Path(lib._name).parent)
    exe = tmp_path / "benchmark"
    subprocess.run(["gcc", "-O2", "-std=gnu99", f"-I{REF_DIR / 'src'}", f"-I{REF_DIR / 'pcg'}",
                    str(src), f"-L{libdir}", "-lgrav_sim_gb300", f"-Wl,-rpath,{libdir}", "-lm",
                    "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 1
    assert r.stdout.startswith("Benchmarking acceleration...\n")
    assert "Test 0:    Skipped since num_times: 0 <= 0" in r.stdout
    assert "Unknown acceleration method. Got: 3" in r.stderr
    assert "benchmark_acceleration" in r.stderr
