"""Batched planetary ensembles on the GPU (WHFast and leapfrog + massless).

Every system of an ensemble must evolve bit for bit as the reference evolves
it alone: checked against the WHFast golden vectors (made by the reference
itself) and, for many uneven systems at once, against the oracle's
restatement system by system.
"""
import ctypes

import numpy as np
import pytest

from conftest import cases, golden

pytestmark = pytest.mark.gpu

GPU_MASSLESS = 102
GPU_PAIRWISE_FP64 = 111
WHFAST = 10
LEAPFROG = 4


def _concat(systems):
    counts = np.array([s[2].size for s in systems], dtype=np.int32)
    ids = np.concatenate([np.arange(s[2].size, dtype=np.int32) for s in systems])
    x = np.concatenate([s[0] for s in systems])
    v = np.concatenate([s[1] for s in systems])
    m = np.concatenate([s[2] for s in systems])
    return counts, ids, x, v, m


def _blocks(counts0, counts, *arrays):
    off = np.concatenate([[0], np.cumsum(counts0)])
    for s in range(counts0.size):
        yield tuple(a[off[s]:off[s] + counts[s]] for a in arrays)


def test_whfast_launch_simulation_golden(g, lib):
    """launch_simulation with integrator 10 reproduces the reference's WHFast
    runs (massless, pairwise, softened, removal of a hyperbolic escaper)."""
    for name, c in cases(golden("whfast")).items():
        method = GPU_PAIRWISE_FP64 if int(c["method"]) == 1 else GPU_MASSLESS
        x, v, m = c["x0"].copy(), c["v0"].copy(), c["m0"].copy()
        ids, xo, vo, mo = g.launch_simulation(
            lib, x, v, m, float(c["G"]), integrator=WHFAST, dt=float(c["dt"]), tf=float(c["tf"]),
            method=method, softening_length=float(c["eps"]))
        assert np.array_equal(ids, c["ids"]), name
        assert np.array_equal(xo, c["x"]), name
        assert np.array_equal(vo, c["v"]), name
        assert np.array_equal(mo, c["m"]), name


@pytest.mark.parametrize("pairwise", [False, True])
def test_whfast_ensemble_matches_oracle(g, lib, wl, orc, pairwise):
    G = wl.G_AU_MSUN_DAY
    systems = wl.planetary_ensemble(48, 2024 + int(pairwise), max_test=300)
    counts0, ids, x, v, m = _concat(systems)
    dt, tf = 8.0, 250.0
    ens = g.Ensemble(lib, counts0, G, integrator=WHFAST,
                     method=GPU_PAIRWISE_FP64 if pairwise else GPU_MASSLESS, dt=dt)
    ens.upload(ids, x, v, m)
    ens.run_until(tf)
    counts, ido, xo, vo, mo = ens.download()
    assert np.array_equal(counts, counts0)
    for s, (i_s, x_s, v_s, m_s) in enumerate(_blocks(counts0, counts, ido, xo, vo, mo)):
        xs, vs, ms = systems[s]
        ri, rx, rv, rm = orc.whfast_run(xs, vs, ms, G, 0.0, dt, tf, pairwise=pairwise)
        assert np.array_equal(i_s, ri), s
        assert np.array_equal(x_s, rx), s
        assert np.array_equal(v_s, rv), s
        assert np.array_equal(m_s, rm), s
    ens.close()


def test_whfast_ensemble_removal_per_system(g, lib, wl, orc):
    """Escapers in some systems only: those systems shrink, the others keep
    their counts, and every system still matches the oracle."""
    G = wl.G_AU_MSUN_DAY
    systems = []
    for s, (x, v, m) in enumerate(wl.planetary_ensemble(12, 77, max_test=40)):
        if s % 3 == 0:
            x = np.concatenate([x, [[1.0, 0.1 * s, 0.0]], [[-1.5, 0.3, 0.1]]])
            v = np.concatenate([v, [[100.0, 0.0, 0.0]], [[0.0, -80.0, 5.0]]])
            m = np.concatenate([m, [0.0, 0.0]])
        systems.append((np.ascontiguousarray(x), np.ascontiguousarray(v), m))
    counts0, ids, x, v, m = _concat(systems)
    ens = g.Ensemble(lib, counts0, G, integrator=WHFAST, method=GPU_MASSLESS, dt=10.0)
    ens.upload(ids, x, v, m)
    ens.run_until(120.0)
    counts, ido, xo, vo, mo = ens.download()
    for s, (i_s, x_s, v_s, m_s) in enumerate(_blocks(counts0, counts, ido, xo, vo, mo)):
        xs, vs, ms = systems[s]
        ri, rx, rv, rm = orc.whfast_run(xs, vs, ms, G, 0.0, 10.0, 120.0)
        assert counts[s] == ri.size, s
        if s % 3 == 0:
            assert ri.size == ms.size - 2
        assert np.array_equal(i_s, ri) and np.array_equal(x_s, rx), s
        assert np.array_equal(v_s, rv) and np.array_equal(m_s, rm), s
    ens.close()


def test_leapfrog_massless_ensemble_matches_oracle(g, lib, wl, orc):
    G = wl.G_AU_MSUN_DAY
    systems = wl.planetary_ensemble(32, 5, max_test=200)
    counts0, ids, x, v, m = _concat(systems)
    dt, tf = 2.0, 61.0
    ens = g.Ensemble(lib, counts0, G, integrator=LEAPFROG, method=GPU_MASSLESS, dt=dt)
    ens.upload(ids, x, v, m)
    ens.run_until(tf)
    counts, ido, xo, vo, mo = ens.download()
    assert np.array_equal(counts, counts0) and np.array_equal(ido, ids)
    for s, (x_s, v_s) in enumerate(_blocks(counts0, counts, xo, vo)):
        xs, vs, ms = systems[s]
        rx, rv = orc.fixed_step_run(4, 2, xs, vs, ms, G, 0.0, dt, tf)
        assert np.array_equal(x_s, rx), s
        assert np.array_equal(v_s, rv), s
    ens.close()


def test_ensemble_graph_replay_equals_run_until(g, lib, wl):
    """run(k) (graph replays of a fixed dt) and run_until(k dt) agree."""
    G = wl.G_AU_MSUN_DAY
    systems = wl.planetary_ensemble(16, 9, max_test=100)
    counts0, ids, x, v, m = _concat(systems)
    out = []
    for mode in ("run", "until"):
        ens = g.Ensemble(lib, counts0, G, integrator=WHFAST, method=GPU_MASSLESS, dt=5.0)
        ens.upload(ids, x, v, m)
        if mode == "run":
            ens.run(20)
        else:
            ens.run_until(100.0)
        out.append(ens.download())
        assert ens.kernels_per_step() == 8   # one sort class, drift, 3 Jacobi -> Cartesian, pairs, accel, kick
        assert all(t in (64, 128, 256, 512) for t in ens.tuning())
        ens.close()
    for a, b in zip(*out):
        assert np.array_equal(a, b)


def test_ensemble_rejects_bad_input(g, lib, wl):
    G = wl.G_AU_MSUN_DAY
    with pytest.raises(g.GravError):
        g.Ensemble(lib, [3, 4], G, integrator=3, method=GPU_MASSLESS, dt=1.0)
    with pytest.raises(g.GravError):
        g.Ensemble(lib, [3, 4], G, integrator=WHFAST, method=103, dt=1.0)
    with pytest.raises(g.GravError):
        g.Ensemble(lib, [3, 0], G, integrator=WHFAST, method=GPU_MASSLESS, dt=1.0)
    with pytest.raises(g.GravError):
        g.Ensemble(lib, [20000], G, integrator=WHFAST, method=GPU_MASSLESS, dt=1.0)
    # a system without the primary's id 0 is reported, not integrated
    systems = wl.planetary_ensemble(2, 3, max_test=5)
    counts0, ids, x, v, m = _concat(systems)
    ids = ids.copy()
    ids[counts0[0]] = 99
    ens = g.Ensemble(lib, counts0, G, integrator=WHFAST, method=GPU_MASSLESS, dt=1.0)
    ens.upload(ids, x, v, m)
    ens.run(2)
    with pytest.raises(g.GravError):
        ens.download()
    ens.close()


@pytest.mark.parametrize("negzero", [False, True])
def test_whfast_planar_systems_match_oracle(g, lib, wl, orc, negzero):
    """Planar systems (z = 0): the interior centres of mass have +0 (or, with
    -0.0 coordinates, -0) components, the case where the massless-run
    shortcuts must keep the reference's zero signs."""
    G = wl.G_AU_MSUN_DAY
    systems = []
    for x, v, m in wl.planetary_ensemble(10, 31, max_test=120):
        x, v = x.copy(), v.copy()
        x[:, 2] = 0.0
        v[:, 2] = 0.0
        if negzero:
            x[::2, 2] = -0.0
            v[1::3, 2] = -0.0
        systems.append((x, v, m))
    counts0, ids, x, v, m = _concat(systems)
    ens = g.Ensemble(lib, counts0, G, integrator=WHFAST, method=GPU_MASSLESS, dt=6.0)
    ens.upload(ids, x, v, m)
    ens.run_until(90.0)
    counts, ido, xo, vo, mo = ens.download()
    for s, (i_s, x_s, v_s) in enumerate(_blocks(counts0, counts, ido, xo, vo)):
        xs, vs, ms = systems[s]
        ri, rx, rv, rm = orc.whfast_run(xs, vs, ms, G, 0.0, 6.0, 90.0)
        assert np.array_equal(i_s, ri), s
        assert x_s.tobytes() == rx.tobytes() and v_s.tobytes() == rv.tobytes(), s
    ens.close()


def test_stumpff_division_matches_ddiv(lib):
    """The drift's division-free quotients by the Stumpff series' constants
    equal __ddiv_rn bit for bit: 2^26 samples over every exponent class and
    next to rounding ties."""
    lib.gsgpu_stumpff_division_selftest.restype = ctypes.c_int
    lib.gsgpu_stumpff_division_selftest.argtypes = [ctypes.c_longlong, ctypes.c_ulonglong,
                                                    ctypes.POINTER(ctypes.c_longlong)]
    bad = ctypes.c_longlong(-1)
    for seed in (1, 2):
        assert lib.gsgpu_stumpff_division_selftest(1 << 26, seed, ctypes.byref(bad)) == 0
        assert bad.value == 0


@pytest.mark.parametrize("pairwise", [False, True])
def test_whfast_many_massive_bodies_match_oracle(g, lib, wl, orc, pairwise):
    """Systems of 70 to 200 bodies that all have mass (the test particles of
    the planetary model given masses of 1e-12 to 1e-10 Msun): the Jacobi ->
    Cartesian recurrence has more than 64 massive slots, so it runs as one
    whole chain per system (k_wh_seq_chain's general path), and eta after
    each sort adds every slot.  Bit for bit against the oracle."""
    G = wl.G_AU_MSUN_DAY
    rng = np.random.default_rng(99 + int(pairwise))
    systems = []
    for x, v, m in wl.planetary_ensemble(60, 515 + int(pairwise), max_test=300):
        if m.size < 70:
            continue
        m = m.copy()
        m[9:] = 10.0 ** rng.uniform(-12, -10, m.size - 9)
        systems.append((x[:200], v[:200], m[:200]))
        if len(systems) == 8:
            break
    assert len(systems) >= 4
    counts0, ids, x, v, m = _concat(systems)
    dt, tf = 6.0, 120.0
    ens = g.Ensemble(lib, counts0, G, integrator=WHFAST,
                     method=GPU_PAIRWISE_FP64 if pairwise else GPU_MASSLESS, dt=dt)
    ens.upload(ids, x, v, m)
    ens.run_until(tf)
    counts, ido, xo, vo, mo = ens.download()
    assert np.array_equal(counts, counts0)
    for s, (i_s, x_s, v_s, m_s) in enumerate(_blocks(counts0, counts, ido, xo, vo, mo)):
        xs, vs, ms = systems[s]
        ri, rx, rv, rm = orc.whfast_run(xs, vs, ms, G, 0.0, dt, tf, pairwise=pairwise)
        assert np.array_equal(i_s, ri), s
        assert np.array_equal(x_s, rx) and np.array_equal(v_s, rv), s
    ens.close()
