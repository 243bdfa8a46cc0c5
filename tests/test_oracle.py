"""The oracle (C restatement) against grav_sim's own outputs.

CPU only.  The golden vectors were produced by the reference library
compiled from its own sources (tests/golden/make_golden.py); where that
library is present on this machine the restatement is also compared with it
on fresh seeded inputs.  Everything here is bit-exact: the restatement
performs the reference's FP64 operations in the reference's order.
"""
import numpy as np
import pytest

from conftest import cases, golden
from oracle import reference


def test_pairwise_golden(orc):
    for name, c in cases(golden("pairwise")).items():
        a = orc.pairwise(c["x"], c["m"], float(c["G"]), float(c["eps"]))
        assert np.array_equal(a, c["a"]), name


def test_massless_golden(orc):
    for name, c in cases(golden("massless")).items():
        a = orc.massless(c["x"], c["m"], 1.0, 0.01)
        assert np.array_equal(a, c["a"]), name


TREE_KEYS = ("keys", "sorted_indices", "num_particles", "num_children", "first_particle",
             "first_child")


def test_octree_golden(orc):
    for name, c in cases(golden("octree")).items():
        t = orc.build_tree(c["x"], c["m"], int(c["leaf"]), True)
        assert t["box_width"] == float(c["box_width"]), name
        for k in TREE_KEYS:
            assert np.array_equal(t[k], c[k]), (name, k)
        internal = c["num_children"] > 0
        assert np.array_equal(t["mass"][internal], c["mass"][internal]), name
        assert np.array_equal(t["com"][internal], c["com"][internal]), name


def test_octree_quirks(orc):
    """Bounding-box maximum wraps to Morton coordinate 0; duplicates stop at
    level 21 as one leaf."""
    c = cases(golden("octree"))["edges_leaf1"]
    t = orc.build_tree(c["x"], c["m"], 1, True)
    center, width = orc.bbox(c["x"])
    keys = orc.morton(c["x"], center, width)
    k10 = int(keys[10])
    # along the axis of largest extent the maximum normalises to 1.0, i.e.
    # 2^21 after scaling, which the 21-bit mask wraps to 0
    w = int(np.argmax(c["x"].max(axis=0) - c["x"].min(axis=0)))
    assert k10 & (0x1249249249249249 << w) == 0
    assert k10 != 0
    deep = (t["depth"] == 21) & (t["num_children"] == 0)
    assert deep.any() and t["num_particles"][deep].max() >= 21


def test_barnes_hut_golden(orc):
    for name, c in cases(golden("barnes_hut")).items():
        for th in (0.5, 1.0):
            a = orc.barnes_hut(c["x"], c["m"], 1.0, 0.01, th, int(c["leaf"]), True)
            assert np.array_equal(a, c[f"a_theta{th}"]), (name, th)


def test_integrators_golden(orc):
    d = golden("integrators")
    for integ in (1, 2, 3, 4):
        xo, vo = orc.fixed_step_run(integ, 1, d["x"], d["v"], d["m"], 1.0, 0.01, 1e-3, 0.0995)
        assert np.array_equal(xo, d[f"int{integ}/x"]), integ
        assert np.array_equal(vo, d[f"int{integ}/v"]), integ


def test_leapfrog_plummer1024_golden(orc):
    d = golden("leapfrog_plummer1024")
    xo, vo = orc.fixed_step_run(4, 1, d["x0"], d["v0"], d["m"], 1.0, 0.01, 1e-3, 1.0)
    assert np.array_equal(xo, d["x"]) and np.array_equal(vo, d["v"])
    e1 = orc.energy(xo, vo, d["m"], 1.0)
    assert abs(e1 - float(d["e1"])) <= 1e-13 * abs(float(d["e1"]))


def test_whfast_golden(orc):
    """WHFast restatement against the reference's runs: massless, pairwise,
    softened, and a removal (hyperbolic escaper), bit for bit."""
    for name, c in cases(golden("whfast")).items():
        ids, x, v, m = orc.whfast_run(c["x0"], c["v0"], c["m0"], float(c["G"]), float(c["eps"]),
                                      float(c["dt"]), float(c["tf"]),
                                      pairwise=int(c["method"]) == 1)
        assert np.array_equal(ids, c["ids"]), name
        assert np.array_equal(x, c["x"]) and np.array_equal(v, c["v"]), name
        assert np.array_equal(m, c["m"]), name
    assert cases(golden("whfast"))["escape"]["ids"].size == cases(golden("whfast"))["escape"]["m0"].size - 1


def test_rk_embedded_golden(orc):
    """Embedded RK restatement against the reference's runs, bit for bit."""
    d = golden("rk_embedded")
    for integ in (5, 6, 7, 8):
        for tag in ("auto", "given"):
            c = f"int{integ}_{tag}"
            xo, vo, steps, t, dt = orc.rk_embedded_run(integ, 1, d["x"], d["v"], d["m"], 1.0, 0.01,
                                                       float(d[f"{c}/tol"]), 0.5,
                                                       float(d[f"{c}/initial_dt"]))
            assert t >= 0.5 and steps > 0, c
            assert np.array_equal(xo, d[f"{c}/x"]) and np.array_equal(vo, d[f"{c}/v"]), c
    xo, vo, *_ = orc.rk_embedded_run(6, 2, d["massless_x0"], d["massless_v0"], d["massless_m"],
                                     float(d["massless_G"]), 0.0, 1e-9, 200.0)
    assert np.array_equal(xo, d["massless_x"]) and np.array_equal(vo, d["massless_v"])


def test_ias15_golden(orc):
    """IAS15 restatement against the reference's runs, bit for bit."""
    d = golden("ias15")
    for tag in ("auto", "given"):
        xo, vo, steps, t, dt = orc.ias15_run(1, d["x"], d["v"], d["m"], 1.0, 0.01,
                                             float(d[f"{tag}/tol"]), 0.5,
                                             float(d[f"{tag}/initial_dt"]))
        assert t >= 0.5 and steps > 0, tag
        assert np.array_equal(xo, d[f"{tag}/x"]) and np.array_equal(vo, d[f"{tag}/v"]), tag
    xo, vo, *_ = orc.ias15_run(2, d["massless_x0"], d["massless_v0"], d["massless_m"],
                               float(d["massless_G"]), 0.0, 1e-9, 200.0)
    assert np.array_equal(xo, d["massless_x"]) and np.array_equal(vo, d["massless_v"])


def test_energy_golden(orc):
    d = golden("energy")
    e = orc.energy(d["x"], d["v"], d["m"], float(d["G"]))
    assert e == float(d["e"])


@pytest.mark.skipif(not reference.available(), reason="reference library not built here")
def test_restatement_vs_reference_fresh(orc, wl):
    rng = np.random.default_rng(1234)
    for trial in range(3):
        n = int(rng.integers(50, 2500))
        x, v, m = wl.plummer(n, 500 + trial)
        m = m * rng.uniform(0.5, 1.5, n)
        assert np.array_equal(orc.pairwise(x, m, 1.0, 0.02), reference.acceleration(x, m, 1.0, 1, eps=0.02))
        leaf = int(rng.integers(1, 9))
        tr = reference.octree(x, m, leaf)
        to = orc.build_tree(x, m, leaf, True)
        for k in TREE_KEYS:
            assert np.array_equal(tr[k], to[k]), (trial, k)
        th = float(rng.uniform(0.3, 1.2))
        assert np.array_equal(orc.barnes_hut(x, m, 1.0, 0.01, th, leaf, True),
                              reference.acceleration(x, m, 1.0, 3, theta=th, eps=0.01, leaf=leaf))


@pytest.mark.skipif(not reference.available(), reason="reference library not built here")
def test_restated_leapfrog_with_barnes_hut_vs_reference(orc, wl):
    """The restated integrator with method 3 (Barnes-Hut, the reference's
    quirks kept) against grav_sim's own launch_simulation with its Barnes-Hut:
    the same state after 20 leapfrog steps, bit for bit."""
    x, v, m = wl.galaxy_pair(1024, 17)
    xo, vo = orc.fixed_step_run(4, 3, x, v, m, 1.0, 0.01, 1e-3, 0.02, bh=(0.5, 4, 1))
    _, xr, vr, _ = reference.launch(x, v, m, 1.0, 4, 1e-3, 0.02, 3, theta=0.5, eps=0.01, leaf=4)
    assert np.array_equal(xo, xr) and np.array_equal(vo, vr)


def test_fixed_mode_tree_is_more_accurate(orc, wl):
    """With true leaf multipoles and own keys (fixed mode) the walk is far
    closer to the direct sum than the reference's walk (zero-mass leaves)."""
    x, v, m = wl.plummer(4000, 9)
    exact = orc.pairwise(x, m, 1.0, 0.01)
    e_ref = np.median(orc.rel_err(orc.barnes_hut(x, m, 1.0, 0.01, 0.5, 1, True), exact))
    e_fix = np.median(orc.rel_err(orc.barnes_hut(x, m, 1.0, 0.01, 0.5, 1, False), exact))
    assert e_fix < 5e-3 < e_ref


def test_octree_node_capacity_margin(orc, wl):
    """The GPU octree holds 4N + 4096 nodes.  The bench's distributions
    need about 1.5 N nodes with one particle per leaf and 0.43 N with eight.
    2,048 coincident pairs need about 9 N: each pair splits down to the depth
    limit.  The GPU answers that input with GRAV_MEMORY_ERROR
    (tests/test_gpu_barnes_hut.py::test_node_capacity_overflow)."""
    n = 65536
    for gen in (wl.plummer, wl.galaxy_pair):
        x, v, m = gen(n, 3)
        assert orc.build_tree(x, m, 1, False)["num_nodes"] < 1.6 * n
        assert orc.build_tree(x, m, 8, False)["num_nodes"] < 0.5 * n
    rng = np.random.default_rng(6)
    x = np.repeat(rng.random((2048, 3)), 2, axis=0)
    m = np.full(4096, 1.0 / 4096)
    nodes = orc.build_tree(x, m, 1, False)["num_nodes"]
    assert nodes > 4 * 4096 + 4096 and nodes > 8 * 4096
    # eight or more per leaf: a coincident pair stays in one leaf
    assert orc.build_tree(x, m, 8, False)["num_nodes"] < 4096


def _snapshot_rows(ids, m, x, v, fm, fx, fv):
    rows = []
    for i in range(len(m)):
        rows.append(f"{ids[i]}," + (fm % m[i]) + "," + ",".join(fx % q for q in x[i]) + ","
                    + ",".join(fv % q for q in v[i]))
    return rows


@pytest.mark.parametrize("name", ["leapfrog", "euler_float"])
def test_output_golden_rows_follow_oracle(orc, name):
    """The reference's snapshot files (output.npz) hold the oracle's state at
    each snapshot time -- t = steps * dt, and for leapfrog v synchronised to
    integer time -- printed as src/output.c:425-462 prints it ("%.17g", or
    "%.8g" for a float output dtype)."""
    import json
    c = cases(golden("output"))[name]
    args = json.loads(bytes(c["args.json"]).decode())
    o = args["output"]
    f = {1: "%.8g", 2: "%.17g"}
    fm = f[o.get("mass_output_dtype", 2)]
    fx = f[o.get("coordinate_output_dtype", 2)]
    fv = f[o.get("velocity_output_dtype", 2)]
    x0, v0, m0, G = c["x0"], c["v0"], c["m0"], float(c["G"])
    dt, eps = args["dt"], args["extra"]["eps"]
    files = sorted(k for k in c if k.startswith("snapshot_"))
    assert len(files) >= 3
    for k, fname in enumerate(files):
        lines = bytes(c[fname]).decode().split("\n")
        assert lines[0] == f"# num_particles: {m0.size}" and lines[1] == "# G: %.17g" % G
        assert lines[4] == "particle_id,m,x,y,z,vx,vy,vz" and lines[-1] == ""
        if k == 0 and o["output_initial"]:
            x, v = x0, v0
        else:
            t = float(lines[2].split(": ")[1])
            steps = round(t / dt)
            assert steps * dt == t and float(lines[3].split(": ")[1]) == dt
            x, v = orc.fixed_step_run(args["integrator"], 1, x0, v0, m0, G, eps, dt, steps * dt)
        assert lines[5:-1] == _snapshot_rows(np.arange(m0.size), m0, x, v, fm, fx, fv), fname


def test_dft_matches_numpy_fft(orc):
    """The oracle's direct DFT has FFTW's r2c / c2r semantics (checked
    against numpy's FFT, an independent implementation)."""
    rng = np.random.default_rng(3)
    for shape in [(4, 6, 8), (5, 3, 7), (8, 8, 8), (1, 1, 2)]:
        a = rng.standard_normal(shape)
        y = orc.dft3_r2c(a)
        scale = np.abs(a).sum()
        assert np.abs(y - np.fft.rfftn(a)).max() <= 1e-14 * scale
        back = orc.dft3_c2r(y, shape[2])
        assert np.abs(back - a * a.size).max() <= 1e-13 * scale * a.size


def test_pm_golden(orc):
    """acceleration_PM and the cosmological leapfrog: the restatement equals
    the reference (built from its sources with the same DFT standing in for
    FFTW) bit for bit."""
    import json
    d = golden("pm")
    c, bw = d["box_center"], float(d["box_width"])
    H0, om, sf = float(d["H0"]), float(d["omega_m"]), float(d["scale_factor"])
    for name, cs in cases(d).items():
        if name == "cosmo":
            continue
        rho = cs["m"].sum() / ((bw * 2) ** 3)
        a = orc.acceleration_pm(cs["x"], cs["m"], c, bw, H0, om, rho, int(cs["grid"]), sf)
        assert np.array_equal(a, cs["a"]), name
    cs = cases(d)["cosmo"]
    kw = json.loads(bytes(cs["args.json"]).decode())
    x, steps, t = orc.leapfrog_cosmology(cs["x0"], cs["v0"], cs["m"], kw["h"], kw["omega_m"],
                                         kw["omega_lambda"], np.array(kw["box_center"]),
                                         kw["box_width"], kw["dt"], kw["a_begin"], kw["a_final"],
                                         kw["pm_grid_size"])
    assert steps == int(cs["steps"]) and t == float(cs["t"])
    assert np.array_equal(x, cs["x"])


@pytest.mark.skipif(not reference._loadable(reference.PM), reason="reference not built here")
def test_pm_against_fresh_reference_run(orc):
    """A fresh case through the reference's own particle-mesh code."""
    rng = np.random.default_rng(77)
    c, bw = np.array([0.0, 1.0, -1.0]), 2.0
    x = c + rng.uniform(-bw, bw, (700, 3))
    m = rng.uniform(0.1, 1.0, 700)
    rho = m.sum() / ((bw * 2) ** 3)
    a_ref = reference.acceleration_pm(x, m, c, bw, 67.0, 0.31, rho, 12, 0.7)
    a = orc.acceleration_pm(x, m, c, bw, 67.0, 0.31, rho, 12, 0.7)
    assert np.array_equal(a, a_ref)
