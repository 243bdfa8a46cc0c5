"""Barnes-Hut on the GPU against grav_sim.

* Octree (construct_octree): bounding-box width, Morton keys, sorted order,
  node numbering and topology, and internal-node mass / centre of mass are
  bit-exact to the reference (tolerance 0).
* Walk: GRAV_GPU_BARNES_HUT_COMPAT (113) reproduces the reference's walk,
  including its zero-mass leaves and its key indexing, and
  GRAV_GPU_BARNES_HUT (103) the corrected walk of the oracle.  Every
  opening decision equals the oracle's (the GPU's interaction counts are
  identical), and accelerations, made of FP32 terms, are held to:
  |a_i - a_ref,i| <= 1e-5 * A_i with A_i the sum of the magnitudes of
  particle i's terms, and per-particle relative error median <= 1e-6,
  99th percentile <= 1e-5.
"""
import ctypes

import numpy as np
import pytest

from conftest import cases, golden

pytestmark = pytest.mark.gpu

TREE_KEYS = ("keys", "sorted_indices", "num_particles", "num_children", "first_particle")


def gpu_octree(lib, g, x, m, leaf, method=3):
    system, keep = g.make_system(x, m, 1.0)
    t = g.LinearOctree()
    p = g.AccelerationParam(method, 1.0, 0.0, int(leaf))
    st = lib.construct_octree(ctypes.byref(t), ctypes.byref(system), ctypes.byref(p), None, -1.0)
    assert st.return_code == 0, g.take_traceback(lib, st)
    n, nn = system.num_particles, t.num_internal_nodes
    out = dict(
        box_width=t.box_width, num_nodes=nn,
        keys=np.ctypeslib.as_array(t.particle_morton_indices_deepest_level, (n,)).copy(),
        sorted_indices=np.ctypeslib.as_array(t.sorted_indices, (n,)).copy(),
        num_particles=np.ctypeslib.as_array(t.tree_num_particles, (nn,)).copy(),
        num_children=np.ctypeslib.as_array(t.tree_num_internal_children, (nn,)).copy(),
        first_particle=np.ctypeslib.as_array(t.tree_first_particle_sorted_idx, (nn,)).copy(),
        first_child=np.ctypeslib.as_array(t.tree_first_internal_children_idx, (nn,)).copy(),
        mass=np.ctypeslib.as_array(t.tree_mass, (nn,)).copy(),
        com=np.stack([np.ctypeslib.as_array(t.tree_center_of_mass_x, (nn,)).copy(),
                      np.ctypeslib.as_array(t.tree_center_of_mass_y, (nn,)).copy(),
                      np.ctypeslib.as_array(t.tree_center_of_mass_z, (nn,)).copy()], 1),
    )
    lib.free_linear_octree(ctypes.byref(t))
    del keep
    return out


def assert_same_tree(gt, ref, name=""):
    assert gt["num_nodes"] == len(ref["num_particles"]), name
    assert gt["box_width"] == float(ref["box_width"]), name
    for k in TREE_KEYS:
        assert np.array_equal(gt[k], ref[k]), (name, k)
    internal = ref["num_children"] > 0
    assert np.array_equal(gt["first_child"][internal], ref["first_child"][internal]), name
    assert np.array_equal(gt["mass"][internal], ref["mass"][internal]), name
    assert np.array_equal(gt["com"][internal], ref["com"][internal]), name


def test_octree_bitexact_golden(lib, g):
    for name, c in cases(golden("octree")).items():
        gt = gpu_octree(lib, g, c["x"], c["m"], int(c["leaf"]))
        assert_same_tree(gt, c, name)


@pytest.mark.parametrize("n,leaf", [(1, 1), (2, 1), (9, 2), (5000, 1), (5000, 3), (100000, 1),
                                    (100000, 16)])
def test_octree_bitexact_fresh(lib, g, orc, wl, n, leaf):
    x, v, m = wl.plummer(n, 1000 + n + leaf)
    gt = gpu_octree(lib, g, x, m, leaf)
    ref = orc.build_tree(x, m, leaf, True)
    assert_same_tree(gt, ref)
    # the corrected tree gives leaves their own mass and centre of mass
    gf = gpu_octree(lib, g, x, m, leaf, method=g.METHOD_GPU_BARNES_HUT)
    rf = orc.build_tree(x, m, leaf, False)
    assert np.array_equal(gf["mass"], rf["mass"]) and np.array_equal(gf["com"], rf["com"])


def test_octree_bitexact_galaxy_collision_2097152(lib, g, orc, wl):
    """Morton keys, order and tree of the galaxy-collision workload at full
    size, bit-exact."""
    x, v, m = wl.galaxy_pair(2097152, 4)
    gt = gpu_octree(lib, g, x, m, 1)
    ref = orc.build_tree(x, m, 1, True)
    assert_same_tree(gt, ref)


def check_terms(a, ref, absum):
    diff = np.linalg.norm(a - ref, axis=1)
    assert np.all(diff <= 1e-5 * absum + 1e-300), float(np.max(diff / (absum + 1e-300)))
    mag = np.linalg.norm(ref, axis=1)
    nz = mag > 0
    rel = diff[nz] / mag[nz]
    med, p99 = float(np.median(rel)), float(np.quantile(rel, 0.99))
    assert med <= 1e-6 and p99 <= 1e-5, (med, p99)
    return med, p99


def gpu_counts(lib):
    c = (ctypes.c_longlong * 2)()
    assert lib.gsgpu_last_interaction_counts(c) == 0
    return int(c[0]), int(c[1])


def test_compat_walk_golden(lib, g, orc):
    for name, c in cases(golden("barnes_hut")).items():
        leaf = int(c["leaf"])
        for th in (0.5, 1.0):
            a = g.acceleration(lib, c["x"], c["m"], 1.0, g.METHOD_GPU_BARNES_HUT_COMPAT,
                               opening_angle=th, softening_length=0.01,
                               max_num_particles_per_leaf=leaf)
            a_o, cnt, mag = orc.bh_counts(c["x"], c["m"], 1.0, 0.01, th, leaf, True)
            assert np.array_equal(a_o, c[f"a_theta{th}"])
            assert gpu_counts(lib) == (int(cnt[:, 0].sum()), int(cnt[:, 1].sum())), (name, th)
            check_terms(a, c[f"a_theta{th}"], mag)


@pytest.mark.parametrize("compat", [True, False])
@pytest.mark.parametrize("theta,leaf", [(0.5, 1), (1.0, 1), (0.7, 8)])
def test_walk_vs_oracle(lib, g, orc, wl, compat, theta, leaf):
    x, v, m = wl.galaxy_pair(65536, 11)
    method = g.METHOD_GPU_BARNES_HUT_COMPAT if compat else g.METHOD_GPU_BARNES_HUT
    a = g.acceleration(lib, x, m, 1.0, method, opening_angle=theta, softening_length=0.01,
                       max_num_particles_per_leaf=leaf)
    a_o, cnt, mag = orc.bh_counts(x, m, 1.0, 0.01, theta, leaf, compat)
    assert gpu_counts(lib) == (int(cnt[:, 0].sum()), int(cnt[:, 1].sum()))
    check_terms(a, a_o, mag)


def test_reference_entry_point_acceleration_barnes_hut(lib, g, orc, wl):
    """acceleration_barnes_hut() with the reference's method code 3 runs the
    reference-compatible GPU walk."""
    x, v, m = wl.plummer(3000, 3)
    system, keep = g.make_system(x, m, 1.0)
    a = np.empty((3000, 3))
    p = g.AccelerationParam(3, 0.5, 0.01, 1)
    lib.acceleration_barnes_hut.restype = g.ErrorStatus
    st = lib.acceleration_barnes_hut(a.ctypes.data_as(g.c_double_p), ctypes.byref(system),
                                     ctypes.byref(p))
    assert st.return_code == 0
    a_o, cnt, mag = orc.bh_counts(x, m, 1.0, 0.01, 0.5, 1, True)
    check_terms(a, a_o, mag)


@pytest.mark.parametrize("theta", [0.5, 1.0])
def test_quadrupole_walk_vs_oracle(lib, g, orc, wl, theta):
    """GRAV_GPU_BARNES_HUT_QUAD: same opening decisions as the corrected walk,
    cells add monopole + quadrupole terms; quadrupoles composed bottom-up on
    the GPU (parallel-axis shifts) against the oracle's direct per-node sums."""
    x, v, m = wl.galaxy_pair(32768, 12)
    a = g.acceleration(lib, x, m, 1.0, g.METHOD_GPU_BARNES_HUT_QUAD, opening_angle=theta,
                       softening_length=0.01, max_num_particles_per_leaf=1)
    a_o, mag, q = orc.bh_quad(x, m, 1.0, 0.01, theta, 1)
    _, cnt, _ = orc.bh_counts(x, m, 1.0, 0.01, theta, 1, False)
    assert gpu_counts(lib) == (int(cnt[:, 0].sum()), int(cnt[:, 1].sum()))
    check_terms(a, a_o, mag)


def test_fixed_walk_accuracy_vs_direct_sum(lib, g, orc, wl):
    """Corrected multipoles: theta=0.5 reaches ~1e-3 median error against the
    FP64 direct sum on the galaxy model (the reference's walk does not)."""
    x, v, m = wl.galaxy_pair(131072, 5)
    rows = np.random.default_rng(1).choice(x.shape[0], 2048, replace=False).astype(np.int32)
    exact = orc.direct_rows(x, m, 1.0, 0.01, rows)
    a = g.acceleration(lib, x, m, 1.0, g.METHOD_GPU_BARNES_HUT, opening_angle=0.5,
                       softening_length=0.01, max_num_particles_per_leaf=1)
    err = orc.rel_err(a[rows], exact)
    print(f"fixed theta=0.5 median {np.median(err):.3g} p99 {np.quantile(err, 0.99):.3g}")
    assert np.median(err) < 3e-3


@pytest.mark.parametrize("theta,leaf", [(0.5, 1), (0.8, 1), (0.5, 64)])
def test_group_walk_accuracy(lib, g, orc, wl, theta, leaf):
    """Group walk (106): its group opening criterion implies the per-particle
    one for every particle, so it is at least about as accurate as the
    per-particle quadrupole walk (105) at the same theta.  leaf=64 exercises
    leaves that overflow one list round."""
    x, v, m = wl.galaxy_pair(131072, 7)
    rows = np.random.default_rng(3).choice(x.shape[0], 2048, replace=False).astype(np.int32)
    exact = orc.direct_rows(x, m, 1.0, 0.01, rows)
    kw = dict(opening_angle=theta, softening_length=0.01, max_num_particles_per_leaf=leaf)
    a_g = g.acceleration(lib, x, m, 1.0, g.METHOD_GPU_BARNES_HUT_GROUP, **kw)
    cells, pairs = gpu_counts(lib)
    a_q = g.acceleration(lib, x, m, 1.0, g.METHOD_GPU_BARNES_HUT_QUAD, **kw)
    e_g = np.median(orc.rel_err(a_g[rows], exact))
    e_q = np.median(orc.rel_err(a_q[rows], exact))
    print(f"theta={theta} leaf={leaf}: group {e_g:.3g} ({cells} cells, {pairs} pairs), "
          f"per-particle quad {e_q:.3g}")
    assert np.isfinite(a_g).all()
    assert e_g <= 1.1 * e_q
    assert cells > 0 and pairs > 0


def test_group_walk_degenerate_and_unsoftened(lib, g, orc, wl):
    """A 200-particle coincident cluster (one depth-21 leaf with more
    particles than one list round) with softening, and an unsoftened
    Plummer sphere (the particle's own term is skipped)."""
    x, v, m = wl.plummer(20000, 11)
    x[100:300] = x[50]
    rows = np.arange(40, 340, dtype=np.int32)
    exact = orc.direct_rows(x, m, 1.0, 0.01, rows)
    a = g.acceleration(lib, x, m, 1.0, g.METHOD_GPU_BARNES_HUT_GROUP, opening_angle=0.6,
                       softening_length=0.01, max_num_particles_per_leaf=1)
    assert np.isfinite(a).all()
    assert np.median(orc.rel_err(a[rows], exact)) < 2e-3
    x2, v2, m2 = wl.plummer(20000, 12)
    rows2 = np.random.default_rng(4).choice(20000, 512, replace=False).astype(np.int32)
    exact2 = orc.direct_rows(x2, m2, 1.0, 0.0, rows2)
    a2 = g.acceleration(lib, x2, m2, 1.0, g.METHOD_GPU_BARNES_HUT_GROUP, opening_angle=0.5,
                        softening_length=0.0, max_num_particles_per_leaf=1)
    assert np.isfinite(a2).all()
    assert np.median(orc.rel_err(a2[rows2], exact2)) < 2e-3


@pytest.mark.parametrize("method", [3, 13, 5, 6])
def test_node_capacity_overflow(lib, g, orc, wl, method):
    """2,048 coincident pairs with one particle per leaf: each pair splits
    down to the depth limit, 36,951 nodes (the oracle's count) against a
    capacity of 4N + 4096 = 20,480.  The build stops at the capacity, the
    kernels after it do no work, and the call reports GRAV_MEMORY_ERROR;
    the same engine then serves a normal input."""
    rng = np.random.default_rng(6)
    x = np.repeat(rng.random((2048, 3)), 2, axis=0)
    m = np.full(4096, 1.0 / 4096)
    assert orc.build_tree(x, m, 1, False)["num_nodes"] > 4 * 4096 + 4096
    gpu = method + 100
    with pytest.raises(g.GravError) as e:
        g.acceleration(lib, x, m, 1.0, gpu, opening_angle=0.5, softening_length=0.01,
                       max_num_particles_per_leaf=1)
    assert e.value.code == g.GRAV_MEMORY_ERROR
    if method == 3:
        system, keep = g.make_system(x, m, 1.0)
        t = g.LinearOctree()
        p = g.AccelerationParam(3, 1.0, 0.0, 1)
        st = lib.construct_octree(ctypes.byref(t), ctypes.byref(system), ctypes.byref(p),
                                  None, -1.0)
        assert st.return_code == g.GRAV_MEMORY_ERROR
        g.take_traceback(lib, st)
    x2, _, m2 = wl.plummer(4096, 3)
    a = g.acceleration(lib, x2, m2, 1.0, gpu, opening_angle=0.5, softening_length=0.01,
                       max_num_particles_per_leaf=1)
    assert np.isfinite(a).all()
    if method in (3, 13):   # the oracle's walk, term for term
        a_o, cnt, mag = orc.bh_counts(x2, m2, 1.0, 0.01, 0.5, 1, method == 13)
        check_terms(a, a_o, mag)
    else:
        rows = np.arange(0, 4096, 16, dtype=np.int32)
        err = orc.rel_err(a[rows], orc.direct_rows(x2, m2, 1.0, 0.01, rows))
        assert np.median(err) < 5e-3


def test_group_walk_in_simulation(lib, g, wl):
    """The group walk drives launch_simulation (graph-captured leapfrog)."""
    x, v, m = wl.galaxy_pair(32768, 8)
    _, xo, vo, _ = g.launch_simulation(lib, x.copy(), v.copy(), m, 1.0, integrator=4, dt=1e-3,
                                       tf=0.01, method=g.METHOD_GPU_BARNES_HUT_GROUP,
                                       opening_angle=0.5, softening_length=0.01,
                                       max_num_particles_per_leaf=1)
    assert np.isfinite(xo).all() and np.isfinite(vo).all()
    assert np.abs(xo - x).max() < 0.1


def test_group_walk_galaxy_1m(lib, g, orc, wl):
    """The full-size galaxy model: dense centres stress the traversal stack
    (an overflow would be reported as an error), accuracy stays below the
    per-particle criterion's."""
    x, v, m = wl.galaxy_pair(1048576, 5)
    a = g.acceleration(lib, x, m, 1.0, g.METHOD_GPU_BARNES_HUT_GROUP, opening_angle=0.5,
                       softening_length=0.01, max_num_particles_per_leaf=1)
    rows = np.random.default_rng(5).choice(x.shape[0], 256, replace=False).astype(np.int32)
    err = orc.rel_err(a[rows], orc.direct_rows(x, m, 1.0, 0.01, rows))
    print(f"group walk N=1048576 theta=0.5: median {np.median(err):.3g}")
    assert np.isfinite(a).all() and np.median(err) < 1e-3


def test_group_walk_particles_on_box_maximum(lib, g, orc, wl):
    """Particles exactly on the bounding-box maximum get Morton coordinate 0
    (the reference's wrap) and sit in a cell on the far side: their group
    does not fit its cell and is walked particle by particle, with the same
    accuracy as everyone else."""
    x, v, m = wl.plummer(50000, 13)
    hi = x.max(axis=0)
    x[7] = hi
    x[8] = hi - 1e-9
    x[9, 0] = hi[0]
    rows = np.array([7, 8, 9, 10, 11], dtype=np.int32)
    a = g.acceleration(lib, x, m, 1.0, g.METHOD_GPU_BARNES_HUT_GROUP, opening_angle=0.5,
                       softening_length=0.01, max_num_particles_per_leaf=1)
    err = orc.rel_err(a[rows], orc.direct_rows(x, m, 1.0, 0.01, rows))
    assert np.isfinite(a).all() and err.max() < 5e-3


def test_group_walk_monopole_vs_per_particle(lib, g, orc, wl):
    """Monopole group walk (107): at least about as accurate as the
    per-particle monopole walk (103) at the same theta."""
    x, v, m = wl.galaxy_pair(131072, 9)
    rows = np.random.default_rng(6).choice(x.shape[0], 2048, replace=False).astype(np.int32)
    exact = orc.direct_rows(x, m, 1.0, 0.01, rows)
    kw = dict(opening_angle=0.5, softening_length=0.01, max_num_particles_per_leaf=1)
    e_g = np.median(orc.rel_err(g.acceleration(lib, x, m, 1.0, g.METHOD_GPU_BARNES_HUT_GROUP_MONO,
                                               **kw)[rows], exact))
    e_p = np.median(orc.rel_err(g.acceleration(lib, x, m, 1.0, g.METHOD_GPU_BARNES_HUT, **kw)[rows],
                                exact))
    print(f"monopole: group {e_g:.3g}, per-particle {e_p:.3g}")
    assert e_g <= 1.1 * e_p


def test_width_division_matches_ddiv(lib):
    """The Morton keys' division-free quotients by the box width equal
    __ddiv_rn bit for bit: 2^26 samples of widths in [2^-100, 2^100] and
    dividends of every class and next to rounding ties."""
    import ctypes
    lib.gsgpu_width_division_selftest.restype = ctypes.c_int
    lib.gsgpu_width_division_selftest.argtypes = [ctypes.c_longlong, ctypes.c_ulonglong,
                                                  ctypes.POINTER(ctypes.c_longlong)]
    bad = ctypes.c_longlong(-1)
    for seed in (1, 2):
        assert lib.gsgpu_width_division_selftest(1 << 26, seed, ctypes.byref(bad)) == 0
        assert bad.value == 0
