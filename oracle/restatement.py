"""ctypes wrapper of the C restatement (oracle/grav_oracle.c).

TEST INFRASTRUCTURE ONLY.  ``load()`` builds liboracle.so with the Makefile
beside this file when it is missing (gcc, a second or two).
"""
from __future__ import annotations

import ctypes
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
LIB_OMP = HERE / "_build" / "liboracle_omp.so"

dp = ctypes.POINTER(ctypes.c_double)
ip = ctypes.POINTER(ctypes.c_int32)
lp = ctypes.POINTER(ctypes.c_int64)

_lib = None
_omp = None


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


class OrcTree(ctypes.Structure):
    _fields_ = [
        ("box_width", ctypes.c_double),
        ("center", ctypes.c_double * 3),
        ("num_nodes", ctypes.c_int),
        ("capacity", ctypes.c_int),
        ("keys", lp),
        ("sorted_indices", ip),
        ("num_particles", ip),
        ("num_children", ip),
        ("first_particle", ip),
        ("first_child", ip),
        ("depth", ip),
        ("mass", dp),
        ("com", dp),
    ]


def load():
    global _lib
    if _lib is not None:
        return _lib
    srcs = [HERE / f for f in ("grav_oracle.c", "grav_oracle.h", "pm_oracle.c", "pm_dft.c")]
    if not LIB.exists() or LIB.stat().st_mtime < max(f.stat().st_mtime for f in srcs):
        build()
    lib = ctypes.CDLL(str(LIB))
    lib.orc_pairwise.argtypes = [ctypes.c_int, dp, dp, ctypes.c_double, ctypes.c_double, dp]
    lib.orc_pairwise_slice.argtypes = [ctypes.c_int, dp, dp, ctypes.c_double, ctypes.c_double,
                                       ctypes.c_int, ctypes.c_int, dp]
    lib.orc_pairwise_slice.restype = ctypes.c_int64
    lib.orc_massless.argtypes = [ctypes.c_int, dp, dp, ctypes.c_double, ctypes.c_double, dp]
    lib.orc_bbox.argtypes = [ctypes.c_int, dp, dp, dp]
    lib.orc_morton.argtypes = [ctypes.c_int, dp, dp, ctypes.c_double, lp]
    lib.orc_radix_sort.argtypes = [ctypes.c_int, lp, ip]
    lib.orc_build_tree.argtypes = [ctypes.c_int, dp, dp, ctypes.c_int, ctypes.c_int,
                                   ctypes.POINTER(OrcTree)]
    lib.orc_free_tree.argtypes = [ctypes.POINTER(OrcTree)]
    lib.orc_bh_walk.argtypes = [ctypes.c_int, dp, dp, ctypes.c_double, ctypes.c_double,
                                ctypes.c_double, ctypes.POINTER(OrcTree), ctypes.c_int,
                                dp, lp, dp]
    lib.orc_barnes_hut.argtypes = [ctypes.c_int, dp, dp, ctypes.c_double, ctypes.c_double,
                                   ctypes.c_double, ctypes.c_int, ctypes.c_int, dp]
    lib.orc_fixed_step_run.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp, dp,
                                       ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                       ctypes.c_double]
    lib.orc_energy.argtypes = [ctypes.c_int, dp, dp, dp, ctypes.c_double]
    lib.orc_energy.restype = ctypes.c_double
    lib.orc_linear_momentum.argtypes = [ctypes.c_int, dp, dp]
    lib.orc_linear_momentum.restype = ctypes.c_double
    lib.orc_angular_momentum.argtypes = [ctypes.c_int, dp, dp, dp]
    lib.orc_angular_momentum.restype = ctypes.c_double
    lib.orc_direct_rows.argtypes = [ctypes.c_int, dp, dp, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_int, ip, dp]
    lib.orc_abs_sum_rows.argtypes = [ctypes.c_int, dp, dp, ctypes.c_double, ctypes.c_double,
                                     ctypes.c_int, ip, dp]
    _lib = lib
    return lib


def _d(a):
    return a.ctypes.data_as(dp)


def _c(a, dt=np.float64):
    return np.ascontiguousarray(a, dtype=dt)


def pairwise(x, m, G, eps):
    x, m = _c(x), _c(m)
    a = np.empty((m.size, 3))
    load().orc_pairwise(m.size, _d(x), _d(m), G, eps, _d(a))
    return a


def pairwise_slice(x, m, G, eps, i_begin, i_end):
    """Run the reference's symmetric loop for outer rows [i_begin, i_end);
    returns (a, pair evaluations)."""
    x, m = _c(x), _c(m)
    a = np.empty((m.size, 3))
    pairs = load().orc_pairwise_slice(m.size, _d(x), _d(m), G, eps, i_begin, i_end, _d(a))
    return a, int(pairs)


def massless(x, m, G, eps):
    x, m = _c(x), _c(m)
    a = np.empty((m.size, 3))
    rc = load().orc_massless(m.size, _d(x), _d(m), G, eps, _d(a))
    assert rc == 0
    return a


def bbox(x):
    x = _c(x)
    c = np.empty(3)
    w = ctypes.c_double()
    load().orc_bbox(x.shape[0], _d(x), _d(c), ctypes.byref(w))
    return c, w.value


def morton(x, center, width):
    x = _c(x)
    k = np.empty(x.shape[0], dtype=np.int64)
    load().orc_morton(x.shape[0], _d(x), _d(_c(center)), width, k.ctypes.data_as(lp))
    return k


def radix_sort(keys):
    k = _c(keys, np.int64).copy()
    idx = np.arange(k.size, dtype=np.int32)
    load().orc_radix_sort(k.size, k.ctypes.data_as(lp), idx.ctypes.data_as(ip))
    return k, idx


def build_tree(x, m, leaf_max, compat):
    """Return a dict of numpy copies of the oracle's node arrays."""
    x, m = _c(x), _c(m)
    t = OrcTree()
    rc = load().orc_build_tree(m.size, _d(x), _d(m), leaf_max, int(compat), ctypes.byref(t))
    assert rc == 0, rc
    nn, n = t.num_nodes, m.size
    out = dict(
        box_width=t.box_width, center=np.array(t.center[:]), num_nodes=nn,
        keys=np.ctypeslib.as_array(t.keys, (n,)).copy(),
        sorted_indices=np.ctypeslib.as_array(t.sorted_indices, (n,)).copy(),
        num_particles=np.ctypeslib.as_array(t.num_particles, (nn,)).copy(),
        num_children=np.ctypeslib.as_array(t.num_children, (nn,)).copy(),
        first_particle=np.ctypeslib.as_array(t.first_particle, (nn,)).copy(),
        first_child=np.ctypeslib.as_array(t.first_child, (nn,)).copy(),
        depth=np.ctypeslib.as_array(t.depth, (nn,)).copy(),
        mass=np.ctypeslib.as_array(t.mass, (nn,)).copy(),
        com=np.ctypeslib.as_array(t.com, (nn * 3,)).copy().reshape(nn, 3),
    )
    load().orc_free_tree(ctypes.byref(t))
    return out


def barnes_hut(x, m, G, eps, theta, leaf_max, compat):
    x, m = _c(x), _c(m)
    a = np.empty((m.size, 3))
    rc = load().orc_barnes_hut(m.size, _d(x), _d(m), G, eps, theta, leaf_max, int(compat), _d(a))
    assert rc == 0
    return a


def bh_counts(x, m, G, eps, theta, leaf_max, compat):
    """Walk with diagnostics: (a, per-particle [accepted cells, leaf pair
    terms], per-particle sum of term magnitudes)."""
    x, m = _c(x), _c(m)
    t = OrcTree()
    lib = load()
    assert lib.orc_build_tree(m.size, _d(x), _d(m), leaf_max, int(compat), ctypes.byref(t)) == 0
    a = np.empty((m.size, 3))
    cnt = np.empty((m.size, 2), dtype=np.int64)
    mag = np.empty(m.size)
    lib.orc_bh_walk(m.size, _d(x), _d(m), G, eps, theta, ctypes.byref(t), int(compat),
                    _d(a), cnt.ctypes.data_as(lp), _d(mag))
    lib.orc_free_tree(ctypes.byref(t))
    return a, cnt, mag


def bh_quad(x, m, G, eps, theta, leaf_max):
    """Corrected walk with quadrupole cell terms: (a, per-particle magnitude
    sum, node quadrupoles [nodes, 6])."""
    x, m = _c(x), _c(m)
    lib = load()
    lib.orc_quadrupoles.argtypes = [ctypes.POINTER(OrcTree), dp, dp, dp]
    lib.orc_bh_walk_quad.argtypes = [ctypes.c_int, dp, dp, ctypes.c_double, ctypes.c_double,
                                     ctypes.c_double, ctypes.POINTER(OrcTree), dp, dp, dp]
    t = OrcTree()
    assert lib.orc_build_tree(m.size, _d(x), _d(m), leaf_max, 0, ctypes.byref(t)) == 0
    q = np.empty((t.num_nodes, 6))
    lib.orc_quadrupoles(ctypes.byref(t), _d(x), _d(m), _d(q))
    a = np.empty((m.size, 3))
    mag = np.empty(m.size)
    lib.orc_bh_walk_quad(m.size, _d(x), _d(m), G, eps, theta, ctypes.byref(t), _d(q), _d(a),
                         _d(mag))
    lib.orc_free_tree(ctypes.byref(t))
    return a, mag, q


def fixed_step_run(integrator, method, x, v, m, G, eps, dt, tf, bh=None):
    """Fixed-step integrators 1-4 of src/integrator.c with acceleration method
    1 (pairwise), 2 (massless) or 3 (Barnes-Hut; bh = (theta, leaf_max,
    compat)); returns (x, v)."""
    x, v, m = _c(x).copy(), _c(v).copy(), _c(m)
    lib = load()
    if bh is not None:
        lib.orc_set_bh_params.argtypes = [ctypes.c_double, ctypes.c_int, ctypes.c_int]
        lib.orc_set_bh_params(float(bh[0]), int(bh[1]), int(bh[2]))
    rc = lib.orc_fixed_step_run(integrator, method, m.size, _d(x), _d(v), _d(m),
                                G, eps, dt, tf)
    assert rc == 0, rc
    return x, v


def rk_embedded_run(integrator, method, x, v, m, G, eps, tolerance, tf, initial_dt=-1.0):
    """Embedded RK (integrators 5-8) for one system; returns (x, v, steps, t, dt)."""
    lib = load()
    lib.orc_rk_embedded_run.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp, dp,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_double,
                                        ctypes.POINTER(ctypes.c_int64),
                                        ctypes.POINTER(ctypes.c_double),
                                        ctypes.POINTER(ctypes.c_double)]
    x, v, m = _c(x).copy(), _c(v).copy(), _c(m)
    steps, t, dt = ctypes.c_int64(), ctypes.c_double(), ctypes.c_double()
    rc = lib.orc_rk_embedded_run(integrator, method, m.size, _d(x), _d(v), _d(m), G, eps,
                                 tolerance, initial_dt, tf, ctypes.byref(steps), ctypes.byref(t),
                                 ctypes.byref(dt))
    assert rc == 0, rc
    return x.reshape(-1, 3), v.reshape(-1, 3), steps.value, t.value, dt.value


def ias15_run(method, x, v, m, G, eps, tolerance, tf, initial_dt=-1.0):
    """IAS15 (integrator 9) for one system; returns (x, v, steps, t, dt)."""
    lib = load()
    lib.orc_ias15_run.argtypes = [ctypes.c_int, ctypes.c_int, dp, dp, dp, ctypes.c_double,
                                  ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                  ctypes.c_double, ctypes.POINTER(ctypes.c_int64),
                                  ctypes.POINTER(ctypes.c_double),
                                  ctypes.POINTER(ctypes.c_double)]
    x, v, m = _c(x).copy(), _c(v).copy(), _c(m)
    steps, t, dt = ctypes.c_int64(), ctypes.c_double(), ctypes.c_double()
    rc = lib.orc_ias15_run(method, m.size, _d(x), _d(v), _d(m), G, eps, tolerance, initial_dt, tf,
                           ctypes.byref(steps), ctypes.byref(t), ctypes.byref(dt))
    assert rc == 0, rc
    return x.reshape(-1, 3), v.reshape(-1, 3), steps.value, t.value, dt.value


def whfast_run(x, v, m, G, eps, dt, tf, remove_invalid=True, pairwise=False, ids=None):
    """WHFast for one system; returns (ids, x, v, m) of the survivors."""
    lib = load()
    lib.orc_whfast_run.argtypes = [ctypes.POINTER(ctypes.c_int), ip, dp, dp, dp, ctypes.c_double,
                                   ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                   ctypes.c_int, ctypes.c_int]
    x, v, m = _c(x).copy(), _c(v).copy(), _c(m).copy()
    ids = np.arange(m.size, dtype=np.int32) if ids is None else _c(ids, np.int32).copy()
    n = ctypes.c_int(m.size)
    rc = lib.orc_whfast_run(ctypes.byref(n), ids.ctypes.data_as(ip), _d(x), _d(v), _d(m), G, eps,
                            dt, tf, int(remove_invalid), int(pairwise))
    assert rc == 0, rc
    k = n.value
    return ids[:k], x.reshape(-1, 3)[:k], v.reshape(-1, 3)[:k], m[:k]


def dft3_r2c(a):
    """FFTW-style r2c of a real (n0, n1, n2) array: complex (n0, n1, n2//2+1)."""
    a = _c(a)
    n0, n1, n2 = a.shape
    out = np.empty((n0, n1, n2 // 2 + 1, 2))
    lib = load()
    lib.orc_dft3_r2c.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp]
    lib.orc_dft3_r2c(n0, n1, n2, _d(a), _d(out))
    return out[..., 0] + 1j * out[..., 1]


def dft3_c2r(y, n2):
    """FFTW-style unnormalised c2r of a half spectrum (n0, n1, n2//2+1)."""
    n0, n1, h = y.shape
    assert h == n2 // 2 + 1
    yy = _c(np.stack([y.real, y.imag], axis=-1))
    out = np.empty((n0, n1, n2))
    lib = load()
    lib.orc_dft3_c2r.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp]
    lib.orc_dft3_c2r(n0, n1, n2, _d(yy), _d(out))
    return out


def acceleration_pm(x, m, box_center, box_width, H0, omega_m, mean_bkg_density, grid,
                    scale_factor):
    """src/acceleration_PM.c:274-391 with the direct DFT."""
    lib = load()
    lib.orc_acceleration_pm.argtypes = [dp, ctypes.c_int, dp, dp, dp, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_int, ctypes.c_double]
    x, m, c = _c(x), _c(m), _c(box_center)
    a = np.empty((m.size, 3))
    lib.orc_acceleration_pm(_d(a), m.size, _d(x), _d(m), _d(c), box_width, H0, omega_m,
                            mean_bkg_density, grid, scale_factor)
    return a


def leapfrog_cosmology(x, v, m, h, omega_m, omega_lambda, box_center, box_width, dt, a_begin,
                       a_final, grid, velocities=False):
    """src/integrator_cosmology_leapfrog.c with output disabled; returns
    (x, steps, t): v is left unchanged, as by the reference.  With
    velocities=True also the velocities a snapshot after the last step
    holds (momentum / a^2): (x, steps, t, v_last)."""
    lib = load()
    lib.orc_leapfrog_cosmology.argtypes = [ctypes.c_int, dp, dp, dp, ctypes.c_double,
                                           ctypes.c_double, ctypes.c_double, dp, ctypes.c_double,
                                           ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                           ctypes.c_int, ctypes.POINTER(ctypes.c_int64),
                                           ctypes.POINTER(ctypes.c_double), dp]
    x, v, m, c = _c(x).copy(), _c(v), _c(m), _c(box_center)
    steps, t = ctypes.c_int64(), ctypes.c_double()
    v_last = np.empty_like(x)
    lib.orc_leapfrog_cosmology(m.size, _d(x), _d(v), _d(m), h, omega_m, omega_lambda, _d(c),
                               box_width, dt, a_begin, a_final, grid, ctypes.byref(steps),
                               ctypes.byref(t), _d(v_last))
    if velocities:
        return x.reshape(-1, 3), steps.value, t.value, v_last.reshape(-1, 3)
    return x.reshape(-1, 3), steps.value, t.value


def energy(x, v, m, G):
    x, v, m = _c(x), _c(v), _c(m)
    return load().orc_energy(m.size, _d(x), _d(v), _d(m), G)


def linear_momentum(v, m):
    v, m = _c(v), _c(m)
    return load().orc_linear_momentum(m.size, _d(v), _d(m))


def angular_momentum(x, v, m):
    x, v, m = _c(x), _c(v), _c(m)
    return load().orc_angular_momentum(m.size, _d(x), _d(v), _d(m))


def direct_rows(x, m, G, eps, rows):
    x, m = _c(x), _c(m)
    rows = _c(rows, np.int32)
    a = np.empty((rows.size, 3))
    load().orc_direct_rows(m.size, _d(x), _d(m), G, eps, rows.size,
                           rows.ctypes.data_as(ip), _d(a))
    return a


def abs_sum_rows(x, m, G, eps, rows=None):
    """A_i = G sum_j m_j |r_ij| / (r_ij^2 + eps^2)^1.5 for the given rows."""
    x, m = _c(x), _c(m)
    rows = np.arange(m.size, dtype=np.int32) if rows is None else _c(rows, np.int32)
    out = np.empty(rows.size)
    load().orc_abs_sum_rows(m.size, _d(x), _d(m), G, eps, rows.size,
                            rows.ctypes.data_as(ip), _d(out))
    return out


def rel_err(a, b):
    """Per-particle |a - b| / |b|."""
    num = np.linalg.norm(np.asarray(a) - np.asarray(b), axis=1)
    den = np.linalg.norm(np.asarray(b), axis=1)
    return num / np.where(den > 0, den, 1.0)


def load_omp():
    """The OpenMP build of the restatement (timing baselines only)."""
    global _omp
    if _omp is not None:
        return _omp
    load()
    if not LIB_OMP.exists() or LIB_OMP.stat().st_mtime < LIB.stat().st_mtime:
        build()
    lib = ctypes.CDLL(str(LIB_OMP))
    lib.orc_build_tree.argtypes = [ctypes.c_int, dp, dp, ctypes.c_int, ctypes.c_int,
                                   ctypes.POINTER(OrcTree)]
    lib.orc_free_tree.argtypes = [ctypes.POINTER(OrcTree)]
    lib.orc_bh_walk_sample.argtypes = [dp, dp, ctypes.c_double, ctypes.c_double,
                                       ctypes.c_double, ctypes.POINTER(OrcTree), ctypes.c_int,
                                       ctypes.c_int64, ctypes.c_int64, ctypes.c_int, dp]
    lib.orc_num_threads.restype = ctypes.c_int
    lib.orc_ensemble_run.argtypes = [ctypes.c_int, ip, lp, ip, dp, dp, dp, ctypes.c_double,
                                     ctypes.c_double, ctypes.c_double, ctypes.c_int]
    _omp = lib
    return lib


def bh_cpu_timing(x, m, G, eps, theta, leaf_max, compat, target_s=10.0):
    """Time grav_sim's Barnes-Hut (src/acceleration_barnes_hut.c:33-248) as
    the reference runs it: the octree built serially, the walk over sorted
    particles OpenMP-parallel.  The walk is timed on a strided sample of the
    sorted particles sized to take about target_s seconds; returns a dict
    with the build time, the walk time per particle, the sample size and the
    threads used."""
    import time
    x, m = _c(x), _c(m)
    n = m.size
    lib = load_omp()
    t = OrcTree()
    t0 = time.perf_counter()
    assert lib.orc_build_tree(n, _d(x), _d(m), leaf_max, int(compat), ctypes.byref(t)) == 0
    build_s = time.perf_counter() - t0
    a = np.zeros((n, 3))
    try:
        count = min(n, 4096)
        while True:
            stride = max(1, n // count)
            count = min(count, (n + stride - 1) // stride)
            t0 = time.perf_counter()
            lib.orc_bh_walk_sample(_d(x), _d(m), G, eps, theta, ctypes.byref(t), int(compat),
                                   stride // 2, stride, count, _d(a))
            walk_s = time.perf_counter() - t0
            if walk_s >= 0.25 * target_s or count >= n:
                break
            count = min(n, int(count * min(64.0, max(2.0, target_s / max(walk_s, 1e-3)))))
    finally:
        lib.orc_free_tree(ctypes.byref(t))
    return {"build_s": build_s, "walk_s_per_particle": walk_s / count, "sample": count,
            "walk_s": walk_s, "threads": int(lib.orc_num_threads())}


def ensemble_cpu_timing(systems, G, dt, steps, integrator):
    """Run the given systems (list of (x, v, m)) for `steps` steps each as
    the reference runs each alone, one system per OpenMP thread; returns
    (seconds, threads)."""
    import time
    lib = load_omp()
    counts = np.array([s_[2].size for s_ in systems], dtype=np.int32)
    off = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.int64)
    ids = np.concatenate([np.arange(c, dtype=np.int32) for c in counts])
    x = _c(np.concatenate([s_[0] for s_ in systems]))
    v = _c(np.concatenate([s_[1] for s_ in systems]))
    m = _c(np.concatenate([s_[2] for s_ in systems]))
    t0 = time.perf_counter()
    rc = lib.orc_ensemble_run(counts.size, counts.ctypes.data_as(ip), off.ctypes.data_as(lp),
                              ids.ctypes.data_as(ip), _d(x), _d(v), _d(m), G, dt,
                              dt * steps * (1 - 1e-9), integrator)
    el = time.perf_counter() - t0
    assert rc == 0, rc
    return el, int(lib.orc_num_threads())
