"""Generate the golden vectors under tests/golden/ from grav_sim itself.

grav_sim ships no tests, fixtures or known-answer vectors for its hot path,
so the vectors are made by running the reference C library -- compiled from
its own sources by ``make -C oracle ref`` into oracle/_ref/ -- on seeded
inputs.  Run on a machine where the reference sources are present:

    python tests/golden/make_golden.py

Outputs (compressed .npz, a few hundred KB in total):
  pairwise.npz       acceleration_pairwise   (src/acceleration.c:177-234)
  massless.npz       acceleration_massless   (src/acceleration.c:236-367)
  octree.npz         construct_octree        (src/linear_octree.c:825-962)
  barnes_hut.npz     acceleration_barnes_hut (src/acceleration_barnes_hut.c:33-248)
  integrators.npz    euler / euler_cromer / rk4 / leapfrog (src/integrator.c)
  leapfrog_plummer1024.npz  leapfrog + pairwise, N=1024, dt=1e-3, 1000 steps
  energy.npz         compute_energy_python   (src/python_interface.c:195-243)
  whfast.npz         WHFast, massless / pairwise / softened / removal
                     (src/integrator_whfast.c:200-407)
  rk_embedded.npz    RKF45 / DOPRI / DVERK / RKF78 (src/integrator_rk_embedded.c)
  ias15.npz          IAS15 (src/integrator_ias15.c)
  output.npz         CSV snapshots written during launch_simulation
                     (src/output.c:340-470), one case per loop family
  pm.npz             acceleration_PM and launch_cosmological_simulation
                     (src/acceleration_PM.c, src/integrator_cosmology_leapfrog.c)
  edges.npz          one- and two-particle systems, tf = 0 and three steps, every
                     integrator of launch_simulation

``python tests/golden/make_golden.py whfast output`` remakes only the named
files of the last group (whfast, rk_embedded, ias15, output, pm, edges).
"""
from __future__ import annotations

import importlib.util
import json
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
OUT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

from oracle import reference as ref  # noqa: E402

spec = importlib.util.spec_from_file_location("wl", ROOT / "gravity-simulator_gb300" / "workloads.py")
wl = importlib.util.module_from_spec(spec)
spec.loader.exec_module(wl)


def pairwise_cases():
    cases = {}
    for n in (1, 2, 3, 17, 1024):
        x, v, m = wl.plummer(n, 100 + n)
        cases[f"plummer{n}"] = (x, m, 1.0, 0.01)
    # unsoftened
    x, v, m = wl.plummer(64, 5)
    cases["plummer64_eps0"] = (x, m, 1.0, 0.0)
    # coincident pairs with softening
    x, v, m = wl.plummer(40, 6)
    x[1] = x[0]
    x[7] = x[3]
    cases["coincident"] = (x, m, 1.0, 0.05)
    # collinear, unequal masses, G != 1
    t = np.linspace(-3.0, 5.0, 33)
    x = np.stack([t, 0.5 * t, -2.0 * t], axis=1)
    m = np.linspace(0.5, 2.0, 33)
    cases["collinear"] = (x, m, 0.7, 0.01)
    return cases


def whfast_systems():
    """Planetary systems for WHFast: (name, x, v, m, method, eps, dt, tf)."""
    G = wl.G_AU_MSUN_DAY
    (x, v, m), = wl.planetary_ensemble(1, 7, max_test=64)
    sys_ = [("massless", x, v, m, 2, 0.0, 10.0, 365.0),
            ("pairwise", x, v, m, 1, 0.0, 10.0, 365.0),
            ("massless_soft", x, v, m, 2, 1e-3, 5.0, 101.0)]
    # a test particle on a fast hyperbolic orbit: its Kepler solve overflows
    # (non-finite Stumpff argument) and WHFast removes it
    xe = np.concatenate([x, [[1.0, 0.2, 0.0]]])
    ve = np.concatenate([v, [[100.0, 0.0, 0.0]]])
    me = np.concatenate([m, [0.0]])
    sys_.append(("escape", xe, ve, me, 2, 0.0, 10.0, 100.0))
    return G, sys_


def whfast_cases():
    """WHFast (src/integrator_whfast.c) run by the reference.  The reference
    kicks the primary's Jacobi velocity with an acceleration it never writes
    (a[0] of a malloc'd array), so a run is kept only when it reproduces the
    oracle's a[0] = 0 policy; up to five attempts per case.
    launch_simulation_python (src/python_interface.c:186-190) does not write
    the shrunken particle count back after removals, so the survivors are the
    first k slots of the returned arrays, k from the oracle's count."""
    from oracle import restatement as orc
    G, systems = whfast_systems()
    out = {}
    for name, x, v, m, method, eps, dt, tf in systems:
        ids0 = np.arange(m.size, dtype=np.int32)
        oi, ox, ov, om = orc.whfast_run(x, v, m, G, eps, dt, tf, pairwise=(method == 1), ids=ids0)
        for attempt in range(5):
            ri, rx, rv, rm = ref.launch(x, v, m, G, 10, dt, tf, method, eps=eps)
            k = oi.size
            ri, rx, rv, rm = ri[:k], rx[:k], rv[:k], rm[:k]
            if (np.array_equal(ri, oi) and np.array_equal(rx, ox) and np.array_equal(rv, ov)
                    and np.array_equal(rm, om)):
                break
        else:
            raise AssertionError(f"whfast {name}: reference and oracle differ")
        out[f"{name}/x0"], out[f"{name}/v0"], out[f"{name}/m0"] = x, v, m
        out[f"{name}/method"], out[f"{name}/eps"] = np.int64(method), np.float64(eps)
        out[f"{name}/dt"], out[f"{name}/tf"], out[f"{name}/G"] = (np.float64(dt), np.float64(tf),
                                                                  np.float64(G))
        out[f"{name}/ids"], out[f"{name}/x"], out[f"{name}/v"], out[f"{name}/m"] = ri, rx, rv, rm
    return out


def rk_embedded_cases():
    """RKF45 / DOPRI / DVERK / RKF78 (src/integrator_rk_embedded.c) run by the
    reference: the initial-step estimate (tolerance 1e-8) and a given
    initial dt (tolerance 1e-6), pairwise sum; one massless run."""
    out = {}
    x, v, m = wl.plummer(64, 31)
    out["x"], out["v"], out["m"] = x, v, m
    for integ in (5, 6, 7, 8):
        for tag, tol, idt in (("auto", 1e-8, -1.0), ("given", 1e-6, 1e-3)):
            _, xr, vr, _ = ref.launch(x, v, m, 1.0, integ, 1e-3, 0.5, 1, eps=0.01, tolerance=tol,
                                      initial_dt=idt)
            out[f"int{integ}_{tag}/x"], out[f"int{integ}_{tag}/v"] = xr, vr
            out[f"int{integ}_{tag}/tol"], out[f"int{integ}_{tag}/initial_dt"] = (np.float64(tol),
                                                                                 np.float64(idt))
    (xs, vs, ms), = wl.planetary_ensemble(1, 11, max_test=30)
    _, xr, vr, _ = ref.launch(xs, vs, ms, wl.G_AU_MSUN_DAY, 6, 1.0, 200.0, 2, tolerance=1e-9)
    out["massless_x0"], out["massless_v0"], out["massless_m"] = xs, vs, ms
    out["massless_G"] = np.float64(wl.G_AU_MSUN_DAY)
    out["massless_x"], out["massless_v"] = xr, vr
    return out


def ias15_cases():
    """IAS15 (src/integrator_ias15.c) run by the reference: the initial-step
    estimate (tolerance 1e-9) and a given initial dt (1e-6), pairwise sum;
    one massless planetary run."""
    out = {}
    x, v, m = wl.plummer(64, 31)
    out["x"], out["v"], out["m"] = x, v, m
    for tag, tol, idt in (("auto", 1e-9, -1.0), ("given", 1e-6, 1e-3)):
        _, xr, vr, _ = ref.launch(x, v, m, 1.0, 9, 1e-3, 0.5, 1, eps=0.01, tolerance=tol,
                                  initial_dt=idt)
        out[f"{tag}/x"], out[f"{tag}/v"] = xr, vr
        out[f"{tag}/tol"], out[f"{tag}/initial_dt"] = np.float64(tol), np.float64(idt)
    (xs, vs, ms), = wl.planetary_ensemble(1, 11, max_test=30)
    _, xr, vr, _ = ref.launch(xs, vs, ms, wl.G_AU_MSUN_DAY, 9, 1.0, 200.0, 2, tolerance=1e-9)
    out["massless_x0"], out["massless_v0"], out["massless_m"] = xs, vs, ms
    out["massless_G"] = np.float64(wl.G_AU_MSUN_DAY)
    out["massless_x"], out["massless_v"] = xr, vr
    return out


OUTPUT_CASES = {
    # name: (system, integrator, method, dt, tf, extra launch arguments, output arguments)
    "leapfrog": ("plummer", 4, 1, 1e-3, 0.0105, {"eps": 0.01},
                 dict(output_initial=True, output_interval=3e-3)),
    "euler_float": ("plummer", 1, 1, 1e-3, 0.006, {"eps": 0.01},
                    dict(output_initial=False, output_interval=2e-3, coordinate_output_dtype=1,
                         mass_output_dtype=1)),
    "rk4": ("plummer", 3, 1, 1e-3, 0.009, {"eps": 0.01},
            dict(output_initial=True, output_interval=4e-3, velocity_output_dtype=1)),
    "rkf45": ("plummer", 5, 1, 1e-3, 0.05, {"eps": 0.01, "tolerance": 1e-8},
              dict(output_initial=True, output_interval=1e-2)),
    "ias15": ("plummer", 9, 1, 1e-3, 0.05, {"eps": 0.01, "tolerance": 1e-9},
              dict(output_initial=True, output_interval=1e-2)),
    "whfast": ("planetary", 10, 2, 1.0, 50.5, {},
               dict(output_initial=True, output_interval=10.0)),
}


def output_system(kind):
    if kind == "plummer":
        x, v, m = wl.plummer(24, 51)
        return x, v, m, 1.0
    (x, v, m), = wl.planetary_ensemble(1, 10, max_test=12)
    return x, v, m, wl.G_AU_MSUN_DAY


def output_cases():
    """Snapshot files the reference writes (CSV output method) for one case of
    each loop family, stored byte for byte as uint8 arrays under
    "<case>/<file name>".  The reference's Python entry point leaves the
    status of the initial snapshot (output_initial) uninitialised, so the
    time and dt lines of snapshot_00000.csv in those cases carry no meaning."""
    out = {}
    for name, (kind, integ, method, dt, tf, extra, oargs) in OUTPUT_CASES.items():
        x, v, m, G = output_system(kind)
        with tempfile.TemporaryDirectory() as tmp:
            d = Path(tmp) / "snaps"
            ref.launch(x, v, m, G, integ, dt, tf, method, output_method=2,
                       output_dir=str(d) + "/", **extra, **oargs)
            files = sorted(d.iterdir())
            assert files, name
            for f in files:
                out[f"{name}/{f.name}"] = np.frombuffer(f.read_bytes(), dtype=np.uint8)
        args = dict(kind=kind, integrator=integ, method=method, dt=dt, tf=tf, extra=extra,
                    output=oargs)
        out[f"{name}/args.json"] = np.frombuffer(json.dumps(args).encode(), dtype=np.uint8)
        out[f"{name}/x0"], out[f"{name}/v0"], out[f"{name}/m0"] = x, v, m
        out[f"{name}/G"] = np.float64(G)
    return out


def pm_cases():
    """Particle-mesh force and cosmological leapfrog of the reference
    (src/acceleration_PM.c, src/integrator_cosmology_leapfrog.c), built from
    its own sources with FFTW's calls served by the oracle's direct DFT
    (oracle/fftw_compat): uniform and clustered particles, an off-centre
    box, particles on the box faces; and a five-step cosmological run with
    particles leaving the box."""
    out = {}
    rng = np.random.default_rng(61)
    c = np.array([1.5, -2.0, 0.25])
    bw = 4.0
    cases = {
        "uniform_g16": (c + rng.uniform(-bw, bw, (2000, 3)), np.full(2000, 1.0 / 2000), 16),
        "clustered_g32": (c + np.clip(wl.plummer(2500, 62)[0] * 0.8, -bw, bw),
                          rng.uniform(0.5, 1.5, 2500) / 2500, 32),
    }
    xf = c + rng.uniform(-bw, bw, (200, 3))
    xf[:20, 0] = c[0] + bw            # on the upper face: cell index g wraps to 0
    xf[20:40, 1] = c[1] - bw          # on the lower face
    cases["faces_g8"] = (xf, np.full(200, 0.005), 8)
    H0, om = 70.0, 0.3
    for name, (x, m, grid) in cases.items():
        rho = m.sum() / ((bw * 2) ** 3)
        a = ref.acceleration_pm(x, m, c, bw, H0, om, rho, grid, 0.5)
        out[f"{name}/x"], out[f"{name}/m"], out[f"{name}/grid"] = x, m, np.int64(grid)
        out[f"{name}/a"] = a
    out["box_center"], out["box_width"] = c, np.float64(bw)
    out["H0"], out["omega_m"], out["scale_factor"] = np.float64(H0), np.float64(om), np.float64(0.5)
    # cosmological run: 1000 particles, 16^3 mesh, a = 0.1 -> 0.2 in steps of 0.02
    n = 1000
    x = c + rng.uniform(-bw, bw, (n, 3))
    v = rng.normal(0.0, 40.0, (n, 3))
    m = np.full(n, 1.0)
    x[0] = c + np.array([bw + 0.5, -bw - 9.0, 0.0])   # starts outside: wrapped first
    kw = dict(h=0.7, omega_m=0.3, omega_lambda=0.7, box_center=c, box_width=bw, dt=0.02,
              a_begin=0.1, a_final=0.2, pm_grid_size=16)
    xr, (t, dt, steps) = ref.cosmological_run(x, v, m, **kw)
    out["cosmo/x0"], out["cosmo/v0"], out["cosmo/m"] = x, v, m
    out["cosmo/x"], out["cosmo/t"], out["cosmo/steps"] = xr, np.float64(t), np.int64(steps)
    out["cosmo/args.json"] = np.frombuffer(json.dumps({k: (list(map(float, v)) if k == "box_center"
                                                           else v) for k, v in kw.items()}).encode(),
                                           dtype=np.uint8)
    return out


def edge_cases():
    """One- and two-particle systems through every integrator of
    launch_simulation, for no time (tf = 0) and three steps, pairwise sum
    (massless for WHFast).  IAS15 with a single particle is left out: its
    error estimate is 0/0 and the reference's step loop never ends.  So is
    WHFast with two particles over steps: the reference kicks the centre-of-
    mass velocity with a[0], which it never writes (src/integrator_whfast.c
    :409-422), and in this run that memory held a non-zero value."""
    out = {}
    x, v, m = wl.plummer(3, 5)
    out["x"], out["v"], out["m"] = x, v, m
    for n in (1, 2):
        for integ in (1, 2, 3, 4, 5, 6, 7, 8, 9, 10):
            if integ == 9 and n == 1:
                continue
            tfs = (0.0,) if (integ == 10 and n == 2) else (0.0, 3e-3)
            for tf in tfs:
                kw = dict(tolerance=1e-8) if 5 <= integ <= 9 else {}
                method = 2 if integ == 10 else 1
                ids, xr, vr, mr = ref.launch(x[:n], v[:n], m[:n], 1.0, integ, 1e-3, tf, method,
                                             eps=0.01, **kw)
                key = f"n{n}_int{integ}_tf{tf:g}"
                out[f"{key}/ids"], out[f"{key}/x"], out[f"{key}/v"] = ids, xr, vr
    return out


LATE = {
    "whfast": lambda: whfast_cases(),
    "rk_embedded": lambda: rk_embedded_cases(),
    "ias15": lambda: ias15_cases(),
    "output": lambda: output_cases(),
    "pm": lambda: pm_cases(),
    "edges": lambda: edge_cases(),
}


def main():
    assert ref.build() or ref.available(), "reference sources not found"
    if len(sys.argv) > 1:
        for name in sys.argv[1:]:
            np.savez_compressed(OUT / f"{name}.npz", **LATE[name]())
            print(name, (OUT / f"{name}.npz").stat().st_size)
        return
    out = {}
    for name, (x, m, G, eps) in pairwise_cases().items():
        a = ref.acceleration(x, m, G, 1, eps=eps)
        out[f"{name}/x"], out[f"{name}/m"] = x, m
        out[f"{name}/G"], out[f"{name}/eps"], out[f"{name}/a"] = np.float64(G), np.float64(eps), a
    np.savez_compressed(OUT / "pairwise.npz", **out)

    out = {}
    x, v, m = wl.plummer(300, 11)
    m1 = m.copy()
    m1[100:] = 0.0                      # massive first
    m2 = m.copy()
    m2[1::4] = 0.0                      # interleaved (loop-index mass read)
    for name, mm in (("massive_first", m1), ("interleaved", m2)):
        out[f"{name}/x"], out[f"{name}/m"] = x, mm
        out[f"{name}/a"] = ref.acceleration(x, mm, 1.0, 2, eps=0.01)
    np.savez_compressed(OUT / "massless.npz", **out)

    out = {}
    tree_cases = {}
    x, v, m = wl.plummer(3000, 21)
    for leaf in (1, 8, 64):
        tree_cases[f"plummer3000_leaf{leaf}"] = (x, m, leaf)
    # particles on the bounding-box maximum (2^21 wraps to 0) and duplicates
    x2, v2, m2 = wl.plummer(500, 22)
    x2[10] = x2.max(axis=0)
    x2[11] = x2.min(axis=0)
    x2[20:40] = x2[5]                   # 21 coincident particles -> level-21 leaf
    tree_cases["edges_leaf1"] = (x2, m2, 1)
    tree_cases["edges_leaf4"] = (x2, m2, 4)
    tree_cases["single"] = (np.array([[0.3, -0.2, 0.1]]), np.array([1.0]), 1)
    tree_cases["pair"] = (np.array([[0.0, 0.0, 0.0], [1.0, 0.5, -0.25]]), np.array([1.0, 2.0]), 1)
    g = wl.galaxy_pair(4096, 4)
    tree_cases["galaxy4096_leaf1"] = (g[0], g[2], 1)
    for name, (xx, mm, leaf) in tree_cases.items():
        t = ref.octree(xx, mm, leaf)
        out[f"{name}/x"], out[f"{name}/m"], out[f"{name}/leaf"] = xx, mm, np.int64(leaf)
        for k in ("keys", "sorted_indices", "num_particles", "num_children", "first_particle",
                  "first_child", "mass", "com"):
            out[f"{name}/{k}"] = t[k]
        out[f"{name}/box_width"] = np.float64(t["box_width"])
    np.savez_compressed(OUT / "octree.npz", **out)

    out = {}
    for name in ("plummer3000_leaf1", "plummer3000_leaf8", "edges_leaf1", "galaxy4096_leaf1"):
        xx, mm, leaf = tree_cases[name]
        out[f"{name}/x"], out[f"{name}/m"], out[f"{name}/leaf"] = xx, mm, np.int64(leaf)
        for th in (0.5, 1.0):
            out[f"{name}/a_theta{th}"] = ref.acceleration(xx, mm, 1.0, 3, theta=th, eps=0.01,
                                                          leaf=leaf)
    np.savez_compressed(OUT / "barnes_hut.npz", **out)

    out = {}
    x, v, m = wl.plummer(64, 31)
    out["x"], out["v"], out["m"] = x, v, m
    for integ in (1, 2, 3, 4):
        _, xr, vr, _ = ref.launch(x, v, m, 1.0, integ, 1e-3, 0.0995, 1, eps=0.01)
        out[f"int{integ}/x"], out[f"int{integ}/v"] = xr, vr
    np.savez_compressed(OUT / "integrators.npz", **out)

    x, v, m = wl.plummer(1024, 1)
    _, xr, vr, _ = ref.launch(x, v, m, 1.0, 4, 1e-3, 1.0, 1, eps=0.01)
    np.savez_compressed(OUT / "leapfrog_plummer1024.npz", x0=x, v0=v, m=m, x=xr, v=vr,
                        e0=ref.energy_python(x, v, m, 1.0), e1=ref.energy_python(xr, vr, m, 1.0))

    x, v, m = wl.plummer(777, 41)
    np.savez_compressed(OUT / "energy.npz", x=x, v=v, m=m, G=np.float64(1.3),
                        e=ref.energy_python(x, v, m, 1.3))

    for name, make in LATE.items():
        np.savez_compressed(OUT / f"{name}.npz", **make())
    for f in sorted(OUT.glob("*.npz")):
        print(f.name, f.stat().st_size)


if __name__ == "__main__":
    main()
