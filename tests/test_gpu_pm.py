"""Particle-mesh gravity and the cosmological leapfrog on the GPU.

acceleration_PM runs its cloud-in-cell deposit, Green's function, gradient
and interpolation as GPU kernels that repeat the reference's FP64
expressions (src/acceleration_PM.c), with the 3-D transforms through cuFFT.
The reference's transforms are FFTW's; the golden vectors were made with the
oracle's direct DFT standing in, and the deposit here adds with atomics in
no fixed order, so the comparison is to a tolerance: every component within
1e-10 of the largest acceleration (FP64 transforms of 16^3-64^3 meshes agree
to ~1e-14 of their largest term).
"""
import json

import numpy as np
import pytest

from conftest import cases, golden

pytestmark = pytest.mark.gpu

REL = 1e-10


def _close(a, ref, rel=REL):
    scale = np.abs(ref).max()
    err = np.abs(a - ref).max()
    assert err <= rel * scale, (err, scale)


def test_acceleration_pm_golden(lib, g):
    d = golden("pm")
    c, bw = d["box_center"], float(d["box_width"])
    H0, om, sf = float(d["H0"]), float(d["omega_m"]), float(d["scale_factor"])
    for name, cs in cases(d).items():
        if name == "cosmo":
            continue
        rho = cs["m"].sum() / ((bw * 2) ** 3)
        a = g.acceleration_pm(lib, cs["x"], cs["m"], c, bw, H0, om, rho, int(cs["grid"]), sf)
        _close(a, cs["a"])


def test_acceleration_pm_oracle_g64(lib, g, orc):
    """A 64^3 mesh with 200,000 clustered particles against the oracle."""
    rng = np.random.default_rng(5)
    c, bw = np.array([0.0, 0.0, 0.0]), 10.0
    n = 200_000
    x = np.clip(rng.standard_normal((n, 3)) * 2.5, -bw, bw)
    m = rng.uniform(0.5, 1.5, n)
    rho = m.sum() / ((bw * 2) ** 3)
    a = g.acceleration_pm(lib, x, m, c, bw, 70.0, 0.3, rho, 64, 0.25)
    a_ref = orc.acceleration_pm(x, m, c, bw, 70.0, 0.3, rho, 64, 0.25)
    _close(a, a_ref)


def test_acceleration_pm_momentum_and_determinism(lib, g):
    """Size-independent properties at 128^3 and 2M particles: the mesh force
    of a periodic box sums to zero (Newton's third law on the mesh, to the
    rounding of the transforms), and two calls agree to the atomic-order
    rounding of the deposit."""
    rng = np.random.default_rng(9)
    c, bw = np.array([5.0, 5.0, 5.0]), 5.0
    n = 2_000_000
    x = c + rng.uniform(-bw, bw, (n, 3))
    m = np.full(n, 1.0)
    rho = m.sum() / ((bw * 2) ** 3)
    a1 = g.acceleration_pm(lib, x, m, c, bw, 70.0, 0.3, rho, 128, 1.0)
    a2 = g.acceleration_pm(lib, x, m, c, bw, 70.0, 0.3, rho, 128, 1.0)
    scale = np.abs(a1).max()
    assert np.isfinite(a1).all() and scale > 0
    assert np.abs(a1 - a2).max() <= 1e-12 * scale
    assert np.abs((m[:, None] * a1).sum(0)).max() <= 1e-8 * scale * m.sum()


def test_cosmological_simulation_golden(lib, g):
    cs = cases(golden("pm"))["cosmo"]
    kw = json.loads(bytes(cs["args.json"]).decode())
    x = cs["x0"].copy()
    v = cs["v0"].copy()
    st = g.launch_cosmological_simulation(lib, x, v, cs["m"], **kw)
    assert st.num_steps == int(cs["steps"]) and st.t == float(cs["t"])
    assert np.array_equal(v, cs["v0"])             # the reference leaves v alone
    assert np.abs(x - cs["x"]).max() <= 1e-9 * kw["box_width"]
    lo = np.array(kw["box_center"]) - kw["box_width"]
    hi = np.array(kw["box_center"]) + kw["box_width"]
    assert ((x >= lo) & (x <= hi)).all()
