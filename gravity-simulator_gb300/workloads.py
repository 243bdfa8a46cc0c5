"""Seeded synthetic initial conditions for the benchmark workloads.

grav_sim publishes no benchmark dataset; its examples draw time-seeded
random ICs (src/utils.c:61-67).  These generators stand in for them with
numpy ``default_rng(seed)`` so every run and test sees the same inputs:

* ``plummer``            -- equal-mass Plummer sphere, G = M = a = 1,
                            Aarseth-Henon-Wielen velocity sampling;
* ``galaxy_pair``        -- two disk + bulge + halo galaxies on a parabolic
                            orbit (the galaxy-collision workload);
* ``planetary_ensemble`` -- Sun + 8 planets + massless test particles per
                            system (the batched-ensemble workload).
"""
from __future__ import annotations

import math

import numpy as np

G_AU_MSUN_DAY = 0.000295912208284119496676630  # grav_sim/system.py:34


def _zero_com(x, v, m):
    M = m.sum()
    x -= (m[:, None] * x).sum(0) / M
    v -= (m[:, None] * v).sum(0) / M


def plummer(n: int, seed: int, scale: float = 1.0):
    """Plummer sphere in virial equilibrium with total mass 1, G = 1."""
    rng = np.random.default_rng(seed)
    m = np.full(n, 1.0 / n)
    # radius from the inverse cumulative mass profile (truncated at 0.999)
    u = rng.uniform(1e-10, 0.999, n)
    r = scale / np.sqrt(u ** (-2.0 / 3.0) - 1.0)
    x = r[:, None] * _iso(rng, n)
    # speed: q = v / v_esc from g(q) = q^2 (1 - q^2)^3.5 by rejection
    q = np.empty(n)
    todo = np.arange(n)
    while todo.size:
        qq = rng.uniform(0.0, 1.0, todo.size)
        yy = rng.uniform(0.0, 0.1, todo.size)
        ok = yy < qq * qq * (1.0 - qq * qq) ** 3.5
        q[todo[ok]] = qq[ok]
        todo = todo[~ok]
    vesc = np.sqrt(2.0) * (1.0 + (r / scale) ** 2) ** (-0.25) / math.sqrt(scale)
    v = (q * vesc)[:, None] * _iso(rng, n)
    _zero_com(x, v, m)
    return np.ascontiguousarray(x), np.ascontiguousarray(v), m


def _iso(rng, n):
    ct = rng.uniform(-1.0, 1.0, n)
    ph = rng.uniform(0.0, 2.0 * math.pi, n)
    st = np.sqrt(1.0 - ct * ct)
    return np.stack([st * np.cos(ph), st * np.sin(ph), ct], axis=1)


def _hernquist_radii(rng, n, a, rmax):
    # M(<r) = r^2/(r+a)^2  ->  r = a sqrt(u)/(1 - sqrt(u)), truncated at rmax
    umax = (rmax / (rmax + a)) ** 2
    s = np.sqrt(rng.uniform(0.0, umax, n))
    return a * s / (1.0 - s)


def _galaxy(rng, n, mass):
    """Exponential disk (20%), Hernquist bulge (10%, a=0.2), Hernquist
    halo (70%, a=5); equal-mass particles; near-circular disk velocities,
    isotropic dispersion ~ local circular speed for the spheroids."""
    nd = int(round(0.2 * n))
    nb = int(round(0.1 * n))
    nh = n - nd - nb
    mp = mass / n
    # disk: exponential in R (scale 1), sech^2 in z (scale 0.1)
    R = np.empty(nd)
    todo = np.arange(nd)
    while todo.size:
        # R from gamma(2, 1) (surface density R e^{-R})
        rr = rng.gamma(2.0, 1.0, todo.size)
        ok = rr < 10.0
        R[todo[ok]] = rr[ok]
        todo = todo[~ok]
    ph = rng.uniform(0.0, 2.0 * math.pi, nd)
    z = 0.1 * np.arctanh(rng.uniform(-0.999, 0.999, nd))
    xd = np.stack([R * np.cos(ph), R * np.sin(ph), z], axis=1)
    rb = _hernquist_radii(rng, nb, 0.2, 5.0)
    xb = rb[:, None] * _iso(rng, nb)
    rh = _hernquist_radii(rng, nh, 5.0, 30.0)
    xh = rh[:, None] * _iso(rng, nh)
    x = np.concatenate([xd, xb, xh])

    # enclosed mass (all components, spherical approximation) -> v_c
    r_all = np.linalg.norm(x, axis=1)
    order = np.argsort(r_all, kind="stable")
    menc = np.empty(n)
    menc[order] = np.arange(1, n + 1) * mp
    vc = np.sqrt(menc / np.maximum(r_all, 1e-3))
    v = np.empty_like(x)
    # disk: circular + 5% dispersion
    vcd = vc[:nd]
    v[:nd, 0] = -vcd * np.sin(ph)
    v[:nd, 1] = vcd * np.cos(ph)
    v[:nd, 2] = 0.0
    v[:nd] += 0.05 * vcd[:, None] * rng.standard_normal((nd, 3))
    # spheroids: isotropic Gaussian with sigma = v_c / sqrt(3)
    sig = vc[nd:] / math.sqrt(3.0)
    v[nd:] = sig[:, None] * rng.standard_normal((n - nd, 3))
    m = np.full(n, mp)
    _zero_com(x, v, m)
    return x, v, m


def galaxy_pair(n_total: int, seed: int, separation: float = 20.0):
    """Two galaxies of mass 1 each, n_total/2 particles each, on a
    parabolic orbit (relative speed sqrt(2 G M_tot / d)) with impact
    parameter 2, 20 units apart."""
    rng = np.random.default_rng(seed)
    n1 = n_total // 2
    n2 = n_total - n1
    x1, v1, m1 = _galaxy(rng, n1, 1.0)
    x2, v2, m2 = _galaxy(rng, n2, 1.0)
    # tilt the second disk
    c, s = math.cos(0.6), math.sin(0.6)
    rot = np.array([[1, 0, 0], [0, c, -s], [0, s, c]])
    x2 = x2 @ rot.T
    v2 = v2 @ rot.T
    d = separation
    b = 2.0
    vrel = math.sqrt(2.0 * 2.0 / math.hypot(d, b))
    x1 += np.array([-d / 2, -b / 2, 0.0])
    x2 += np.array([d / 2, b / 2, 0.0])
    v1 += np.array([vrel / 2, 0.0, 0.0])
    v2 += np.array([-vrel / 2, 0.0, 0.0])
    x = np.concatenate([x1, x2])
    v = np.concatenate([v1, v2])
    # equal-mass particles, total mass 2 (each galaxy has mass 1)
    m = np.full(n_total, 2.0 / n_total)
    _zero_com(x, v, m)
    return np.ascontiguousarray(x), np.ascontiguousarray(v), m


PLANET_MASSES = np.array([1.660e-7, 2.448e-6, 3.003e-6, 3.227e-7,
                          9.548e-4, 2.859e-4, 4.366e-5, 5.151e-5])


def kepler_to_cartesian(a, e, inc, argp, node, f, mu):
    """Keplerian elements -> heliocentric Cartesian (vectorised)."""
    p = a * (1.0 - e * e)
    r = p / (1.0 + e * np.cos(f))
    xo = r * np.cos(f)
    yo = r * np.sin(f)
    h = np.sqrt(mu * p)
    vxo = -mu / h * np.sin(f)
    vyo = mu / h * (e + np.cos(f))
    cO, sO = np.cos(node), np.sin(node)
    cw, sw = np.cos(argp), np.sin(argp)
    ci, si = np.cos(inc), np.sin(inc)
    r11 = cO * cw - sO * sw * ci
    r12 = -cO * sw - sO * cw * ci
    r21 = sO * cw + cO * sw * ci
    r22 = -sO * sw + cO * cw * ci
    r31 = sw * si
    r32 = cw * si
    x = np.stack([r11 * xo + r12 * yo, r21 * xo + r22 * yo, r31 * xo + r32 * yo], -1)
    v = np.stack([r11 * vxo + r12 * vyo, r21 * vxo + r22 * vyo, r31 * vxo + r32 * vyo], -1)
    return x, v


def planetary_ensemble(num_systems: int, seed: int, max_test: int = 4096):
    """List of (x, v, m) per system: Sun (1 Msun) + 8 planets with a
    log-spaced over 0.39-30 AU, e~U[0,0.1], i~U[0,3 deg], random angles;
    L = floor(exp(U[0, ln(max_test+1)))) - 1 massless test particles with
    a~U[2.0,3.5] AU, e~U[0,0.1], i~U[0,5 deg].  Massive bodies come first."""
    rng = np.random.default_rng(seed)
    out = []
    a_pl = np.exp(np.linspace(math.log(0.39), math.log(30.0), 8))
    G = G_AU_MSUN_DAY
    for _ in range(num_systems):
        L = int(math.floor(math.exp(rng.uniform(0.0, math.log(max_test + 1))))) - 1
        L = max(0, min(max_test, L))
        e = rng.uniform(0.0, 0.1, 8)
        inc = np.radians(rng.uniform(0.0, 3.0, 8))
        ang = rng.uniform(0.0, 2.0 * math.pi, (3, 8))
        xp, vp = kepler_to_cartesian(a_pl, e, inc, ang[0], ang[1], ang[2],
                                     G * (1.0 + PLANET_MASSES))
        at = rng.uniform(2.0, 3.5, L)
        et = rng.uniform(0.0, 0.1, L)
        it = np.radians(rng.uniform(0.0, 5.0, L))
        angt = rng.uniform(0.0, 2.0 * math.pi, (3, L))
        xt, vt = kepler_to_cartesian(at, et, it, angt[0], angt[1], angt[2], G)
        x = np.concatenate([np.zeros((1, 3)), xp, xt])
        v = np.concatenate([np.zeros((1, 3)), vp, vt])
        m = np.concatenate([[1.0], PLANET_MASSES, np.zeros(L)])
        _zero_com(x, v, m)
        out.append((np.ascontiguousarray(x), np.ascontiguousarray(v), m))
    return out
