"""FP64 restatement of the learned method's 32 per-particle features
(k_learned.cu, k_features), for tests/test_gpu_learned.py.

The features are this library's own design (grav_sim has no learned
method), so this is not a restatement of the reference: it computes, in FP64
with numpy, what the kernel's header comment defines, on the oracle's octree
of the same positions (whose topology, masses and centres of mass equal the
GPU tree's).  For sorted particle s with leaf L, parent P and grandparent GP
(P = L at the root, GP = P below it), cell widths hL = W / 2^depth(L) and
hP = 2 hL (W the box width), the position x, centres of mass c, masses M,
traceless quadrupoles Q = sum m (3 d d^T - |d|^2 I) about the centre of mass,
and a_c the cheap walk's acceleration:

    0-2   (x - c_L) / hL            3   M_L / M_P
    4-6   a_c / |a_c|               7-12  Q_L / (M_L hL^2)  (xx xy xz yy yz zz)
    13    ln(M_P / m) / 10 (0 for a massless particle)
    14    log10(|a_c| hP^2 / (G M_P)) / 5
    15    log10(M_GP / M_P) / 3 (0 when GP = P)
    16    log10(|a_c| W^2 / (G M_root)) / 5
    17-22 Q_P / (M_P hP^2)          23  log10(M_P / hP^3) / 5
    24-31 the 8 smallest of |x - c_k| / hP over the candidate cells k, in
          ascending order, 4 where there are fewer than 8 below 4: the
          children of GP whose depth is at least L's or that are leaves, and
          the children of GP's other children, other than L itself.
"""
from __future__ import annotations

import numpy as np


def node_quadrupoles(T: dict, xs: np.ndarray, ms: np.ndarray) -> np.ndarray:
    """(num_nodes, 6) traceless quadrupoles of every node about its centre
    of mass, from its particles (sorted order xs, ms)."""
    nn = T["num_nodes"]
    fp, npart, com = T["first_particle"], T["num_particles"], T["com"]
    Q = np.zeros((nn, 6))
    for i in range(nn):
        a, b = fp[i], fp[i] + npart[i]
        if b <= a:
            continue
        d = xs[a:b] - com[i]
        w = ms[a:b]
        r2 = np.einsum("ij,ij->i", d, d)
        Q[i] = [np.sum(w * (3 * d[:, 0] * d[:, 0] - r2)), np.sum(w * 3 * d[:, 0] * d[:, 1]),
                np.sum(w * 3 * d[:, 0] * d[:, 2]), np.sum(w * (3 * d[:, 1] * d[:, 1] - r2)),
                np.sum(w * 3 * d[:, 1] * d[:, 2]), np.sum(w * (3 * d[:, 2] * d[:, 2] - r2))]
    return Q


def features(T: dict, x: np.ndarray, m: np.ndarray, G: float, a_cheap: np.ndarray) -> np.ndarray:
    """(N, 32) features of every particle, row s for sorted particle s."""
    n = m.shape[0]
    nn = T["num_nodes"]
    nc, fc = T["num_children"], T["first_child"]
    fp, npart, depth = T["first_particle"], T["num_particles"], T["depth"]
    mass, com, sidx, W = T["mass"], T["com"], T["sorted_indices"], T["box_width"]
    tiny = np.finfo(np.float32).tiny
    parent = np.full(nn, -1)
    leaf_of = np.empty(n, dtype=np.int64)
    for i in range(nn):
        if nc[i] > 0:
            parent[fc[i]:fc[i] + nc[i]] = i
        else:
            leaf_of[fp[i]:fp[i] + npart[i]] = i
    xs, ms = x[sidx], m[sidx]
    Q = node_quadrupoles(T, xs, ms)
    L = leaf_of
    P = np.where(parent[L] >= 0, parent[L], L)
    GP = np.where(parent[P] >= 0, parent[P], P)
    hL = W / 2.0 ** np.minimum(depth[L], 30)
    hP = 2.0 * hL
    ML, MP = np.maximum(mass[L], tiny), np.maximum(mass[P], tiny)
    a = a_cheap[sidx]
    am = np.linalg.norm(a, axis=1)
    ia = np.where(am > 0, 1.0 / np.where(am > 0, am, 1.0), 0.0)
    f = np.zeros((n, 32))
    f[:, 0:3] = (xs - com[L]) / hL[:, None]
    f[:, 3] = ML / MP
    f[:, 4:7] = a * ia[:, None]
    f[:, 7:13] = Q[L] / (ML * hL * hL)[:, None]
    with np.errstate(divide="ignore"):
        f[:, 13] = np.where(ms > 0, np.log(MP / np.where(ms > 0, ms, 1.0)) / 10.0, 0.0)
    lam = np.log10(np.maximum(am, tiny))
    f[:, 14] = (lam + 2 * np.log10(hP) - np.log10(G) - np.log10(MP)) / 5.0
    f[:, 15] = np.where(GP != P, (np.log10(np.maximum(mass[GP], tiny)) - np.log10(MP)) / 3.0, 0.0)
    f[:, 16] = (lam + 2 * np.log10(W) - np.log10(G) - np.log10(max(mass[0], tiny))) / 5.0
    f[:, 17:23] = Q[P] / (MP * hP * hP)[:, None]
    f[:, 23] = (np.log10(MP) - 3 * np.log10(hP)) / 5.0
    # nearest cells: the candidates depend on the leaf alone
    f[:, 24:32] = 4.0
    for leaf in np.unique(L):
        rows = np.arange(fp[leaf], fp[leaf] + npart[leaf])
        p_, gp = P[rows[0]], GP[rows[0]]
        if gp == leaf:
            continue
        cand = []
        for u in range(fc[gp], fc[gp] + nc[gp]):
            if nc[u] <= 0 or depth[u] >= depth[leaf]:
                cand.append(u)
            else:
                cand.extend(range(fc[u], fc[u] + nc[u]))
        cand = [c for c in cand if c != leaf]
        if not cand:
            continue
        d = np.linalg.norm(xs[rows][:, None, :] - com[cand][None, :, :], axis=2) / hP[rows][:, None]
        d = np.concatenate([d, np.full((rows.size, 8), 4.0)], axis=1)
        f[rows, 24:32] = np.sort(d, axis=1)[:, :8]
    return f
