"""The FP64 restatement of the learned method's features
(tests/learned_features.py), on the oracle's tree, without a GPU: the
properties its definition implies, and one row recomputed by hand from the
tree.  tests/test_gpu_learned.py compares the GPU's features with it."""
import numpy as np

import learned_features as lf


def test_feature_properties(orc, wl):
    n = 4096
    x, v, m = wl.galaxy_pair(n, 12)
    T = orc.build_tree(x, m, 16, False)
    a = np.random.default_rng(3).standard_normal((n, 3))
    f = lf.features(T, x, m, 1.0, a)
    assert f.shape == (n, 32) and np.all(np.isfinite(f))
    assert np.all((f[:, 3] > 0) & (f[:, 3] <= 1))                       # M_L / M_P
    assert np.allclose(np.linalg.norm(f[:, 4:7], axis=1), 1.0)          # direction
    near = f[:, 24:32]
    assert np.all(np.diff(near, axis=1) >= 0) and np.all(near <= 4.0) and np.all(near > 0)
    # traceless quadrupoles
    assert np.allclose(f[:, 7] + f[:, 10] + f[:, 12], 0.0, atol=1e-9)
    assert np.allclose(f[:, 17] + f[:, 20] + f[:, 22], 0.0, atol=1e-9)


def test_one_row_by_hand(orc, wl):
    """The row of sorted position n / 2, from the tree's arrays directly."""
    n = 2048
    x, v, m = wl.galaxy_pair(n, 13)
    T = orc.build_tree(x, m, 16, False)
    a = np.random.default_rng(4).standard_normal((n, 3))
    f = lf.features(T, x, m, 1.0, a)
    nc, fc, fp, npart = T["num_children"], T["first_child"], T["first_particle"], T["num_particles"]
    s = n // 2
    pid = T["sorted_indices"][s]
    leaf = [i for i in range(T["num_nodes"]) if nc[i] == 0 and fp[i] <= s < fp[i] + npart[i]]
    assert len(leaf) == 1
    L = leaf[0]
    P = [i for i in range(T["num_nodes"]) if nc[i] > 0 and fc[i] <= L < fc[i] + nc[i]][0]
    hL = T["box_width"] / 2.0 ** T["depth"][L]
    assert np.allclose(f[s, 0:3], (x[pid] - T["com"][L]) / hL)
    assert np.isclose(f[s, 3], T["mass"][L] / T["mass"][P])
    assert np.allclose(f[s, 4:7], a[pid] / np.linalg.norm(a[pid]))
    assert np.isclose(f[s, 13], np.log(T["mass"][P] / m[pid]) / 10.0)
    assert np.isclose(f[s, 23], np.log10(T["mass"][P] / (2 * hL) ** 3) / 5.0)
