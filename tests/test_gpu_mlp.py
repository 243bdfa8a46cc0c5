"""The learned residual network's tcgen05 kernels against the CPU oracle.

Forward: |pred_gpu - pred_cpu| <= 1e-2 |pred_cpu| + 3e-3 elementwise and
||pred_gpu - pred_cpu|| <= 1e-3 ||pred_cpu||.
Backward: for every parameter tensor, ||g_gpu - g_cpu|| <= 2e-2 ||g_cpu||
(both round operands to BF16 at the same points; they differ by FP32
accumulation order, the hardware exp, and the BF16 rounding of values that
land on either side of a rounding boundary).  Training: Adam on a smooth
synthetic regression lowers the loss tenfold.
"""
import ctypes

import numpy as np
import pytest

from oracle import mlp as omlp

pytestmark = pytest.mark.gpu

fp = ctypes.POINTER(ctypes.c_float)


def _bind(lib):
    lib.gsgpu_mlp_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_ulonglong]
    lib.gsgpu_mlp_destroy.argtypes = [ctypes.c_void_p]
    lib.gsgpu_mlp_get_params.argtypes = [ctypes.c_void_p, fp]
    lib.gsgpu_mlp_set_params.argtypes = [ctypes.c_void_p, fp]
    lib.gsgpu_mlp_forward.argtypes = [ctypes.c_void_p, fp, ctypes.c_int, fp]
    lib.gsgpu_mlp_gradients.argtypes = [ctypes.c_void_p, fp, fp, ctypes.c_int, fp,
                                        ctypes.POINTER(ctypes.c_double)]
    lib.gsgpu_mlp_train_step.argtypes = [ctypes.c_void_p, fp, fp, ctypes.c_int, ctypes.c_float,
                                         ctypes.POINTER(ctypes.c_double)]
    assert lib.gsgpu_mlp_num_params() == omlp.NPARAM


def _f(a):
    return np.ascontiguousarray(a, dtype=np.float32)


@pytest.fixture()
def net(lib):
    _bind(lib)
    h = ctypes.c_void_p()
    assert lib.gsgpu_mlp_create(ctypes.byref(h), 1234) == 0
    yield h
    lib.gsgpu_mlp_destroy(h)


def _params(lib, h, rng=None):
    p = np.empty(omlp.NPARAM, dtype=np.float32)
    assert lib.gsgpu_mlp_get_params(h, p.ctypes.data_as(fp)) == 0
    if rng is not None:   # make the last layer non-trivial for the checks
        d = omlp.unpack(p)
        d["W4"][:3] = rng.uniform(-0.3, 0.3, (3, 64))
        d["b4"][:3] = rng.uniform(-0.1, 0.1, 3)
        for k in ("b1", "b2", "b3"):
            d[k] = rng.uniform(-0.2, 0.2, d[k].shape)
        p = omlp.pack(d)
        assert lib.gsgpu_mlp_set_params(h, p.ctypes.data_as(fp)) == 0
    return p


@pytest.mark.parametrize("n", [1, 127, 128, 1000, 20000])
def test_forward_matches_oracle(lib, net, n):
    rng = np.random.default_rng(n)
    p = _params(lib, net, rng)
    x = _f(rng.standard_normal((n, 32)))
    out = np.empty((n, 3), dtype=np.float32)
    assert lib.gsgpu_mlp_forward(net, x.ctypes.data_as(fp), n, out.ctypes.data_as(fp)) == 0
    ref = omlp.forward(p, x)
    # a hidden value landing on the other side of a BF16 rounding boundary
    # moves an output by ~1e-3 at this weight scale
    assert np.all(np.abs(out - ref) <= 1e-2 * np.abs(ref) + 3e-3), float(np.max(np.abs(out - ref)))
    assert np.linalg.norm(out - ref) <= 1e-3 * np.linalg.norm(ref)


@pytest.mark.parametrize("n", [128, 3000, 20000])
def test_gradients_match_oracle(lib, net, n):
    rng = np.random.default_rng(7 + n)
    p = _params(lib, net, rng)
    x = _f(rng.standard_normal((n, 32)))
    t = _f(rng.standard_normal((n, 3)) * 0.3)
    g = np.empty(omlp.NPARAM, dtype=np.float32)
    loss = ctypes.c_double()
    assert lib.gsgpu_mlp_gradients(net, x.ctypes.data_as(fp), t.ctypes.data_as(fp), n,
                                   g.ctypes.data_as(fp), ctypes.byref(loss)) == 0
    gref, lref = omlp.gradients(p, x, t)
    assert abs(loss.value - lref) <= 1e-2 * lref
    G, R = omlp.unpack(g), omlp.unpack(gref)
    for name, _ in omlp.SIZES:
        num = np.linalg.norm(G[name] - R[name])
        den = np.linalg.norm(R[name])
        assert num <= 2e-2 * den + 1e-9, (name, num / max(den, 1e-30))


def test_training_lowers_loss(lib, net):
    rng = np.random.default_rng(3)
    n = 8192
    x = _f(rng.standard_normal((n, 32)))
    wtrue = rng.standard_normal((32, 3)) * 0.3
    t = _f(np.tanh(x @ wtrue) + 0.2 * np.sin(x[:, :3]))
    loss = ctypes.c_double()
    losses = []
    for step in range(300):
        assert lib.gsgpu_mlp_train_step(net, x.ctypes.data_as(fp), t.ctypes.data_as(fp), n,
                                        ctypes.c_float(3e-3), ctypes.byref(loss)) == 0
        losses.append(loss.value / n)
    print(f"loss {losses[0]:.4g} -> {losses[-1]:.4g}")
    assert losses[-1] < 0.1 * losses[0]
