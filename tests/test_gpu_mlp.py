"""The accelerator's MLP kernels (csrc/bte_mlp.cuh) against the CPU oracle
(oracle/mlp.py: FP64 with the same BF16 rounding points), and GPU training."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _lib(sbte):
    L, _ = sbte._load()
    return L


def _data(n, seed=0):
    rng = np.random.default_rng(seed)
    X = rng.normal(0, 1, (n, 8)).astype(np.float32)
    X[:, :3] /= np.abs(X[:, :3]).sum(1, keepdims=True)  # like d_i / s
    Y = (X[:, 0] * 2.0 - X[:, 1] + 0.5 * np.tanh(X[:, 6])).astype(np.float32)
    return X, Y


def test_mlp_param_count(sbte):
    from oracle import mlp
    assert _lib(sbte).bte_mlp_param_count() == mlp.NPARAM == 34305


def test_mlp_forward_matches_oracle(sbte):
    from oracle import mlp
    from staticbtesolver_gb300 import learned
    p = learned.init_params(3)
    p[mlp.OFF_B1:mlp.OFF_W2] = 0.05  # non-zero biases
    p[mlp.OFF_B4] = 0.25
    X, _ = _data(1000, 1)
    y = np.zeros(len(X), np.float32)
    st = _lib(sbte).bte_mlp_predict(X.ctypes.data_as(C.c_void_p), len(X), p.ctypes.data_as(C.c_void_p),
                                    y.ctypes.data_as(C.c_void_p))
    assert st == 0
    yo, _ = mlp.forward(p, X)
    assert np.linalg.norm(y - yo) <= 2e-3 * np.linalg.norm(yo)


def test_mlp_gradient_matches_oracle(sbte):
    from oracle import mlp
    from staticbtesolver_gb300 import learned
    p = learned.init_params(5)
    X, Y = _data(777, 2)  # not a multiple of 16 or of the 256-row slices
    g = np.zeros(mlp.NPARAM, np.float32)
    loss = C.c_double(0)
    st = _lib(sbte).bte_mlp_gradient(X.ctypes.data_as(C.c_void_p), Y.ctypes.data_as(C.c_void_p), len(Y),
                                     p.ctypes.data_as(C.c_void_p), g.ctypes.data_as(C.c_void_p), C.byref(loss))
    assert st == 0
    lo, go = mlp.loss_grad(p, X, Y)
    assert abs(loss.value - lo) <= 1e-3 * lo
    # every block of the flat layout, relative L2
    cuts = [mlp.OFF_W1, mlp.OFF_B1, mlp.OFF_W2, mlp.OFF_B2, mlp.OFF_W3, mlp.OFF_B3, mlp.OFF_W4, mlp.OFF_B4, mlp.NPARAM]
    for a, b in zip(cuts[:-1], cuts[1:]):
        ref = go[a:b]
        assert np.linalg.norm(g[a:b] - ref) <= 2e-2 * np.linalg.norm(ref) + 1e-9, (a, b)


def test_mlp_training_reduces_loss(sbte):
    from staticbtesolver_gb300 import learned
    X, Y = _data(20000, 4)
    p, loss = learned.train(X, Y, steps=400, batch=1024, lr=2e-3, seed=1)
    assert np.isfinite(loss).all()
    assert loss[-20:].mean() < 0.1 * loss[:20].mean()
