"""The learned preconditioner's MLP: numpy reference (oracle/mlp_ref.py) self-check
on CPU, and the CUDA forward / backward / Adam kernels against it on the GPU.

Bars: CUDA forward within 1e-5 relative of the FP64 reference; CUDA gradient
within 2e-3 relative (norm-wise, FP32 arithmetic) of the analytic FP64
gradient; the reference's analytic gradient within 1e-6 of central finite
differences.
"""
import numpy as np
import pytest

import mlp_ref


def _data(n, seed):
    rng = np.random.default_rng(seed)
    X = rng.normal(size=(n, mlp_ref.IN)).astype(np.float32)
    g = (np.tanh(X[:, 0] - 0.5 * X[:, 2]) + 0.3 * X[:, 5]).astype(np.float32)
    w = rng.uniform(0.2, 2.0, n).astype(np.float32)
    return X, g, w


def _params(seed):
    rng = np.random.default_rng(seed)
    return (rng.normal(size=mlp_ref.NPARAM) * 0.2).astype(np.float32)


def test_reference_gradient_matches_finite_differences():
    X, g, w = _data(40, 1)
    p = _params(2).astype(np.float64)
    _, grad = mlp_ref.loss_and_grad(p, X, g, w)
    rng = np.random.default_rng(3)
    for k in rng.choice(mlp_ref.NPARAM, 25, replace=False):
        e = np.zeros_like(p)
        e[k] = 1e-6
        fd = (mlp_ref.loss_and_grad(p + e, X, g, w)[0] - mlp_ref.loss_and_grad(p - e, X, g, w)[0]) / 2e-6
        assert abs(fd - grad[k]) <= 1e-6 * max(1.0, abs(grad[k]))


def _wf():
    from quantum_package_gb300 import generate as G
    from quantum_package_gb300.sigma import Wavefunction
    p = G.make_problem(1, n_det=500)
    return Wavefunction.from_problem(p)


@pytest.mark.gpu
def test_cuda_forward_matches_reference():
    wf = _wf()
    p = _params(5)
    wf.mlp_set_weights(p)
    X, _, _ = _data(3000, 6)
    y = wf.mlp_predict(X)
    yr, _ = mlp_ref.forward(p, X)
    assert np.abs(y - yr).max() <= 1e-5 * max(1.0, np.abs(yr).max())


@pytest.mark.gpu
def test_cuda_gradient_matches_reference():
    wf = _wf()
    p = _params(7)
    wf.mlp_set_weights(p)
    X, g, w = _data(5000, 8)
    grad, loss = wf.mlp_gradient(X, g, w)
    lr_, gr = mlp_ref.loss_and_grad(p, X, g, w)
    assert abs(loss - lr_) <= 1e-4 * abs(lr_)
    assert np.linalg.norm(grad - gr) <= 2e-3 * np.linalg.norm(gr)
    # per-block agreement (each layer's parameters)
    o = 0
    for size in (512, 64, 4096, 64, 64, 1):
        blk = slice(o, o + size)
        assert np.linalg.norm(grad[blk] - gr[blk]) <= 5e-3 * max(np.linalg.norm(gr[blk]), 1e-6)
        o += size


@pytest.mark.gpu
def test_cuda_training_reduces_loss():
    wf = _wf()
    wf.mlp_init(seed=1)
    X, g, w = _data(20000, 9)
    wf.mlp_add_samples(X, g, w)
    _, l0 = wf.mlp_gradient(X[:4000], g[:4000], w[:4000])
    l1 = wf.mlp_train(epochs=15, batch=1024, lr=3e-3, seed=2)
    assert l1 < 0.3 * l0
    # the trained network reproduces the reference forward pass of its own weights
    y = wf.mlp_predict(X[:1000])
    yr, _ = mlp_ref.forward(wf.mlp_weights(), X[:1000])
    assert np.abs(y - yr).max() <= 1e-5 * max(1.0, np.abs(yr).max())
