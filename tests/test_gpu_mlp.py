"""The GPU network's forward pass and gradients against the float64 CPU
oracle (oracle/mlp_ref.py), and a training run that reduces the loss."""
import numpy as np
import pytest

from oracle import mlp_ref

pytestmark = pytest.mark.gpu


def _data(n, widths, seed):
    rng = np.random.default_rng(seed)
    X = rng.uniform(-1, 1, (n, widths[0])).astype(np.float32)
    T = rng.uniform(-1, 1, (n, widths[-1])).astype(np.float32)
    M = (rng.uniform(0, 1, (n, widths[-1])) < 0.6).astype(np.float32)
    M[0] = 1.0
    return X, T, M


@pytest.mark.parametrize("shape,n", [((3, 32, 3, 5), 200), ((3, 256, 3, 5), 1000),
                                     ((4, 64, 2, 3), 77)])
def test_mlp_forward_and_gradients_match_cpu_oracle(shape, n):
    import torch
    from goma_gb300.mlp import GpuMLP
    n_in, width, depth, n_out = shape
    net = GpuMLP(n_in, width, depth, n_out, seed=5)
    widths = net.widths
    X, T, M = _data(n, widths, 1)
    dx, dt, dm = (torch.tensor(a, device="cuda") for a in (X, T, M))
    y = net.forward(dx).cpu().numpy()
    p = net.params()
    H = mlp_ref.forward(p, widths, X)
    assert np.abs(y - H[-1]).max() <= 1e-5 * max(1.0, np.abs(H[-1]).max())
    loss = net.loss_grad(dx, dt, dm)
    g = net.grads()
    loss_ref, g_ref = mlp_ref.loss_and_grad(p, widths, X, T, M)
    assert abs(loss - loss_ref) <= 1e-5 * loss_ref
    assert np.abs(g - g_ref).max() <= 1e-4 * np.abs(g_ref).max()


def test_mlp_training_reduces_loss():
    import torch
    from goma_gb300.mlp import GpuMLP
    net = GpuMLP(3, 64, 3, 2, seed=2)
    rng = np.random.default_rng(0)
    X = rng.uniform(-1, 1, (2048, 3)).astype(np.float32)
    T = np.stack([np.sin(2 * X[:, 0]) * X[:, 2], X[:, 1] ** 2 - X[:, 0]], 1).astype(np.float32)
    M = np.ones_like(T)
    dx, dt, dm = (torch.tensor(a, device="cuda") for a in (X, T, M))
    l0 = net.loss_grad(dx, dt, dm)
    net.train(dx, dt, dm, steps=400, batch=512, lr=3e-3, seed=1)
    l1 = net.loss_grad(dx, dt, dm)
    assert l1 < 0.05 * l0
