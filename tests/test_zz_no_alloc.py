"""gb_mlp_forward_noalloc: the predictor network's forward pass for callers
that cannot allocate device memory when they ask for a prediction (their
GPU memory is held by another allocator, or they must not take cudaMalloc's
implicit synchronisation inside the Newton loop).  Through the C ABI it
must give the same output as the allocating entry point,
gb_mlp_forward_device, on two calls in a row (the second call finds the
first call's activations in the shared static scratch), and must refuse
batches its fixed scratch cannot hold."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-5


def test_forward_noalloc_matches_allocating_forward_on_two_calls():
    import torch
    from goma_gb300.mlp import GpuMLP
    net = GpuMLP(3, 256, 3, 5, seed=9)
    for B, seed in ((1000, 1), (2500, 2)):
        x = torch.tensor(np.random.default_rng(seed).uniform(-1, 1, (B, 3)).astype(np.float32),
                         device="cuda")
        y_ref = net.forward(x)
        y = torch.full((B, 5), float("nan"), dtype=torch.float32, device="cuda")
        net.forward_noalloc(x, y)
        ref = y_ref.cpu().numpy()
        got = y.cpu().numpy()
        assert np.isfinite(got).all()
        assert np.abs(got - ref).max() <= TOL * max(1.0, np.abs(ref).max())


def test_forward_noalloc_rejects_batch_beyond_its_scratch():
    import torch
    from goma_gb300 import _lib
    from goma_gb300.mlp import GpuMLP
    net = GpuMLP(3, 256, 3, 5, seed=3)
    B = _lib.MLP_NOALLOC_MAX_ACT // 256 + 1
    x = torch.zeros((B, 3), dtype=torch.float32, device="cuda")
    y = torch.zeros((B, 5), dtype=torch.float32, device="cuda")
    with pytest.raises(_lib.GbError, match="exceeds the static scratch"):
        net.forward_noalloc(x, y)
