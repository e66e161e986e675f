"""gb_mlp_forward_noalloc: the predictor network's forward pass for callers
that cannot allocate device memory when they ask for a prediction (their
GPU memory is held by another allocator, or they must not take cudaMalloc's
implicit synchronisation inside the Newton loop).

Through the C ABI it must give the float64 CPU oracle's output on a fresh
network (so it cannot be leaning on buffers the allocating path made), the
same output as the allocating entry point, gb_mlp_forward_device, on two
calls in a row (the second call finds the first call's activations in the
shared static scratch), take no device memory on a repeated call, follow
the order of the stream it is given, and refuse batches its fixed scratch
cannot hold.  Kept in a file of its own, collected last."""
import numpy as np
import pytest

from oracle import mlp_ref

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _x(B, seed):
    return np.random.default_rng(seed).uniform(-1, 1, (B, 3)).astype(np.float32)


def test_forward_noalloc_on_a_fresh_network_matches_the_cpu_oracle():
    import torch
    from goma_gb300.mlp import GpuMLP
    net = GpuMLP(3, 256, 3, 5, seed=4)
    X = _x(777, 11)
    x = torch.tensor(X, device="cuda")
    y = torch.full((777, 5), float("nan"), dtype=torch.float32, device="cuda")
    net.forward_noalloc(x, y)
    ref = mlp_ref.forward(net.params(), net.widths, X)[-1]
    got = y.cpu().numpy()
    assert np.isfinite(got).all()
    assert np.abs(got - ref).max() <= TOL * max(1.0, np.abs(ref).max())


def test_forward_noalloc_matches_allocating_forward_on_two_calls():
    import torch
    from goma_gb300.mlp import GpuMLP
    net = GpuMLP(3, 256, 3, 5, seed=9)
    free_after_first = None
    for B, seed in ((1000, 1), (2500, 2)):
        x = torch.tensor(_x(B, seed), device="cuda")
        y = torch.full((B, 5), float("nan"), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        net.forward_noalloc(x, y)
        torch.cuda.synchronize()
        if free_after_first is not None:
            # the repeated call takes no device memory at all
            assert torch.cuda.mem_get_info()[0] == free_before
        free_after_first = torch.cuda.mem_get_info()[0]
        got = y.cpu().numpy()
        ref = net.forward(x).cpu().numpy()
        assert np.isfinite(got).all()
        assert np.abs(got - ref).max() <= TOL * max(1.0, np.abs(ref).max())


def test_forward_noalloc_follows_the_callers_stream():
    import torch
    from goma_gb300.mlp import GpuMLP
    net = GpuMLP(3, 256, 3, 5, seed=6)
    B = 3000
    X = _x(B, 21)
    xh = torch.tensor(X).pin_memory()
    side = torch.cuda.Stream()
    x = torch.zeros((B, 3), dtype=torch.float32, device="cuda")
    y = torch.zeros((B, 5), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    with torch.cuda.stream(side):
        # keep the side stream busy, then write x on it; the pass queued
        # behind them must read the new x
        big = torch.ones((4096, 4096), device="cuda")
        for _ in range(8):
            big = big @ big * 1e-4
        x.copy_(xh, non_blocking=True)
        net.forward_noalloc(x, y, stream=side)
        out = y.clone()
    side.synchronize()
    ref = mlp_ref.forward(net.params(), net.widths, X)[-1]
    got = out.cpu().numpy()
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
