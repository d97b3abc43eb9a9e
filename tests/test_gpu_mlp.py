"""The warm-start MLP's forward and backward pass on the tensor-core kernels against the CPU oracle
(oracle/mlp_oracle.py), which rounds to BF16 where the GPU does and sums in FP64. Tolerance: 2e-3 of each gradient
array's largest element (BF16 rounding of intermediate gradients and FP32 accumulation order)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_forward_backward_matches_oracle():
    import torch

    from oracle import mlp_oracle
    from sosfuse2_gb300.learned import MLP

    net = MLP(100, 200, width=256, depth=2, device='cuda:0', seed=1)
    rng = np.random.default_rng(0)
    R = 256
    X = np.zeros((R, net.n_in_p), np.float32)
    X[:, :100] = rng.standard_normal((R, 100))
    Xb = mlp_oracle.bf16(X)
    dOut = np.zeros((R, net.n_out_p), np.float32)
    dOut[:, :200] = rng.standard_normal((R, 200)).astype(np.float32) * 1e-2
    for i in range(len(net.b)):
        net.b[i].normal_(0, 0.1)
    out = net.forward(torch.as_tensor(Xb, device='cuda:0').to(torch.bfloat16), keep=True)
    dW, db = net.backward(torch.as_tensor(dOut, device='cuda:0'))
    net.check()
    W = [w.cpu().numpy() for w in net.W]
    b = [x.cpu().numpy().astype(np.float64) for x in net.b]
    ref_out, ref_dW, ref_db = mlp_oracle.forward_backward(Xb, W, b, dOut)
    np.testing.assert_allclose(out.cpu().numpy(), ref_out, rtol=0, atol=2e-3 * np.abs(ref_out).max())
    for g, r in zip(dW, ref_dW):
        np.testing.assert_allclose(g.cpu().numpy(), r, rtol=0, atol=2e-3 * np.abs(r).max())
    for g, r in zip(db, ref_db):
        np.testing.assert_allclose(g.cpu().numpy(), r, rtol=0, atol=2e-3 * np.abs(r).max())


def test_training_reduces_loss():
    import torch

    from sosfuse2_gb300.learned import MLP

    net = MLP(64, 64, width=256, depth=3, device='cuda:0', seed=2)
    g = torch.Generator(device='cuda:0').manual_seed(5)
    X = torch.randn(8192, net.n_in_p, device='cuda:0', generator=g)
    X[:, 64:] = 0
    T = torch.zeros(8192, net.n_out_p, device='cuda:0')
    T[:, :64] = torch.tanh(X[:, :64] @ torch.randn(64, 64, device='cuda:0', generator=g) / 8)
    losses = net.train(X.to(torch.bfloat16), T, epochs=8, batch=1024, lr=2e-3)
    assert losses[-1] < 0.5 * losses[0]
