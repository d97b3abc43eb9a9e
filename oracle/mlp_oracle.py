"""CPU oracle of the warm-start MLP's forward and backward pass (TEST INFRASTRUCTURE ONLY).

It follows the GPU training step operation for operation in where it rounds to BF16 (weights, the input, hidden
activations after GELU, the output gradient and the pre-activation gradients that feed the GEMMs) and computes every
product and sum in FP64, so the GPU's FP32-accumulated tensor-core GEMMs agree with it to FP32 summation-order error.
GELU is the exact (erf) form.
"""

import math

import numpy as np


def bf16(x):
    """Round FP32 to BF16 (nearest, ties to even), returned as FP32."""
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def _erf(x):
    return np.vectorize(math.erf)(x)


def gelu(z):
    return 0.5 * z * (1.0 + _erf(z / math.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + _erf(z / math.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / math.sqrt(2 * math.pi)


def forward_backward(X, W, b, dOut):
    """X [R, in] (already BF16 values), weights W_i [out, in] FP32 masters, biases b_i; dOut [R, out] FP32.
    Returns (output FP64, [dW_i], [db_i]) like MLP.forward(keep) + MLP.backward."""
    H = [np.asarray(X, np.float64)]
    Z = []
    n = len(W)
    for i in range(n):
        z = H[-1] @ bf16(W[i]).astype(np.float64).T + b[i]
        Z.append(z)
        if i < n - 1:
            H.append(bf16(gelu(z).astype(np.float32)).astype(np.float64))
    dW, db = [None] * n, [None] * n
    dz_f = np.asarray(dOut, np.float64)
    dz_b = bf16(dOut.astype(np.float32)).astype(np.float64)
    for i in range(n - 1, -1, -1):
        dW[i] = dz_b.T @ H[i]
        db[i] = dz_f.sum(0)
        if i > 0:
            dH = dz_b @ bf16(W[i]).astype(np.float64)
            g = dH * gelu_grad(Z[i - 1])
            dz_f = g
            dz_b = bf16(g.astype(np.float32)).astype(np.float64)
    return Z[-1], dW, db
