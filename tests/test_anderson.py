"""The fixed-point loop and Anderson mixing on an affine operator with a known fixed point (the reference's
DummyKernel pattern, src/sosfuse2/tests/test_iteration.py:9-64), on the CPU: convergence to the fixed point,
mixed per-wavelength convergence, E_NOT_CONVERGED, E_NONFINITE_SOURCE, and the weight guard."""

import numpy as np
import pytest

from oracle.sos_oracle import anderson_solve, anderson_weights


def affine(shape, contraction, seed=0):
    # forcing + D x with a positive diagonal contraction D (spectral radius `contraction`): x* = forcing / (1 - D)
    rng = np.random.default_rng(seed)
    forcing = rng.uniform(0.5, 1.5, shape).astype(np.float32)
    D = rng.uniform(0.2, 1.0, shape).astype(np.float32)
    D *= np.float32(contraction) / D.max()

    def apply(x):
        return (forcing + D * x).astype(np.float32)

    return apply, forcing.astype(np.float64) / (1.0 - D.astype(np.float64))


def boxes_of(apply):
    return lambda x: np.asarray(x[:5, :7, :], np.float64).reshape(5, 7, -1) + 1.0


def test_converges_to_known_fixed_point():
    shape = (6, 12, 3)
    apply, fixed = affine(shape, 0.9)
    x, stats = anderson_solve(apply, boxes_of(apply), shape, 64, 1e-5)
    assert stats['converged'] == [True] * 3
    np.testing.assert_allclose(x, fixed, rtol=1e-3, atol=1e-4)
    plain = 0
    y = np.zeros(shape, np.float32)
    while np.max(np.abs(apply(y) - y)) / np.max(np.abs(apply(y))) > 1e-5 and plain < 500:
        y = apply(y)
        plain += 1
    assert stats['evaluations'] < plain


def test_not_converged_raises():
    shape = (6, 12, 2)
    apply, _ = affine(shape, 0.999)
    with pytest.raises(RuntimeError, match='E_NOT_CONVERGED'):
        anderson_solve(apply, boxes_of(apply), shape, 3, 1e-9)


def test_nonfinite_source_raises():
    shape = (6, 12, 1)

    def apply(x):
        out = np.ones(shape, np.float32)
        out[2, 3, 0] = np.nan
        return out

    with pytest.raises(RuntimeError, match='E_NONFINITE_SOURCE'):
        anderson_solve(apply, lambda x: np.ones((5, 7, 1)), shape, 4, 1e-3)


def test_weight_guard():
    assert anderson_weights(np.eye(3)) is not None
    np.testing.assert_allclose(anderson_weights(np.diag([1.0, 1.0])).sum(), 1.0, rtol=1e-6)
    # nearly parallel residuals give huge alternating weights: rejected
    f = np.array([[1.0, 1.0 + 1e-7], [1.0, 1.0]])
    assert anderson_weights(f.T @ f) is None
