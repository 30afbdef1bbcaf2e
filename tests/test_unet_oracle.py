"""The network oracle's own gradients against finite differences (CPU).

With BF16 rounding switched off the oracle's backward pass must be the exact
derivative of its forward pass; this pins the oracle before it is used to
check the CUDA kernels."""
import numpy as np
import pytest

import unet_oracle as U


@pytest.fixture()
def exact(monkeypatch):
    monkeypatch.setattr(U, "bf16", lambda x: np.asarray(x, dtype=np.float32))


def test_parameter_count_matches_layout():
    offs, n = U.offsets()
    assert n == 256337
    assert offs[0] == (0, 2304)


def test_oracle_gradient_matches_finite_differences(exact):
    rng = np.random.Generator(np.random.PCG64(3))
    p = U.init_params(1).astype(np.float64)
    x = rng.normal(size=(1, 8, 8, 5))
    dz = rng.normal(size=(1, 8, 8))
    z, cache = U.forward(p, x)
    g = U.backward(p, cache, dz.astype(np.float32))
    f = lambda q: float(np.sum(U.forward(q, x)[0].astype(np.float64) * dz))
    # a few parameters of every layer and of the head
    offs, n = U.offsets()
    picks = []
    for wo, bo in offs:
        picks += [wo, (wo + bo) // 2, bo]
    picks += [n - 5, n - 1]
    h = 1e-3
    for k in picks:
        e = np.zeros_like(p)
        e[k] = h
        fd = (f(p + e) - f(p - e)) / (2 * h)
        # ReLU kinks and float32 sums: a loose but discriminating tolerance
        assert abs(fd - g[k]) <= 2e-2 * max(1.0, abs(fd)), (k, fd, g[k])


def test_loss_gradient(exact):
    rng = np.random.Generator(np.random.PCG64(4))
    z = rng.normal(size=(2, 4, 4)).astype(np.float32)
    t = rng.normal(size=(2, 4, 4)).astype(np.float32)
    m = rng.random((2, 4, 4)) > 0.3
    L, dz = U.loss(z, t, m)
    h = 1e-3
    for idx in [(0, 1, 1), (1, 2, 3)]:
        e = np.zeros_like(z)
        e[idx] = h
        fd = (U.loss(z + e, t, m)[0] - U.loss(z - e, t, m)[0]) / (2 * h)
        assert abs(fd - dz[idx]) < 1e-2 * max(1.0, abs(fd))
