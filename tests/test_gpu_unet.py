"""The learned preconditioner's CUDA kernels against the network oracle:
forward output and every parameter gradient (BF16 storage, FP32
accumulation on both sides), and a short training run."""
import numpy as np
import pytest

from helpers import rel_l2

pytestmark = pytest.mark.gpu

TOL_Z = 2e-2   # BF16 activations: roundings flipped by FP32 summation order
TOL_G = 5e-2   # gradients go through ~30 BF16 roundings


def _params(seed):
    from simcoflow_gb300 import learned as Lr
    rng = np.random.Generator(np.random.PCG64(seed))
    p = Lr.init_params(seed)
    import unet_oracle as U
    offs, n = U.offsets()
    for (cin, cout, *_), (wo, bo) in zip(U.LAYERS, offs):
        p[bo:bo + cout] = rng.uniform(-0.1, 0.1, cout)  # nonzero biases
    p[-1] = 0.05
    return p


@pytest.mark.parametrize("shape", [(2, 16, 32), (1, 24, 40)], ids=["2x16x32", "1x24x40"])
def test_unet_forward_and_gradients_match_oracle(cuda, shape):
    import unet_oracle as U
    from simcoflow_gb300 import learned as Lr
    n, H, W = shape
    rng = np.random.Generator(np.random.PCG64(11))
    p = _params(3)
    x5 = rng.normal(size=(n, H, W, 5)).astype(np.float32)
    dz = rng.normal(size=(n, H, W)).astype(np.float32)
    net = Lr.UNet(n, H, W)
    try:
        net.set_params(p)
        net.set_input(x5)
        zg = net.forward()
        net.set_dz(dz)
        net.backward()
        gg = net.grads()
    finally:
        net.close()
    zo, cache = U.forward(p, x5)
    go = U.backward(p, cache, dz)
    assert rel_l2(zg, zo) < TOL_Z
    offs, npar = U.offsets()
    assert gg.size == npar
    for i, (wo, bo) in enumerate(offs):
        cout = U.LAYERS[i][1]
        assert rel_l2(gg[wo:bo], go[wo:bo]) < TOL_G, f"layer {i} weights"
        assert rel_l2(gg[bo:bo + cout], go[bo:bo + cout]) < TOL_G, f"layer {i} bias"
    assert rel_l2(gg[-17:], go[-17:]) < TOL_G, "head"


def test_unet_training_reduces_loss(cuda):
    from simcoflow_gb300 import learned as Lr
    pairs = Lr.generate_pairs(n_inst=4, n_iter=4, size=64)
    assert pairs["r"].shape == (16, 64 * 64)
    _, hist = Lr.train(pairs, steps=200, batch=4, lr=1e-3, seed=1)
    assert np.isfinite(hist).all()
    # weight-gradient atomics make the run order-dependent: compare means
    # over 20 steps with a margin that the decrease clears by far
    assert np.mean(hist[-20:]) < 0.9 * np.mean(hist[:20])
